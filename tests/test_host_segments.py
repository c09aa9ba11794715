"""Host side of the several-systems solve: the block-diagonal layout built by
concat_systems (CPU tensors, no GPU)."""
import numpy as np
import scipy.sparse as sp
import torch

from petgem_gb300.engine import concat_systems


def _csr(n, seed):
    rng = np.random.default_rng(seed)
    a = sp.random(n, n, density=0.3, random_state=seed, format="csr") + sp.eye(n)
    a.data = a.data + 1j * rng.normal(size=a.data.size)
    a.sort_indices()
    return a


def test_concat_systems_is_block_diagonal():
    mats = [_csr(n, s) for s, n in enumerate((5, 1, 7))]
    systems = []
    for j, a in enumerate(mats):
        b = torch.arange(a.shape[0], dtype=torch.float64).to(torch.complex128) + j
        systems.append((torch.as_tensor(a.indptr, dtype=torch.int64), torch.as_tensor(a.indices, dtype=torch.int32),
                        torch.as_tensor(a.data, dtype=torch.complex128), b))
    rowptr, col, vals, b, rows = concat_systems(systems)
    assert rows.tolist() == [0, 5, 6, 13]
    got = sp.csr_matrix((vals.numpy(), col.numpy(), rowptr.numpy()), shape=(13, 13))
    want = sp.block_diag(mats, format="csr")
    assert abs(got - want).max() == 0
    assert col.dtype == torch.int32 and rowptr.dtype == torch.int64
    assert torch.equal(b, torch.cat([s[3] for s in systems]))
    # every row references only its own system's columns
    for j in range(3):
        seg = col[rowptr[rows[j]]:rowptr[rows[j + 1]]]
        assert int(seg.min()) >= rows[j] and int(seg.max()) < rows[j + 1]


def test_batched_workload_meshes_and_sources():
    from petgem_gb300 import synthetic
    sizes = synthetic.config2_extra_sizes()
    assert len(sizes) == 8 and all(8 <= v <= 20 for v in sizes)
    assert sizes == synthetic.config2_extra_sizes()          # seeded
    srcs = synthetic.config2_sources()
    assert len(srcs) == 64
    xs = np.array([s["position"][0] for s in srcs])
    # every source lies inside the [-1000, 1000] m box of the two-layer meshes
    assert np.all(np.abs(xs) <= 1000.0) and np.all(np.diff(xs) > 0)


def _block_map(rows, k, active=None):
    import ctypes
    from petgem_gb300 import _lib
    lib = _lib.load()
    rows = np.ascontiguousarray(rows, dtype=np.int64)
    S = rows.size - 1
    blk = np.zeros(S + 1, dtype=np.int32)
    act = None if active is None else np.ascontiguousarray(active, dtype=np.uint8)
    st = lib.pg_segments_block_map(ctypes.c_void_p(rows.ctypes.data), S, k,
                                   ctypes.c_void_p(0 if act is None else act.ctypes.data),
                                   ctypes.c_void_p(blk.ctypes.data))
    assert st == 0
    return blk


def test_segment_block_map_invariants():
    """The launch's block map (host code of pg_cocg_segments): every system
    holds at least one block, shares follow the rows, and the re-split after
    a residual check keeps the grid size, gives converged systems one block
    and hands the rest to the systems still iterating."""
    rng = np.random.default_rng(0)
    for trial in range(300):
        S = int(rng.integers(1, 40))
        k = int(rng.choice([1, 2, 4, 8, 16, 32]))
        sizes = rng.integers(0, 2_000_000 if trial % 2 else 300, S)
        rows = np.concatenate([[0], np.cumsum(sizes)])
        if rows[-1] == 0:
            continue
        blk = _block_map(rows, k)
        counts = np.diff(blk)
        assert blk[0] == 0 and counts.min() >= 1
        total = int(blk[-1])
        act = rng.random(S) < 0.5
        r = _block_map(rows, k, act)
        rc = np.diff(r)
        assert r[0] == 0 and int(r[-1]) == total and rc.min() >= 1
        if act.any() and (~act).any():
            assert np.all(rc[~act] == 1)
        # no system gets more blocks than it has (row, rhs) items to spread over, except the largest active one
        cap = np.maximum((sizes * k + 255) // 256, 1)
        big = np.argmax(np.where(act, sizes, -1)) if act.any() else S - 1
        over = np.nonzero(rc > cap)[0]
        assert set(over.tolist()) <= {int(big)}
    # proportional shares on a large, even case
    rows = np.array([0, 1_000_000, 3_000_000], dtype=np.int64)
    c = np.diff(_block_map(rows, 1))
    assert abs(c[1] / c[0] - 2.0) < 0.01


def test_segment_block_map_rejects_bad_rows():
    import ctypes
    from petgem_gb300 import _lib
    lib = _lib.load()
    rows = np.array([0, 10, 5], dtype=np.int64)
    blk = np.zeros(3, dtype=np.int32)
    st = lib.pg_segments_block_map(ctypes.c_void_p(rows.ctypes.data), 2, 1, ctypes.c_void_p(0),
                                   ctypes.c_void_p(blk.ctypes.data))
    assert st == -1


def test_csr_solvers_reject_bad_arrays_before_the_library():
    """dtype, shape and device checks of the CSR solve entry points run on the
    host and raise ValueError (no device needed)."""
    import pytest
    from petgem_gb300.engine import solve_csr, solve_csr_frequencies, solve_csr_segments
    rp = torch.tensor([0, 1, 2], dtype=torch.int64)
    col = torch.tensor([0, 1], dtype=torch.int32)
    vals = torch.ones(2, dtype=torch.complex128)
    b = torch.ones(2, dtype=torch.complex128)
    with pytest.raises(ValueError, match="CUDA device"):
        solve_csr(rp, col, vals, b)                          # host tensors
    with pytest.raises(ValueError, match="int64"):
        solve_csr(rp.to(torch.int32), col, vals, b)
    with pytest.raises(ValueError, match="complex128"):
        solve_csr(rp, col, vals.to(torch.complex64), b, ksp="cocg")
    with pytest.raises(ValueError, match="sizes disagree"):
        solve_csr(rp, col, vals, torch.ones(3, dtype=torch.complex128))
    with pytest.raises(ValueError, match="CUDA device"):
        solve_csr_frequencies(rp, col, vals, b.reshape(2, 1), [1.0])
    with pytest.raises(ValueError, match=r"system 0\): rowptr must be int64"):
        solve_csr_segments([(rp, col.to(torch.int64), vals, b), (rp, col, vals, b)])


def test_csr_solvers_need_contiguous_arrays_and_a_row_major_solution():
    """The library reads rowptr / col / vals and writes x through their data
    pointers: strided inputs are rejected, and the solution buffer is
    row-major even when b is a transposed view."""
    import pytest
    from petgem_gb300.engine import _new_x, solve_csr
    rp = torch.tensor([0, 1, 2], dtype=torch.int64)
    col = torch.tensor([0, 1], dtype=torch.int32)
    vals = torch.ones(4, dtype=torch.complex128)[::2]          # strided view
    b = torch.ones(2, dtype=torch.complex128)
    with pytest.raises(ValueError, match="vals must be contiguous"):
        solve_csr(rp, col, vals, b)
    bt = torch.arange(8, dtype=torch.float64).to(torch.complex128).reshape(4, 2).t()   # [2, 4], not row-major
    assert not bt.is_contiguous()
    x = _new_x("t", bt, None)
    assert x.shape == bt.shape and x.is_contiguous() and bool((x == 0).all())
    x = _new_x("t", bt, bt)
    assert x.is_contiguous() and torch.equal(x, bt)
    with pytest.raises(ValueError, match="x0 must match b"):
        _new_x("t", bt, torch.zeros(4, 2, dtype=torch.complex128))
