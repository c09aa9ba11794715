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
