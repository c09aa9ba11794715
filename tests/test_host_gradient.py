"""Host logic of the gradient correction, on the CPU: the block-diagonal map
that several systems share (engine.concat_gradients) shifts each system's
rows by its first row and its columns by the columns before it, in both G
and its transpose, and rejects a map whose rows do not match its system."""
import numpy as np
import pytest
import scipy.sparse as sp
import torch

from petgem_gb300.engine import GradientMap, concat_gradients


def _map(n_rows, n_cols, density, seed):
    rng = np.random.default_rng(seed)
    G = sp.random(n_rows, n_cols, density=density, random_state=rng, format="csr")
    G.data = rng.standard_normal(G.nnz)
    G.sort_indices()
    Gt = G.T.tocsr()
    Gt.sort_indices()
    pad = 7   # the map's entry arrays are sized by an upper bound
    t = lambda a, dt: torch.as_tensor(np.concatenate([a, np.zeros(pad, a.dtype)]), dtype=dt)
    return G, GradientMap(n_cols, torch.as_tensor(G.indptr, dtype=torch.int64), t(G.indices, torch.int32),
                          t(G.data, torch.float64), torch.as_tensor(Gt.indptr, dtype=torch.int64),
                          t(Gt.indices, torch.int32), t(Gt.data, torch.float64))


def _csr(rp, ix, v, shape):
    n = int(rp[-1])
    return sp.csr_matrix((v[:n].numpy(), ix[:n].numpy().astype(np.int64), rp.numpy()), shape=shape)


def test_concat_gradients_is_block_diagonal():
    shapes = [(40, 13), (25, 9), (61, 20)]
    pairs = [_map(r, c, 0.15, s) for s, (r, c) in enumerate(shapes)]
    rows = np.cumsum([0] + [r for r, _ in shapes])
    g = concat_gradients([m for _, m in pairs], rows)
    ref = sp.block_diag([G for G, _ in pairs]).tocsr()
    ref.sort_indices()
    assert g.n_cols == sum(c for _, c in shapes)
    got = _csr(g.rowptr, g.col, g.val, ref.shape)
    assert (got != ref).nnz == 0
    got_t = _csr(g.t_rowptr, g.t_row, g.t_val, (ref.shape[1], ref.shape[0]))
    assert (got_t != ref.T.tocsr()).nnz == 0
    # the transpose rows stay ascending
    for c in range(g.n_cols):
        seg = g.t_row[int(g.t_rowptr[c]):int(g.t_rowptr[c + 1])].numpy()
        assert (np.diff(seg) > 0).all()


def test_concat_gradients_rejects_mismatched_rows():
    _, a = _map(10, 4, 0.3, 1)
    _, b = _map(12, 5, 0.3, 2)
    with pytest.raises(ValueError):
        concat_gradients([a, b], np.array([0, 10, 21]))


@pytest.mark.parametrize("p", [1, 2, 3])
def test_gradient_map_sizes_match_oracle(p):
    """pg_gradient_map_sizes (host-only C-ABI query): the column count of the
    oracle's map and an upper bound of its stored entries; orders outside
    1..3 are rejected."""
    import ctypes
    from oracle import gradient, system
    from petgem_gb300 import _lib, synthetic
    nodes, tets = synthetic.kuhn_box(3)
    mm = system.mesh_maps(nodes, tets, p)
    nE, nF = int(mm["elemsE"].max()) + 1, int(mm["elemsF"].max()) + 1
    G, _ = gradient.gradient_map(tets, mm["elemsE"], mm["elemsF"], mm["eo"], mm["fo"], mm["dofs"], mm["N"],
                                 len(nodes), p)
    nc, me = ctypes.c_int64(), ctypes.c_int64()
    lib = _lib.load()
    assert lib.pg_gradient_map_sizes(len(nodes), nE, nF, len(tets), p, 0, ctypes.byref(nc), ctypes.byref(me)) == 0
    assert nc.value == G.shape[1]
    assert G.nnz <= me.value
    assert lib.pg_gradient_map_sizes(len(nodes), nE, nF, len(tets), 4, 0, ctypes.byref(nc), ctypes.byref(me)) == -1
    assert lib.pg_gradient_map_workspace_bytes(len(nodes), nE, nF, len(tets), 3, p, 0) > 0
    assert lib.pg_gradient_map_workspace_bytes(len(nodes), nE, nF, len(tets), 3, 0, 0) == 0
    # with the vector P1 columns (p >= 2): 3 more per vertex
    vst = lib.pg_gradient_map_sizes(len(nodes), nE, nF, len(tets), p, 1, ctypes.byref(nc), ctypes.byref(me))
    if p == 1:
        assert vst == -1
    else:
        assert vst == 0 and nc.value == G.shape[1] + 3 * len(nodes)
        Gv, _ = gradient.gradient_map(tets, mm["elemsE"], mm["elemsF"], mm["eo"], mm["fo"], mm["dofs"], mm["N"],
                                      len(nodes), p, vector=True, nodes=nodes)
        assert Gv.shape[1] == nc.value and Gv.nnz <= me.value
        assert lib.pg_gradient_map_workspace_bytes(len(nodes), nE, nF, len(tets), 3, p, 1) > \
            lib.pg_gradient_map_workspace_bytes(len(nodes), nE, nF, len(tets), 3, p, 0)
