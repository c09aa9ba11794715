"""The gradient map's oracle, pinned by its defining properties (petgem has no
counterpart to check against): every column of G is exactly representable in
petgem's H(curl) basis, petgem's curl-curl matrix annihilates it (K G = 0,
petgem/hvfem.py:223-316), and the mass matrix does not; rows are unique per
DOF and PEC columns are dropped."""
import numpy as np
import pytest
import scipy.sparse as sp

from oracle import gradient, system
from petgem_gb300 import synthetic


def _box(n=3):
    nodes, tets = synthetic.kuhn_box(n)
    lo, hi = (-1000.0,) * 3, (1000.0,) * 3
    return synthetic.jitter_interior(nodes, n, 0.15, 0, lo, hi), tets


def _global(mats, dofs, N):
    T, nd = dofs.shape
    rows = np.repeat(dofs, nd, axis=1).reshape(-1)
    cols = np.tile(dofs, (1, nd)).reshape(-1)
    return sp.coo_matrix((mats.reshape(-1), (rows, cols)), shape=(N, N)).tocsr()


@pytest.mark.parametrize("p", [1, 2, 3])
def test_gradient_columns_are_curl_free_gradients(p):
    nodes, tets = _box()
    mm = system.mesh_maps(nodes, tets, p)
    M, K = system.element_matrices(nodes[tets], mm["eo"], mm["fo"], np.ones((len(tets), 2)), p, processes=1)
    Kg, Mg = _global(K, mm["dofs"], mm["N"]), _global(M, mm["dofs"], mm["N"])
    G, res = gradient.gradient_map(tets, mm["elemsE"], mm["elemsF"], mm["eo"], mm["fo"], mm["dofs"], mm["N"],
                                   len(nodes), p)
    assert res < 1e-12
    nE, nF = int(mm["elemsE"].max()) + 1, int(mm["elemsF"].max()) + 1
    n_cols = {1: 64, 2: 64 + nE, 3: 64 + 2 * nE + nF}[p]   # 3^3 box: 64 nodes
    assert G.shape == (mm["N"], n_cols)
    assert abs(Kg @ G).max() <= 1e-12 * abs(Kg).max()
    # a gradient has mass: M G is not small
    assert abs(Mg @ G).max() >= 0.1 * abs(Mg).max()
    # every column is used
    assert (np.diff(G.tocsc().indptr) > 0).all()


@pytest.mark.parametrize("p", [1, 2, 3])
def test_gradient_pec_columns_dropped(p):
    nodes, tets = _box()
    mm = system.mesh_maps(nodes, tets, p)
    G, _ = gradient.gradient_map(tets, mm["elemsE"], mm["elemsF"], mm["eo"], mm["fo"], mm["dofs"], mm["N"],
                                 len(nodes), p, pec=mm["bnd"])
    assert G[mm["bnd"]].nnz == 0
    kept = np.diff(G.tocsc().indptr) > 0
    G0, _ = gradient.gradient_map(tets, mm["elemsE"], mm["elemsF"], mm["eo"], mm["fo"], mm["dofs"], mm["N"],
                                  len(nodes), p)
    touched = np.unique(G0[mm["bnd"]].indices)
    assert kept.sum() == G0.shape[1] - len(touched)
    assert kept[:64].sum() == 8   # interior vertices of the 3^3 box


@pytest.mark.parametrize("p", [2, 3])
def test_vector_p1_columns_exact_and_consistent(p):
    """The vector P1 columns (lambda_v e_d) are exactly representable for
    p >= 2 and every element around a DOF gives the same coefficients: the
    map taken from the lowest-index elements equals the one taken from the
    highest-index ones, and Pi times the nodal values of a linear vector
    field reproduces that field's interpolation (checked by the mass-weighted
    residual against the oracle's own elemental mass matrices)."""
    nodes, tets = _box()
    mm = system.mesh_maps(nodes, tets, p)
    args = (tets, mm["elemsE"], mm["elemsF"], mm["eo"], mm["fo"], mm["dofs"], mm["N"], len(nodes), p)
    G, res = gradient.gradient_map(*args, vector=True, nodes=nodes)
    assert res < 1e-12
    n_grad = G.shape[1] - 3 * len(nodes)
    # reversed element order: rows from the highest-index elements
    rev = np.arange(len(tets))[::-1]
    Gr, _ = gradient.gradient_map(tets[rev], mm["elemsE"][rev], mm["elemsF"][rev], mm["eo"][rev], mm["fo"][rev],
                                  mm["dofs"][rev], mm["N"], len(nodes), p, vector=True, nodes=nodes)
    assert abs(G - Gr).max() <= 1e-9 * abs(G).max()
    # a constant field e_x: sum_v lambda_v = 1, so Pi applied to (1, 0, 0) at every vertex is e_x
    ex = np.zeros(G.shape[1])
    ex[n_grad + 0::3] = 1.0
    u = G @ ex
    # e_x = grad(x): the gradient columns represent it through the vertex hats' x coordinates
    gx = np.zeros(G.shape[1])
    gx[:len(nodes)] = nodes[:, 0]
    assert abs(u - G @ gx).max() <= 1e-9 * abs(u).max()


@pytest.mark.parametrize("p", [2, 3])
def test_auxiliary_diagonal_across_frequencies(p):
    """The several-frequency solver keeps one diagonal d = diag(Bᵀ A0 B) of
    the auxiliary map B = [G Π] and divides each column by Re d + i s_j Im d:
    with A_j = Re A0 + i s_j Im A0 and B real that is diag(Bᵀ A_j B) exactly.
    The plain rescale s_j d holds on the gradient columns only (K G = 0, so
    Re d vanishes there) and not on the vector P1 columns."""
    nodes, tets = _box()
    mm = system.mesh_maps(nodes, tets, p)
    M, K = system.element_matrices(nodes[tets], mm["eo"], mm["fo"], np.ones((len(tets), 2)), p, processes=1)
    Kg, Mg = _global(K, mm["dofs"], mm["N"]), _global(M, mm["dofs"], mm["N"])
    Bfull, _ = gradient.gradient_map(tets, mm["elemsE"], mm["elemsF"], mm["eo"], mm["fo"], mm["dofs"], mm["N"],
                                     len(nodes), p, pec=mm["bnd"], vector=True, nodes=nodes)
    # the columns PEC left (vector columns come after the gradient columns)
    used = np.flatnonzero(np.diff(Bfull.tocsc().indptr) > 0)
    is_vec = used >= Bfull.shape[1] - 3 * len(nodes)
    assert is_vec.any() and (~is_vec).any()
    B = Bfull.tocsc()[:, used]
    # a frequency at which curl-curl and mass terms are of one size (where the
    # rescale's error matters)
    c = 0.7 * abs(Kg).max() / abs(Mg).max()
    A0 = (Kg - 1j * c * Mg).tocsr()
    d0 = np.asarray((B.T @ (A0 @ B)).diagonal())
    for s in (0.25, 0.5, 2.0):
        Aj = (Kg - 1j * c * s * Mg).tocsr()
        dj = np.asarray((B.T @ (Aj @ B)).diagonal())
        split = d0.real + 1j * s * d0.imag
        assert abs(dj - split).max() <= 1e-12 * abs(dj).max()
        scaled = s * d0
        assert abs(dj - scaled)[~is_vec].max() <= 1e-10 * abs(dj).max()
        assert abs(dj - scaled)[is_vec].max() >= 1e-2 * abs(dj[is_vec]).max()
