"""GPU elemental matrices against the reference's golden matrices and the oracle.

Tolerance: 1e-12 normwise relative per element (the bar for elemental
matrices); the kernel integrates with its own exact quadrature and a
factored (geometry x reference-table) form, so agreement is to rounding.
"""
import numpy as np
import pytest
import torch

from tests.helpers import load, load_test_mesh, rel_norm

pytestmark = pytest.mark.gpu
TOL = 1e-12


def _gpu_elemental(coords, eo, fo, sigma, p):
    from petgem_gb300 import kernels
    k = coords.shape[0]
    dev = torch.device("cuda:0")
    nodes = torch.as_tensor(np.ascontiguousarray(coords.reshape(-1, 3)), dtype=torch.float64, device=dev)
    elemsN = torch.arange(4 * k, dtype=torch.int32, device=dev).view(k, 4)
    eo_t = torch.as_tensor(np.asarray(eo), dtype=torch.int8, device=dev).contiguous()
    fo_t = torch.as_tensor(np.asarray(fo), dtype=torch.int8, device=dev).contiguous()
    sig = torch.as_tensor(np.asarray(sigma), dtype=torch.float64, device=dev).contiguous()
    tup, codes = kernels.orientation_tuples(eo_t, fo_t)
    tabs = kernels.tuple_tables(codes, p)
    M, K = kernels.elemental_matrices(nodes, elemsN, sig, tup, tabs, p)
    return M.cpu().numpy(), K.cpu().numpy()


@pytest.mark.parametrize("p", [1, 2, 3])
def test_elemental_vs_reference_golden(p):
    g = load("elemental.npz")
    M, K = _gpu_elemental(g[f"p{p}_coords"], g[f"p{p}_eo"], g[f"p{p}_fo"], g[f"p{p}_sigma"], p)
    for e in range(M.shape[0]):
        assert rel_norm(M[e], g[f"p{p}_M"][e]) < TOL, e
        assert rel_norm(K[e], g[f"p{p}_K"][e]) < TOL, e


@pytest.mark.parametrize("p", [2, 3])
def test_elemental_test_mesh_many_tuples(p):
    """All 9,453 elements of petgem's test mesh (1,510 orientation tuples)."""
    from oracle import fem, topology
    pts, tets, _ = load_test_mesh()
    elemsE, edgesN = topology.compute_edges(tets)
    elemsF, facesN = topology.compute_faces(tets)
    facesE = topology.compute_faces_edges(elemsF, elemsE, facesN.shape[0])
    eo, fo = topology.element_orientation(tets, elemsE, edgesN, elemsF, facesE)
    rng = np.random.default_rng(7)
    sigma = 10.0 ** rng.uniform(-2, 0.5, (len(tets), 2))
    M, K = _gpu_elemental(pts[tets], eo, fo, sigma, p)
    for e in rng.choice(len(tets), 40, replace=False):
        J, iJ = fem.jacobian(pts[tets[e]])
        Mo, Ko = fem.elemental_matrices(eo[e], fo[e], J, iJ, p, sigma[e])
        assert rel_norm(M[e], Mo) < TOL
        assert rel_norm(K[e], Ko) < TOL
    assert np.allclose(M, np.transpose(M, (0, 2, 1)), rtol=0, atol=0)


def test_degenerate_element_reports_status():
    from petgem_gb300 import _lib
    coords = np.zeros((1, 4, 3))
    coords[0, 1] = [1, 0, 0]
    coords[0, 2] = [2, 0, 0]
    coords[0, 3] = [0, 1, 0]            # all four vertices coplanar: det(J) = 0
    with pytest.raises(_lib.PetgemError) as ei:
        _gpu_elemental(coords, np.zeros((1, 6)), np.zeros((1, 4)), np.ones((1, 2)), 2)
    assert ei.value.status == -5
