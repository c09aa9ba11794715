"""Oracle MT pieces against golden vectors made by running petgem's own
functions (tests/golden/make_mt_golden.py)."""
import numpy as np

from oracle import mt, topology
from tests.helpers import load, rel_norm

MU = 4e-7 * np.pi


def _mesh():
    g = load("mt_n4.npz")
    tets = g["tets"]
    eE, eN = topology.compute_edges(tets)
    eF, fN = topology.compute_faces(tets)
    fE = topology.compute_faces_edges(eF, eE, fN.shape[0])
    eo, fo = topology.element_orientation(tets, eE, eN, eF, fE)
    return g, eE, eF, fN, eo, fo


def test_boundary_faces_and_planes_match_reference():
    g, eE, eF, fN, eo, fo = _mesh()
    bd = mt.Boundary(g["nodes"], g["tets"], eF, fN, fN.shape[0])
    assert np.array_equal(bd.bfaces, g["p1_bFaces"])
    assert np.array_equal(bd.belem, g["p1_bElems"])
    assert np.array_equal(bd.planes, g["p1_planes"])


def test_mt_rhs_matches_reference_with_reference_field():
    """Same 1-D field and the reference's triangle rule: the face integral
    agrees with petgem's assembly to rounding."""
    g, eE, eF, fN, eo, fo = _mesh()
    bd = mt.Boundary(g["nodes"], g["tets"], eF, fN, fN.shape[0])
    for p in (1, 2):
        dofs, _, _, _, N = topology.compute_connectivity_dofs(eE, eF, p)
        rp, rw = g[f"rule{2 * p}_points"], g[f"rule{2 * p}_weights"]
        _, zpts = mt.mt_field_at_faces(bd, g["sigma"], rp, 2 * np.pi, MU, n_nodes=16)
        assert np.abs(zpts - g[f"p{p}_zpts"]).max() <= 1e-9
        for k, pol in enumerate((1, 2)):
            b = mt.mt_rhs(bd, eo, fo, dofs, N, p, g[f"p{p}_u"], rp, rw, 2 * np.pi, pol, MU)
            assert rel_norm(b, g[f"p{p}_b"][k]) < 1e-12


def test_mt1d_field_matches_reference():
    """The 1e6-node 1-D solve is conditioned ~1e12: two LU factorisations of
    it agree to ~6e-7 (extended-precision check: each is ~2e-7 from the exact
    discrete solution), so the field is pinned at 1e-6."""
    g, eE, eF, fN, eo, fo = _mesh()
    u = mt.mt1d_field(float(g["p2_za"]), float(g["p2_zb"]), g["p2_s4"], g["p2_cz4"], 2 * np.pi, MU,
                      interpolate_at=g["p2_zpts"])
    assert rel_norm(u, g["p2_u"]) < 1e-6


def test_impedance_matches_reference():
    g = load("mt_n4.npz")
    rho, phase, tip, Z = mt.impedance(list(g["imp_fields"]), 2 * np.pi, MU)
    assert rel_norm(np.stack(Z), g["imp_Z"]) < 1e-13
    assert rel_norm(np.stack(rho), g["imp_rho"]) < 1e-13
    assert rel_norm(np.stack(phase), g["imp_phase"]) < 1e-13
    assert rel_norm(np.stack(tip), g["imp_tipper"]) < 1e-13
