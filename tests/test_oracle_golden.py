"""The CPU oracle against golden vectors produced by petgem's own code
(tests/golden/make_golden.py) and the asserts of petgem's tests/test_mesh.py."""
import json

import numpy as np
import pytest

from oracle import basis, fem, topology
from tests.helpers import load, load_test_mesh, rel_norm, sha, topology_json


@pytest.mark.parametrize("p", [1, 2, 3, 4, 5, 6])
def test_basis_matches_reference(p):
    g = load("basis.npz")
    eo, fo, X = g[f"p{p}_eo"], g[f"p{p}_fo"], g[f"p{p}_X"]
    for a in range(eo.shape[0]):
        N, C = basis.shape3d(X, p, eo[a], fo[a])
        np.testing.assert_allclose(np.moveaxis(N, 2, 0), g[f"p{p}_N"][a], rtol=0, atol=1e-13)
        np.testing.assert_allclose(np.moveaxis(C, 2, 0), g[f"p{p}_C"][a], rtol=0, atol=1e-12)


@pytest.mark.parametrize("p", [1, 2, 3])
def test_elemental_matches_reference(p):
    g = load("elemental.npz")
    for c, eo, fo, s, Mr, Kr in zip(g[f"p{p}_coords"], g[f"p{p}_eo"], g[f"p{p}_fo"], g[f"p{p}_sigma"],
                                    g[f"p{p}_M"], g[f"p{p}_K"]):
        J, iJ = fem.jacobian(c)
        M, K = fem.elemental_matrices(eo, fo, J, iJ, p, s)
        assert rel_norm(M, Mr) < 1e-12
        assert rel_norm(K, Kr) < 1e-12


def test_quadrature_exactness():
    # monomial x^a y^b z^c over the unit tet = a! b! c! / (a+b+c+3)!
    from math import factorial
    for deg in (2, 4, 6):
        pts, w = basis.tet_rule(deg)
        for a in range(deg + 1):
            for b in range(deg + 1 - a):
                c = deg - a - b
                exact = factorial(a) * factorial(b) * factorial(c) / factorial(a + b + c + 3)
                got = np.sum(w * pts[:, 0] ** a * pts[:, 1] ** b * pts[:, 2] ** c)
                assert abs(got - exact) < 1e-15


def _topo(tets, ps=(1, 2, 3)):
    elemsE, edgesN = topology.compute_edges(tets)
    elemsF, facesN = topology.compute_faces(tets)
    facesE = topology.compute_faces_edges(elemsF, elemsE, facesN.shape[0])
    bfN, bF, nbF = topology.compute_boundary_faces(elemsF, facesN)
    bE = topology.compute_boundary_edges(facesE, bF)
    eo, fo = topology.element_orientation(tets, elemsE, edgesN, elemsF, facesE)
    out = {"elemsE": elemsE, "edgesN": edgesN, "elemsF": elemsF, "facesN": facesN, "facesE": facesE,
           "bF": bF, "bE": bE, "eo": eo, "fo": fo}
    for p in ps:
        dofs, de, df, dv, nd = topology.compute_connectivity_dofs(elemsE, elemsF, p)
        _, bnd = topology.compute_boundaries(dofs, de, df, bE, bF, p)
        out[p] = (dofs, nd, bnd)
    return out


def test_topology_reference_test_mesh_asserts():
    # petgem tests/test_mesh.py:31-36
    pts, tets, _ = load_test_mesh()
    t = _topo(tets, ps=())
    assert tets.shape[0] == 9453 and pts.shape[0] == 2163
    assert t["facesN"].shape[0] == 20039 and t["edgesN"].shape[0] == 12748
    assert t["elemsE"][0].tolist() == [10591, 10600, 10831, 10832, 10601, 11465]
    assert t["elemsF"][0].tolist() == [17369, 17370, 17400, 17977]


@pytest.mark.parametrize("case", ["test_mesh", "kuhn3"])
def test_topology_bit_exact(case):
    ref = topology_json()[case]
    if case == "test_mesh":
        _, tets, _ = load_test_mesh()
    else:
        from petgem_gb300 import synthetic
        _, tets = synthetic.kuhn_box(3)
    t = _topo(tets)
    got = {"elemsE": t["elemsE"], "elemsF": t["elemsF"], "edgesNodes": t["edgesN"], "facesN": t["facesN"],
           "facesE": t["facesE"], "bFaces": t["bF"], "bEdges": t["bE"], "eo": t["eo"], "fo": t["fo"]}
    for k, v in got.items():
        assert sha(v) == ref["sha"][k], k
    for p in (1, 2, 3):
        dofs, nd, bnd = t[p]
        assert nd == ref[f"p{p}"]["total_num_dofs"]
        assert sha(dofs) == ref[f"p{p}"]["dofs_sha"]
        assert sha(bnd) == ref[f"p{p}"]["boundary_sha"]


@pytest.mark.parametrize("p", [1, 2, 3])
def test_assembly_and_source_match_reference(p):
    g = load("system_n2.npz")
    import scipy.sparse as sp
    pts, tets, sigma = g["points"], g["tets"], g["sigma"]
    src = json.loads(str(g["src"]))
    t = _topo(tets, ps=(p,))
    dofs, nd, bnd = t[p]
    coords = pts[tets]
    M, K = fem.element_matrices_batch(coords, t["eo"], t["fo"], sigma, p)
    A = fem.assemble(M, K, dofs, nd, src["frequency"])
    Ar = sp.csr_matrix((g[f"p{p}_data"], g[f"p{p}_indices"], g[f"p{p}_indptr"]), shape=A.shape)
    assert np.array_equal(A.indptr, Ar.indptr) and np.array_equal(A.indices, Ar.indices)
    assert rel_norm(A.data, Ar.data) < 1e-12
    assert np.array_equal(bnd, g[f"p{p}_bnd"])
    b, se = fem.source_vector(pts, tets, t["eo"], t["fo"], dofs, nd, p, src)
    assert se == int(g[f"p{p}_src_elem"])
    assert rel_norm(b, g[f"p{p}_b"]) < 1e-12


def test_pipeline_fields_match_reference():
    g = load("pipeline_n3.npz")
    pts, tets, sigma = g["points"], g["tets"], g["sigma"]
    src = json.loads(str(g["src"]))
    p = 2
    t = _topo(tets, ps=(p,))
    dofs, nd, bnd = t[p]
    assert np.array_equal(bnd, g["bnd"])
    F, el = fem.interpolate_fields(g["x"], pts, tets, t["eo"], t["fo"], dofs, p, g["receivers"], src["frequency"])
    assert F.shape == g["fields"].shape          # the receiver outside the mesh is dropped
    assert rel_norm(F, g["fields"]) < 1e-12


def _maps(tets, p):
    eE, eN = topology.compute_edges(tets)
    eF, fN = topology.compute_faces(tets)
    fE = topology.compute_faces_edges(eF, eE, fN.shape[0])
    eo, fo = topology.element_orientation(tets, eE, eN, eF, fE)
    dofs, _, _, _, _ = topology.compute_connectivity_dofs(eE, eF, p)
    return eo, fo, dofs


def test_node_fields_match_reference_loop():
    """oracle.fem.node_fields against petgem's own VTK nodal loop
    (postprocessing.py:172-261, run by tests/golden/make_node_fields_golden.py)."""
    g = load("node_fields.npz")
    cases = [("n3", g["n3_points"], g["n3_tets"], 2, g["n3_x"], g["n3_frequency"], g["n3_fields"])]
    for p in (1, 3):
        cases.append((f"tm_p{p}", g["tm_points"], g["tm_tets"], p, g[f"tm_p{p}_x"], g["tm_frequency"],
                      g[f"tm_p{p}_fields"]))
    for name, pts, tets, p, x, f, ref in cases:
        eo, fo, dofs = _maps(tets, p)
        F = fem.node_fields(x, pts, tets, eo, fo, dofs, p, float(f))
        assert rel_norm(F[:, :3], ref[:, :3]) < 1e-12, name
        assert rel_norm(F[:, 3:], ref[:, 3:]) < 1e-12, name
