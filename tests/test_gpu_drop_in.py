"""petgem-compatible entry points on the GPU: hvfem / mesh functions with the
reference's signatures, and the params-file pipeline (Preprocessing ->
Solver -> Postprocessing) against the oracle on petgem's own test mesh."""
import json
import os

import numpy as np
import pytest
import scipy.sparse.linalg as spla

from oracle import fem, topology
from tests.helpers import load, load_test_mesh, rel_norm, sha, topology_json

pytestmark = pytest.mark.gpu


def test_mesh_functions_bit_exact():
    from petgem_gb300 import mesh
    ref = topology_json()["test_mesh"]
    pts, tets, _ = load_test_mesh()
    T = len(tets)
    eE, eN = mesh.computeEdges(tets, T)
    eF, fN = mesh.computeFaces(tets, T)
    fE = mesh.computeFacesEdges(eF, eE, fN.shape[0], T)
    bfN, bF, nbF = mesh.computeBoundaryFaces(eF, fN)
    bE = mesh.computeBoundaryEdges(eN, bfN)
    for k, v in {"elemsE": eE, "edgesNodes": eN, "elemsF": eF, "facesN": fN, "facesE": fE, "bFaces": bF,
                 "bEdges": bE}.items():
        assert sha(v) == ref["sha"][k], k
    from petgem_gb300 import hvfem
    for p in (1, 2, 3):
        dofs, de, df, dv, nd = hvfem.computeConnectivityDOFS(eE, eF, p)
        assert nd == ref[f"p{p}"]["total_num_dofs"] and sha(dofs) == ref[f"p{p}"]["dofs_sha"]
        inner, bnd = mesh.computeBoundaries(dofs, de, df, bE, bF, p)
        assert sha(bnd) == ref[f"p{p}"]["boundary_sha"]
        assert len(inner) + len(bnd) == nd


def test_single_element_hvfem_functions():
    from petgem_gb300 import hvfem
    g = load("elemental.npz")
    for p in (1, 2, 3):
        for c, eo, fo, s, Mr, Kr in list(zip(g[f"p{p}_coords"], g[f"p{p}_eo"], g[f"p{p}_fo"], g[f"p{p}_sigma"],
                                              g[f"p{p}_M"], g[f"p{p}_K"]))[:3]:
            J, iJ = hvfem.computeJacobian(c)
            M, K = hvfem.computeElementalMatrices(eo, fo, J, iJ, p, s)
            assert rel_norm(M, Mr) < 1e-12 and rel_norm(K, Kr) < 1e-12
            xi = np.array([[0.1, 0.2, 0.3], [0.25, 0.25, 0.25]])
            B, C = hvfem.computeBasisFunctions(eo, fo, J, iJ, p, xi)
            Bo, Co = fem.basis_at(np.vstack([np.zeros(3), J]), eo, fo, p, xi)
            assert rel_norm(B, Bo) < 1e-12 and rel_norm(C, Co) < 1e-11
    # orientation of a test-mesh element against the oracle
    pts, tets, _ = load_test_mesh()
    eE, eN = topology.compute_edges(tets)
    eF, fN = topology.compute_faces(tets)
    fE = topology.compute_faces_edges(eF, eE, fN.shape[0])
    eo, fo = topology.element_orientation(tets, eE, eN, eF, fE)
    for e in (0, 17, 4242):
        a, b = hvfem.computeElementOrientation(eE[e], tets[e], eN[eE[e]], fE[eF[e]])
        assert a.tolist() == eo[e].tolist() and b.tolist() == fo[e].tolist()


@pytest.mark.parametrize("p", [1, 2])
def test_params_pipeline_vs_oracle(tmp_path, p):
    from petgem_gb300 import gmsh
    from petgem_gb300.pipeline import run_kernel
    pts, tets, phys = load_test_mesh()
    msh = tmp_path / "mesh.msh"
    gmsh.write(str(msh), pts, tets, phys)
    rx = np.array([[1750.0, 1750.0, -1000.0 + 30.0 * k] for k in range(5)] + [[1e6, 0.0, 0.0]])
    np.save(tmp_path / "rx.npy", rx)
    params = tmp_path / "params.yaml"
    params.write_text(f"""model:
  mode: csem
  csem:
    sigma:
      horizontal: [1., 0.01, 1., 3.3333]
      vertical: [1., 0.01, 1., 3.3333]
    source:
      frequency: 2.0
      position: [1750., 1750., -975.]
      azimuth: 0
      dip: 0
      current: 1.
      length: 1.
  mesh: {msh}
  receivers: {tmp_path / 'rx.npy'}
run:
  nord: {p}
  cuda: True
output:
  vtk: False
  directory: {tmp_path / 'out'}
  directory_scratch: {tmp_path / 'tmp'}
""")
    setup, solver, post = run_kernel(str(params), ["-ksp_type", "cocg", "-ksp_rtol", "1e-11", "-ksp_max_it", "100000"])
    assert solver.info[0].relres <= 1e-11
    # oracle: assembly, PEC, direct solve, fields
    eE, eN = topology.compute_edges(tets)
    eF, fN = topology.compute_faces(tets)
    fE = topology.compute_faces_edges(eF, eE, fN.shape[0])
    eo, fo = topology.element_orientation(tets, eE, eN, eF, fE)
    dofs, de, df, dv, nd = topology.compute_connectivity_dofs(eE, eF, p)
    sh = np.array([1., 0.01, 1., 3.3333])[phys - 1]
    sigma = np.stack([sh, sh], 1)
    M, K = fem.element_matrices_batch(pts[tets], eo, fo, sigma, p)
    A = fem.assemble(M, K, dofs, nd, 2.0)
    src = setup.model["csem"]["source"]
    b, _ = fem.source_vector(pts, tets, eo, fo, dofs, nd, p, src)
    bF = topology.compute_boundary_faces(eF, fN)[1]
    bE = topology.compute_boundary_edges(fE, bF)
    _, bnd = topology.compute_boundaries(dofs, de, df, bE, bF, p)
    Ap, bp = fem.apply_pec(A, b, bnd)
    x = spla.spsolve(Ap.tocsc(), bp)
    F, keep = fem.interpolate_fields(x, pts, tets, eo, fo, dofs, p, rx, 2.0)
    assert post.fields.shape == F.shape == (5, 6)
    assert rel_norm(post.fields, F) < 1e-6
    assert os.path.exists(post.output_file)
