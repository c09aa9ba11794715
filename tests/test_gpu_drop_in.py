"""petgem-compatible entry points on the GPU: hvfem / mesh functions with the
reference's signatures, and the params-file pipeline (Preprocessing ->
Solver -> Postprocessing) against the oracle on petgem's own test mesh."""
import json
import os

import numpy as np
import torch
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


# petgem options files may name hypre's AMS; it runs as Jacobi plus the
# discrete-gradient correction
PC_OPTS = {"default": [], "hypre": ["-pc_type", "hypre", "-pc_hypre_type", "ams"]}


@pytest.mark.parametrize("pc", ["default", "hypre"])
@pytest.mark.parametrize("p", [1, 2])
def test_params_pipeline_vs_oracle(tmp_path, p, pc):
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
    setup, solver, post = run_kernel(str(params), ["-ksp_type", "cocg", "-ksp_rtol", "1e-11", "-ksp_max_it", "100000"]
                                     + PC_OPTS[pc])
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
    _check_result_file(post.output_file, "csem", [post.fields])


def test_petgem_petsc_test_system_solved_by_gpu_gmres():
    """petgem's tests/test_petsc.py: read its PETSc-binary system and solve it
    with the GPU KSP (GMRES + Jacobi, zero initial guess from vector-x)."""
    import os

    import scipy.sparse as sp
    import scipy.sparse.linalg as spla

    from petgem_gb300 import petsc_io
    from petgem_gb300.engine import solve_csr
    fix = os.path.join(os.path.dirname(__file__), "golden")
    rp, col, vals, shape = petsc_io.read_mat(os.path.join(fix, "petgem_matrix-A.dat"))
    b = petsc_io.read_vec(os.path.join(fix, "petgem_vector-b.dat"))
    x0 = petsc_io.read_vec(os.path.join(fix, "petgem_vector-x.dat"))
    dev = torch.device("cuda:0")
    t = lambda a, dt: torch.as_tensor(np.ascontiguousarray(a), dtype=dt, device=dev)  # noqa: E731
    x, info = solve_csr(t(rp, torch.int64), t(col, torch.int32), t(vals, torch.complex128), t(b, torch.complex128),
                        x0=t(x0, torch.complex128), rtol=1e-10, max_it=20000, ksp="gmres")
    assert info.status == 0
    A = sp.csr_matrix((vals, col, rp), shape=shape)
    xg = x.cpu().numpy()
    assert np.linalg.norm(A @ xg - b) <= 1.01e-10 * np.linalg.norm(b)
    xd = spla.spsolve(A.tocsc(), b)
    assert np.linalg.norm(xg - xd) <= 1e-6 * np.linalg.norm(xd)


@pytest.mark.parametrize("pc", ["default", "hypre"])
def test_params_pipeline_mt_vs_oracle(tmp_path, pc):
    """MT mode through the params file: boundary excitation for both
    polarisations, one batched solve, receiver fields and impedances against
    the oracle (petgem's formulation restated, direct solve).  The 1e6-node
    1-D MT solve is conditioned ~1e12 (two LU solves differ by ~6e-7), so the
    comparison is at 5e-6."""
    from oracle import mt
    from petgem_gb300 import gmsh, mt1d
    from petgem_gb300.pipeline import computeImpedance, run_kernel
    g = load("mt_n4.npz")
    pts, tets = g["nodes"], g["tets"]
    cz = pts[tets].mean(axis=1)[:, 2]
    phys = np.where(cz > 0.0, 1, np.where(cz > -1000.0, 2, 3))
    msh = tmp_path / "mesh.msh"
    gmsh.write(str(msh), pts, tets, phys)
    gx = np.linspace(-2000.0, 2000.0, 3)
    X, Y = np.meshgrid(gx, gx, indexing="ij")
    rx = np.stack([X.ravel(), Y.ravel(), np.full(9, -20.0)], axis=1)
    np.save(tmp_path / "rx.npy", rx)
    params = tmp_path / "params.yaml"
    params.write_text(f"""model:
  mode: mt
  mt:
    sigma:
      horizontal: [0.3, 0.1, 0.05]
      vertical: [0.3, 0.1, 0.05]
    frequency: 1.0
    polarization: ['x', 'y']
  mesh: {msh}
  receivers: {tmp_path / 'rx.npy'}
run:
  nord: 2
  cuda: True
output:
  vtk: True
  directory: {tmp_path / 'out'}
  directory_scratch: {tmp_path / 'tmp'}
""")
    setup, solver, post = run_kernel(str(params), ["-ksp_type", "cocg", "-ksp_rtol", "1e-11", "-ksp_max_it", "100000"]
                                     + PC_OPTS[pc])
    assert all(i.status == 0 for i in solver.info)
    from petgem_gb300 import vtk
    _, _, vfields = vtk.read(post.vtk_file)
    assert "mt_Ex_real_modex" in vfields and "mt_Hz_imag_modey" in vfields and "sigma_horizontal" in vfields
    p = 2
    eE, eN = topology.compute_edges(tets)
    eF, fN = topology.compute_faces(tets)
    fE = topology.compute_faces_edges(eF, eE, fN.shape[0])
    eo, fo = topology.element_orientation(tets, eE, eN, eF, fE)
    dofs, de, df, dv, nd = topology.compute_connectivity_dofs(eE, eF, p)
    sh = np.array([0.3, 0.1, 0.05])[phys - 1]
    sigma = np.stack([sh, sh], 1)
    M, K = fem.element_matrices_batch(pts[tets], eo, fo, sigma, p)
    A = fem.assemble(M, K, dofs, nd, 1.0)
    bd = mt.Boundary(pts, tets, eF, fN, fN.shape[0])
    rp, rw = mt1d.triangle_rule(2 * p + 2)
    u, _ = mt.mt_field_at_faces(bd, sigma, rp, 2 * np.pi)
    Fo = []
    for pol in (1, 2):
        b = mt.mt_rhs(bd, eo, fo, dofs, nd, p, u, rp, rw, 2 * np.pi, pol)
        x = spla.spsolve(A.tocsc(), b)
        Fo.append(fem.interpolate_fields(x, pts, tets, eo, fo, dofs, p, rx, 1.0)[0])
    for k in range(2):
        assert rel_norm(post.fields[k], Fo[k]) < 5e-6
    Zo = mt.impedance(Fo, 2 * np.pi, fem.MU0)[3]
    assert rel_norm(np.stack(post.impedance), np.stack(Zo)) < 5e-6
    Zr = computeImpedance(post.fields, 2 * np.pi, fem.MU0)[3]
    assert rel_norm(np.stack(Zr), np.stack(post.impedance)) == 0.0
    assert os.path.exists(post.output_file)
    _check_result_file(post.output_file, "mt", post.fields, post.impedance)
    assert os.path.exists(os.path.join(str(tmp_path / "tmp"), "x1.dat"))


def _check_result_file(path, mode, fields, impedance=None):
    """petgem's result file (postprocessing.py:341-461): name
    {mode}_petgemV{version}_{date}.h5 and its group / dataset paths, read back."""
    import datetime
    import os
    assert os.path.basename(path) == f"{mode}_petgemV1.0_{datetime.date.today():%Y-%m-%d}.h5"
    try:
        import h5py
    except ImportError:
        from petgem_gb300 import hdf5
        d = hdf5.read(path)
    else:
        with h5py.File(path, "r") as f:
            d = {}
            f.visititems(lambda k, v: d.__setitem__(k, v[()]) if isinstance(v, h5py.Dataset) else None)
    for k in ("machine/machine", "machine/num_processors", "machine/petgem_version", "model/date", "model/mesh_file",
              "model/receivers_file", "model/nord", "model/dof", "model/cuda", "model/vtk", "model/mode",
              "model/num-polarizations", "model/solver", "model/run-time (s)", "model/frequency (Hz)"):
        assert k in d, k
    if mode == "csem":
        for k in ("source_position (m)", "source_azimuth (deg)", "source_dip (deg)", "source_current (Am)",
                  "source_length (m)"):
            assert "model/" + k in d, k
        groups = [("E-fields", "H-fields")]
    else:
        pols = [str(q.decode() if isinstance(q, bytes) else q) for q in np.atleast_1d(d["model/polarization"])]
        groups = [(f"E-fields_mode_{q}", f"H-fields_mode_{q}") for q in pols]
    for (ge, gh), F in zip(groups, fields):
        for c, k in enumerate("xyz"):
            assert np.array_equal(d[f"model/{ge}/{k}"], F[:, c])
            assert np.array_equal(d[f"model/{gh}/{k}"], F[:, 3 + c])
    if impedance is not None:
        for j, k in enumerate(("xx", "xy", "yx", "yy")):
            assert np.array_equal(d[f"model/impedance/{k}"], impedance[j])
            assert f"model/apparent_resistivity/{k}" in d and f"model/phase/{k}" in d
        assert "model/tipper/x" in d and "model/tipper/y" in d
