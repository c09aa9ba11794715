"""GPU pipeline parity: topology / DOF maps / PEC DOFs bit-exact against the
reference's golden hashes; CSR pattern bit-exact and values within 1e-12 of
the oracle; source RHS within 1e-12 of the reference; solves to a 1e-8 true
relative residual with receiver fields within 1e-6 of the reference's
fieldInterpolator applied to a direct solution."""
import json

import numpy as np
import pytest
import scipy.sparse as sp
import torch

from oracle import fem, topology
from tests.helpers import load, load_test_mesh, rel_norm, sha, topology_json

pytestmark = pytest.mark.gpu

ELEM_TOL = 1e-12      # elemental / assembled values, normwise relative
FIELD_TOL = 1e-6      # receiver E/H at a 1e-8 relative residual


def _mesh(pts, tets, p, pattern=True):
    from petgem_gb300.engine import DeviceMesh
    return DeviceMesh(pts, tets, p, pattern=pattern)


@pytest.mark.parametrize("case", ["test_mesh", "kuhn3"])
def test_topology_dofs_boundary_bit_exact(case):
    ref = topology_json()[case]
    if case == "test_mesh":
        pts, tets, _ = load_test_mesh()
    else:
        from petgem_gb300 import synthetic
        pts, tets = synthetic.kuhn_box(3)
    for p in (1, 2, 3):
        m = _mesh(pts, tets, p, pattern=False)
        assert (m.nE, m.nF) == (ref["nEdges"], ref["nFaces"])
        got = {"elemsE": m.elemsE, "elemsF": m.elemsF, "edgesNodes": m.edgesNodes, "facesN": m.facesN,
               "facesE": m.facesE, "eo": m.eo, "fo": m.fo}
        for k, v in got.items():
            assert sha(v.cpu().numpy()) == ref["sha"][k], (p, k)
        assert m.N == ref[f"p{p}"]["total_num_dofs"]
        assert sha(m.dofs.cpu().numpy()) == ref[f"p{p}"]["dofs_sha"]
        assert sha(m.bnd.cpu().numpy()) == ref[f"p{p}"]["boundary_sha"]
    if case == "test_mesh":
        # petgem tests/test_mesh.py:31-36
        assert m.elemsE[0].tolist() == [10591, 10600, 10831, 10832, 10601, 11465]
        assert m.elemsF[0].tolist() == [17369, 17370, 17400, 17977]


def _oracle_A(pts, tets, sigma, p, freq):
    t = {}
    elemsE, edgesN = topology.compute_edges(tets)
    elemsF, facesN = topology.compute_faces(tets)
    facesE = topology.compute_faces_edges(elemsF, elemsE, facesN.shape[0])
    eo, fo = topology.element_orientation(tets, elemsE, edgesN, elemsF, facesE)
    dofs, de, df, dv, nd = topology.compute_connectivity_dofs(elemsE, elemsF, p)
    M, K = fem.element_matrices_batch(pts[tets], eo, fo, sigma, p)
    return fem.assemble(M, K, dofs, nd, freq)


def _csr(m, vals):
    return sp.csr_matrix((vals.cpu().numpy(), m.col.cpu().numpy(), m.rowptr.cpu().numpy()), shape=(m.N, m.N))


@pytest.mark.parametrize("p", [1, 2, 3])
@pytest.mark.parametrize("fused", [True, False])
def test_assembly_vs_reference_golden(p, fused):
    g = load("system_n2.npz")
    pts, tets, sigma = g["points"], g["tets"], g["sigma"]
    src = json.loads(str(g["src"]))
    m = _mesh(pts, tets, p)
    vals = m.assemble(sigma, src["frequency"], fused=fused)
    A = _csr(m, vals)
    assert np.array_equal(A.indptr, g[f"p{p}_indptr"]) and np.array_equal(A.indices, g[f"p{p}_indices"])
    assert rel_norm(A.data, g[f"p{p}_data"]) < ELEM_TOL
    b, se = m.source_vector(src)
    assert se == int(g[f"p{p}_src_elem"])
    assert rel_norm(b.cpu().numpy(), g[f"p{p}_b"]) < ELEM_TOL
    assert np.array_equal(m.bnd.cpu().numpy(), g[f"p{p}_bnd"])


@pytest.mark.parametrize("p", [1, 2])
def test_assembly_test_mesh_vs_oracle_and_deterministic(p):
    pts, tets, phys = load_test_mesh()
    rng = np.random.default_rng(3)
    s = 10.0 ** rng.uniform(-2, 0.5, len(tets))
    sigma = np.stack([s, s * rng.uniform(0.5, 1.0, len(tets))], 1)
    m = _mesh(pts, tets, p)
    v1 = m.assemble(sigma, 2.0, fused=True)
    v2 = m.assemble(sigma, 2.0, fused=True)
    assert torch.equal(v1, v2)                       # bitwise reproducible
    v3 = m.assemble(sigma, 2.0, fused=False)
    A = _csr(m, v1)
    Ao = _oracle_A(pts, tets, sigma, p, 2.0)
    assert np.array_equal(A.indptr, Ao.indptr) and np.array_equal(A.indices, Ao.indices)
    assert rel_norm(A.data, Ao.data) < ELEM_TOL
    assert rel_norm(v3.cpu().numpy(), Ao.data) < ELEM_TOL


def test_pec_matches_oracle():
    g = load("system_n2.npz")
    pts, tets, sigma = g["points"], g["tets"], g["sigma"]
    src = json.loads(str(g["src"]))
    p = 2
    m = _mesh(pts, tets, p)
    vals = m.assemble(sigma, src["frequency"])
    b, _ = m.source_vector(src)
    m.apply_pec(vals, b)
    Ar = sp.csr_matrix((g["p2_data"], g["p2_indices"], g["p2_indptr"]), shape=(m.N, m.N))
    Ao, bo = fem.apply_pec(Ar, g["p2_b"], g["p2_bnd"])
    A = _csr(m, vals)
    assert abs(A - Ao).max() <= ELEM_TOL * abs(Ao).max()
    assert rel_norm(b.cpu().numpy(), bo) < ELEM_TOL


@pytest.mark.parametrize("p", [1, 2, 3])
def test_assembly_df64_and_fused_pec_vs_golden(p):
    """Double-float arithmetic, PEC fused into the assembly pass, and the
    record-based pass (bit-identical to the item-list pass)."""
    g = load("system_n2.npz")
    pts, tets, sigma = g["points"], g["tets"], g["sigma"]
    src = json.loads(str(g["src"]))
    m = _mesh(pts, tets, p)
    f = src["frequency"]
    v_df = m.assemble(sigma, f, arithmetic="df64")
    assert torch.equal(v_df, m.assemble(sigma, f, arithmetic="df64"))          # bitwise reproducible
    assert torch.equal(v_df, m.assemble(sigma, f, arithmetic="df64", records=False))
    assert rel_norm(v_df.cpu().numpy(), g[f"p{p}_data"]) < ELEM_TOL
    v64 = m.assemble(sigma, f)
    assert torch.equal(v64, m.assemble(sigma, f, records=False))
    Ar = sp.csr_matrix((g[f"p{p}_data"], g[f"p{p}_indices"], g[f"p{p}_indptr"]), shape=(m.N, m.N))
    Ao, bo = fem.apply_pec(Ar, g[f"p{p}_b"], g[f"p{p}_bnd"])
    # fused PEC in FP64 equals assemble + apply_pec bit for bit
    v_sep = v64.clone()
    b_sep, _ = m.source_vector(src)
    m.apply_pec(v_sep, b_sep)
    for rec in (True, False):
        assert torch.equal(m.assemble(sigma, f, pec=True, records=rec), v_sep)
    b, _ = m.source_vector(src)
    m.pec_rhs(b)
    assert torch.equal(b, b_sep)
    assert rel_norm(b.cpu().numpy(), bo) < ELEM_TOL
    for rec in (True, False):
        A = _csr(m, m.assemble(sigma, f, arithmetic="df64", pec=True, records=rec))
        assert abs(A - Ao).max() <= ELEM_TOL * abs(Ao).max()


@pytest.mark.parametrize("p", [1, 2])
def test_assembly_df64_test_mesh_vs_oracle(p):
    pts, tets, phys = load_test_mesh()
    rng = np.random.default_rng(5)
    s = 10.0 ** rng.uniform(-3, 1, len(tets))
    sigma = np.stack([s, s * rng.uniform(0.2, 1.0, len(tets))], 1)
    m = _mesh(pts, tets, p)
    Ao = _oracle_A(pts, tets, sigma, p, 7.5)
    # double-float element coefficients against the FP64 ones, per element
    c64 = m.element_coefficients(sigma, 7.5).cpu().numpy()
    cdf = m.element_coefficients(sigma, 7.5, arithmetic="df64").cpu().numpy().astype(np.float64)
    cdf = cdf[..., 0] + cdf[..., 1]
    err = np.abs(cdf - c64).max(axis=1) / np.abs(c64).max(axis=1)
    assert err.max() < 1e-13
    v = m.assemble(sigma, 7.5, arithmetic="df64")
    assert torch.equal(v, m.assemble(sigma, 7.5, arithmetic="df64", records=False))
    assert rel_norm(v.cpu().numpy(), Ao.data) < ELEM_TOL
    # each entry to df64 rounding relative to its row scale
    d = np.abs(v.cpu().numpy() - Ao.data)
    rowmax = np.maximum.reduceat(np.abs(Ao.data), Ao.indptr[:-1])
    scale = np.repeat(rowmax, np.diff(Ao.indptr))
    assert (d <= 1e-12 * scale).all()


@pytest.mark.parametrize("ksp,precision", [("gmres", "fp64"), ("gmres", "mixed"), ("cocg", "fp64"),
                                           ("cocg", "mixed"), ("cocg", "df64"), ("cocg", "ir32")])
def test_solve_and_receivers_vs_reference(precision, ksp):
    g = load("pipeline_n3.npz")
    pts, tets, sigma = g["points"], g["tets"], g["sigma"]
    src = json.loads(str(g["src"]))
    m = _mesh(pts, tets, 2)
    vals = m.assemble(sigma, src["frequency"])
    b, se = m.source_vector(src)
    assert se == int(g["src_elem"])
    m.apply_pec(vals, b)
    assert rel_norm(b.cpu().numpy(), g["b"]) < ELEM_TOL
    x, info = m.solve(vals, b, rtol=1e-10, precision=precision, ksp=ksp)
    assert info.relres <= 1e-10
    A = _csr(m, vals)
    xn = x.cpu().numpy()
    assert np.linalg.norm(A @ xn - b.cpu().numpy()) <= 1e-10 * np.linalg.norm(b.cpu().numpy()) * 1.01
    F, keep = m.receiver_fields(x, g["receivers"], src["frequency"])
    assert keep.cpu().numpy().tolist() == [True] * 7 + [False]     # the receiver outside is dropped
    assert rel_norm(F.cpu().numpy(), g["fields"]) < FIELD_TOL


def test_multi_rhs_matches_single():
    from petgem_gb300 import synthetic
    mdl = synthetic.csem_two_layer(4, 2, block=False)
    m = _mesh(mdl.nodes, mdl.tets, 2)
    vals = m.assemble(mdl.sigma, 1.0)
    m.apply_pec(vals, None)
    bs = []
    for x0 in (-600.0, -200.0, 200.0, 600.0):
        src = dict(mdl.source, position=[x0, 10.0, 50.0])
        b, _ = m.source_vector(src)
        m.apply_pec(vals.clone(), b)                     # zero the PEC entries of b
        bs.append(b)
    B = torch.stack(bs, 1).contiguous()
    ref = [m.solve(vals, bs[k], rtol=1e-11)[0].cpu().numpy() for k in range(4)]
    for ksp, prec in (("gmres", "fp64"), ("gmres", "mixed"), ("cocg", "fp64"), ("cocg", "mixed"), ("cocg", "df64"),
                      ("cocg", "ir32")):
        if True:
            X, info = m.solve(vals, B, rtol=1e-9, precision=prec, ksp=ksp)
            assert max(info.relres_per_rhs) <= 1e-9
            for k in range(4):
                assert rel_norm(X[:, k].cpu().numpy(), ref[k]) < 1e-6


def test_gmres_maxit_status_is_returned():
    from petgem_gb300 import _lib, synthetic
    mdl = synthetic.csem_two_layer(4, 2, block=False)
    m = _mesh(mdl.nodes, mdl.tets, 2)
    vals = m.assemble(mdl.sigma, 1.0)
    b, _ = m.source_vector(mdl.source)
    m.apply_pec(vals, b)
    x, info = m.solve(vals, b, rtol=1e-14, max_it=5, raise_on_fail=False)
    assert info.status == -7 and info.iterations <= 30
    with pytest.raises(_lib.PetgemError):
        m.solve(vals, b, rtol=1e-14, max_it=5)
    x, info = m.solve(vals, b, rtol=1e-14, max_it=5, raise_on_fail=False, ksp="cocg", check_every=5)
    assert info.status == -7 and info.iterations == 5


def test_source_outside_mesh_raises():
    from petgem_gb300 import _lib, synthetic
    mdl = synthetic.csem_two_layer(2, 1, block=False)
    m = _mesh(mdl.nodes, mdl.tets, 1)
    with pytest.raises(_lib.PetgemError):
        m.source_vector(dict(mdl.source, position=[5000.0, 0.0, 0.0]))


@pytest.mark.parametrize("p", [4, 5, 6])
def test_assembly_high_order_vs_oracle(p):
    """p = 4..6 (petgem's run.nord range): pattern, FP64 and double-float
    values against the oracle on a small jittered Kuhn mesh."""
    from petgem_gb300 import synthetic
    nodes, tets = synthetic.kuhn_box(2)
    nodes = synthetic.jitter_interior(nodes, 2, 0.15, 0, (-1000.0,) * 3, (1000.0,) * 3)
    rng = np.random.default_rng(p)
    s = 10.0 ** rng.uniform(-2, 0.5, len(tets))
    sigma = np.stack([s, s * rng.uniform(0.3, 1.0, len(tets))], 1)
    m = _mesh(nodes, tets, p)
    Ao = _oracle_A(nodes, tets, sigma, p, 1.5)
    for ar in ("fp64", "df64"):
        v = m.assemble(sigma, 1.5, arithmetic=ar)
        A = _csr(m, v)
        assert np.array_equal(A.indptr, Ao.indptr) and np.array_equal(A.indices, Ao.indices)
        assert rel_norm(A.data, Ao.data) < ELEM_TOL
        assert torch.equal(v, m.assemble(sigma, 1.5, arithmetic=ar, records=False))


@pytest.mark.parametrize("precond", ["block", "jacobi"])
@pytest.mark.parametrize("nrhs", [1, 4])
def test_ir32_refinement_matches_fp64(precond, nrhs):
    """complex64 inner solves + FP64 refinement (precision "ir32") reach the
    FP64 true-residual target and the FP64 COCG solution, p = 2, several
    refinement steps (inner_rtol 1e-2 against rtol 1e-10)."""
    from petgem_gb300 import synthetic
    mdl = synthetic.config1(6)
    m = _mesh(mdl.nodes, mdl.tets, 2)
    vals = m.assemble(mdl.sigma, 1.0, pec=True)
    bs = []
    for x0 in (0.0, -400.0, 300.0, 650.0)[:nrhs]:
        b, _ = m.source_vector(dict(mdl.source, position=[x0, 20.0, 50.0]))
        m.pec_rhs(b)
        bs.append(b)
    B = bs[0] if nrhs == 1 else torch.stack(bs, 1).contiguous()
    ref, _ = m.solve(vals, B, rtol=1e-11, ksp="cocg", precision="fp64", precond=precond, max_it=100000)
    X, info = m.solve(vals, B, rtol=1e-10, ksp="cocg", precision="ir32", precond=precond, max_it=100000)
    assert info.status == 0 and max(info.relres_per_rhs) <= 1e-10
    assert info.restarts >= 3                      # several refinement steps were needed
    A = _csr(m, vals)
    Xn, Bn = X.cpu().numpy(), B.cpu().numpy()
    R = A @ Xn - Bn
    assert np.linalg.norm(R) <= 1e-10 * np.linalg.norm(Bn) * 1.01 * np.sqrt(nrhs)
    assert rel_norm(Xn, ref.cpu().numpy()) < 1e-8
