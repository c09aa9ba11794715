"""Parity at the configurations the benchmark numbers are quoted on.

* The plain FP64 CSEM workload, p = 1 (16^3 cubes x 6 tets, 31,024 DOFs,
  seawater / sediment / resistive block, x-HED at 1 Hz, 20 receivers):
  matrix, right-hand side and PEC DOFs against the oracle; petgem's own KSP
  (restarted GMRES(30) + Jacobi, complex128) to a 1e-8 true residual, with
  receiver E within 1e-6 of the oracle's direct solve.
* The p = 2 workload the assembly rate is quoted on (32^3 cubes x 6 tets,
  196,608 tets, 1,276,096 DOFs, 54,751,616 stored entries, jittered nodes,
  log-uniform sigma), assembled with the benchmark's own calls (records,
  PEC fused, FP64 and double-float): pattern bit-exact, values within 1e-12
  normwise of the oracle, right-hand side within 1e-12.

The oracle runs its elemental loop in processes started with ``spawn``.
"""
import os

import numpy as np
import pytest
import scipy.sparse as sp
import torch

from tests.helpers import rel_norm

pytestmark = pytest.mark.gpu

ELEM_TOL = 1e-12      # assembled values and b, normwise relative
FIELD_TOL = 1e-6      # receiver E at a 1e-8 relative residual


def _csr(m, vals):
    return sp.csr_matrix((vals.cpu().numpy(), m.col.cpu().numpy(), m.rowptr.cpu().numpy()), shape=(m.N, m.N))


def _bench_assembly(mesh, sigma_np, freq, arithmetic):
    """The benchmark's step: coefficients, then the record-driven fused
    assembly with PEC, exactly as bench.py calls them."""
    sigma = mesh.sigma_tensor(sigma_np)
    mesh.records()
    mesh.tables_entry_major(arithmetic)
    if arithmetic == "df64":
        coef = torch.empty((mesh.T, 12, 2), dtype=torch.float32, device="cuda")
    else:
        coef = torch.empty((mesh.T, 12), dtype=torch.float64, device="cuda")
    vals = torch.empty(mesh.nnz, dtype=torch.complex128, device="cuda")
    mesh.element_coefficients(sigma, freq, out=coef, check=True, arithmetic=arithmetic)
    mesh.assemble(sigma, freq, out=vals, coef=coef, arithmetic=arithmetic, pec=True)
    return vals


def test_config0_plain_fp64_gmres30_jacobi_vs_oracle():
    from oracle import solve as osolve
    from oracle import system
    from petgem_gb300 import synthetic
    from petgem_gb300.engine import DeviceMesh
    model = synthetic.config0()
    f = model.source["frequency"]
    S = system.csem_system(model.nodes, model.tets, model.sigma, 1, model.source,
                           processes=min(16, os.cpu_count() or 1))
    A = S["A"]
    mesh = DeviceMesh(model.nodes, model.tets, 1)
    assert (mesh.T, mesh.N, mesh.nnz) == (24576, 31024, 482608)
    assert np.array_equal(np.sort(mesh.bnd.cpu().numpy()), np.sort(S["bnd"]))
    vals = _bench_assembly(mesh, model.sigma, f, "fp64")
    Ag = _csr(mesh, vals)
    assert np.array_equal(Ag.indptr, A.indptr) and np.array_equal(Ag.indices, A.indices)
    assert rel_norm(Ag.data, A.data) < ELEM_TOL
    b, se = mesh.source_vector(model.source)
    mesh.pec_rhs(b)
    assert se == S["src_elem"]
    bn = b.cpu().numpy()
    assert rel_norm(bn, S["b"]) < ELEM_TOL
    # petgem's KSP: -ksp_type gmres (restart 30) -pc_type jacobi, complex128
    x, info = mesh.solve(vals, b, rtol=1e-8, ksp="gmres", precond="jacobi", precision="fp64", restart=30,
                         max_it=20000)
    assert info.status == 0 and info.relres <= 1e-8
    xn = x.cpu().numpy()
    assert np.linalg.norm(A @ xn - S["b"]) <= 1e-8 * np.linalg.norm(S["b"]) * 1.01
    xd = osolve.direct(A, S["b"])
    Fd, _ = system.receiver_fields(S, xd, model.nodes, model.tets, 1, model.receivers, f)
    F, keep = mesh.receiver_fields(x, model.receivers, f)
    assert bool(keep.all()) and F.shape[0] == len(model.receivers)
    assert rel_norm(F.cpu().numpy()[:, :3], Fd[:, :3]) < FIELD_TOL


def test_config1_full_size_assembly_vs_oracle():
    """The 32^3 p = 2 workload with the benchmark's exact calls, FP64 and
    double-float, against the oracle's elemental loop + COO assembly + PEC."""
    from oracle import system
    from petgem_gb300 import synthetic
    from petgem_gb300.engine import DeviceMesh
    model = synthetic.config1(32)
    f = model.source["frequency"]
    S = system.csem_system(model.nodes, model.tets, model.sigma, 2, model.source,
                           processes=min(16, os.cpu_count() or 1))
    A = S["A"]
    mesh = DeviceMesh(model.nodes, model.tets, 2)
    assert (mesh.T, mesh.N, mesh.nnz) == (196608, 1276096, 54751616)
    rp, cl = mesh.rowptr.cpu().numpy(), mesh.col.cpu().numpy()
    assert np.array_equal(rp, A.indptr) and np.array_equal(cl, A.indices)
    rows = np.repeat(np.arange(mesh.N), np.diff(rp))
    rowmax = np.zeros(mesh.N)
    np.maximum.at(rowmax, rows, np.abs(A.data))
    for ar in ("fp64", "df64"):
        v = _bench_assembly(mesh, model.sigma, f, ar).cpu().numpy()
        assert rel_norm(v, A.data) < ELEM_TOL, ar
        # entrywise, against the largest entry of each row
        assert float(np.max(np.abs(v - A.data) / rowmax[rows])) < ELEM_TOL, ar
    b = torch.zeros(mesh.N, dtype=torch.complex128, device="cuda")
    mesh.source_rhs(model.source, mesh.locate_source(model.source), b)
    mesh.pec_rhs(b)
    assert rel_norm(b.cpu().numpy(), S["b"]) < ELEM_TOL
