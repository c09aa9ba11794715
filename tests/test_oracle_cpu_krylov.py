"""The CPU baseline solvers (compiled C + OpenMP COCG and petgem's restarted
GMRES(m) + Jacobi, measurement infrastructure) solve the reference's
assembled system (golden A, b, PEC)."""
import numpy as np
import pytest
import scipy.sparse as sp

from oracle import fem
from tests.helpers import load


def test_cpu_cocg_solves_golden_system():
    try:
        from oracle import build_cpu
        build_cpu.build()
    except Exception as exc:   # no compiler in this environment
        pytest.skip(f"CPU baseline solver not buildable: {exc}")
    g = load("system_n2.npz")
    A = sp.csr_matrix((g["p2_data"], g["p2_indices"], g["p2_indptr"]))
    Ap, bp = fem.apply_pec(A, g["p2_b"], g["p2_bnd"])
    x, its, rel, st = build_cpu.cocg(Ap.indptr, Ap.indices, Ap.data, bp, 10000, 1e-10)
    assert st == 0 and rel <= 1e-10
    assert np.linalg.norm(Ap @ x - bp) <= 1.01e-10 * np.linalg.norm(bp)


@pytest.mark.parametrize("reorth", [False, True])
def test_cpu_gmres_matches_scipy_gmres(reorth):
    """The compiled GMRES(30) + Jacobi (petgem's KSP, measurement
    infrastructure) solves the golden system to its true-residual target and
    takes the Arnoldi steps scipy's restarted GMRES takes on the same
    right-preconditioned system (the same algorithm; rounding only)."""
    try:
        from oracle import build_cpu
        build_cpu.build()
    except Exception as exc:   # no compiler in this environment
        pytest.skip(f"CPU baseline solver not buildable: {exc}")
    import scipy.sparse.linalg as spla
    g = load("system_n2.npz")
    A = sp.csr_matrix((g["p2_data"], g["p2_indices"], g["p2_indptr"]))
    Ap, bp = fem.apply_pec(A, g["p2_b"], g["p2_bnd"])
    x, its, rel, st = build_cpu.gmres(Ap.indptr, Ap.indices, Ap.data, bp, 30, 20000, 1e-8, reorth)
    assert st == 0 and rel <= 1e-8
    assert np.linalg.norm(Ap @ x - bp) <= 1.01e-8 * np.linalg.norm(bp)
    # scipy on A D^-1 (right Jacobi preconditioning), the same restart and target
    d = Ap.diagonal()
    AD = (Ap @ sp.diags(1.0 / d)).tocsr()
    count = [0]

    def cb(_):
        count[0] += 1

    y, info = spla.gmres(AD, bp, rtol=1e-8, atol=0.0, restart=30, maxiter=2000, callback=cb,
                         callback_type="pr_norm")
    assert info == 0
    assert abs(its - count[0]) <= max(3, 0.05 * count[0])
    # a restart shorter than needed is cut at max_it with status 1
    _, its2, _, st2 = build_cpu.gmres(Ap.indptr, Ap.indices, Ap.data, bp, 5, 7, 1e-8, reorth)
    assert st2 == 1 and its2 == 7
