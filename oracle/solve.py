"""Oracle: scipy stand-ins for the PETSc KSP solve (petgem/solver.py:584-594).

Test infrastructure only (see ``oracle/__init__.py``).  PETSc is third-party
and absent; the benchmark's solve is ``-ksp_type gmres -pc_type jacobi
-ksp_rtol 1e-8`` (petgem's examples use ``-pc_type sor``), restated here with
scipy's GMRES and a Jacobi preconditioner, and a direct solve for tight
golden solutions.
"""
import numpy as np
import scipy.sparse as sp
import scipy.sparse.linalg as spla


def gmres_jacobi(A, b, rtol=1e-8, restart=30, maxiter=None):
    """Restarted GMRES(restart) with Jacobi; returns (x, inner iterations, true relres)."""
    D = A.diagonal()
    its = [0]

    def cb(_):
        its[0] += 1

    x, info = spla.gmres(A, b, M=sp.diags(1.0 / D), rtol=rtol, restart=restart,
                         maxiter=maxiter, callback=cb, callback_type="pr_norm")
    rel = np.linalg.norm(A @ x - b) / np.linalg.norm(b)
    return x, its[0], rel


def direct(A, b):
    """Sparse LU solve, for golden solutions far tighter than 1e-8."""
    return spla.spsolve(A.tocsc(), b)
