"""The CPU baseline solver (compiled C + OpenMP COCG, measurement
infrastructure) solves the reference's assembled system (golden A, b, PEC)."""
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
