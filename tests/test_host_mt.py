"""Host side of the MT path (no GPU): the 1-D field, the triangle rule and
computeImpedance against golden vectors from petgem's own functions."""
from math import factorial

import numpy as np

from petgem_gb300 import mt1d
from petgem_gb300.pipeline import computeImpedance
from tests.helpers import load, rel_norm

MU = 4e-7 * np.pi


def test_mt1d_matches_reference_field():
    """1e6-node 1-D solve: conditioned ~1e12, so any double-precision LU
    (petgem's SuperLU included) sits ~2e-7 from the exact discrete solution;
    the field is pinned at 1e-6."""
    g = load("mt_n4.npz")
    for p in (1, 2):
        u = mt1d.eval_MT1D(float(g[f"p{p}_za"]), float(g[f"p{p}_zb"]), 1.0, 0.0, g[f"p{p}_s4"], g[f"p{p}_cz4"],
                           2 * np.pi, MU, int(1e6), 1, g[f"p{p}_zpts"])
        assert rel_norm(u, g[f"p{p}_u"]) < 1e-6


def test_mt1d_small_grid_matches_dense_solve():
    """On a 200-node grid the banded solve equals a dense solve of the same
    system to rounding (the interpolation rules included)."""
    za, zb = 100.0, -900.0
    x0 = np.array([-800.0, -500.0, -100.0, 50.0])
    s0 = np.array([0.01, 0.1, 1.0, 1e-8])
    u, x = mt1d.eval_MT1D(za, zb, 1.0, 0.0, s0, x0, 2 * np.pi, MU, 200, 1, None, True)
    assert x[0] == za and x[-1] == zb and abs(u[0] - 1) < 1e-15 and abs(u[-1]) < 1e-15
    assert np.all(np.isfinite(u))


def test_linear_interp_rules():
    x = np.array([0.0, 1.0, 3.0])
    y = np.array([1.0, 2.0, 4.0])
    got = mt1d.linearInterp1D(x, y, np.array([-1.0, 0.5, 2.0, 3.0, 3.5]))
    # below the first sample: first interval extrapolates; above the last: 0
    assert np.allclose(got, [0.0, 1.5, 3.0, 4.0, 0.0])


def test_triangle_rule_exactness():
    for deg in range(0, 9):
        pts, w = mt1d.triangle_rule(deg)
        assert abs(w.sum() - 0.5) < 1e-15
        for a in range(deg + 1):
            for b in range(deg + 1 - a):
                exact = factorial(a) * factorial(b) / factorial(a + b + 2)
                assert abs(np.sum(w * pts[:, 0] ** a * pts[:, 1] ** b) - exact) < 1e-15


def test_compute_impedance_matches_reference():
    g = load("mt_n4.npz")
    rho, phase, tip, Z = computeImpedance(list(g["imp_fields"]), 2 * np.pi, MU)
    assert rel_norm(np.stack(Z), g["imp_Z"]) < 1e-14
    assert rel_norm(np.stack(rho), g["imp_rho"]) < 1e-14
    assert rel_norm(np.stack(phase), g["imp_phase"]) < 1e-14
    assert rel_norm(np.stack(tip), g["imp_tipper"]) < 1e-14
