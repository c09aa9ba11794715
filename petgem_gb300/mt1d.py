"""1-D magnetotelluric field for the MT boundary excitation (host side).

petgem solves, on [zb, za], the 1-D problem  -u'' + i omega mu sigma(z) u = 0
with u(za) = 1, u(zb) = 0 by linear finite elements on ~1e6 nodes, with
sigma(z) linearly interpolated from boundary-element samples, and reads u at
the z of every face quadrature point (petgem/mt1d.py:21-76,
eval_MT1D).  The system is tridiagonal, so here it is assembled in closed
vectorised form and solved with a banded LU (LAPACK gbsv) instead of a
general sparse factorisation; the element integrals use the same 3-point
Gauss rule on the same (descending) node grid, and the interpolation keeps
the reference's rules: points below the first sample extrapolate from the
first interval, points above the last sample get 0 (mt1d.py:101-133).

This is the one part of the MT right-hand side that stays on the host: a
1-D solve of O(1e6) unknowns, independent of the 3-D mesh size.
"""
import numpy as np
from scipy.linalg import solve_banded

# 3-point Gauss-Legendre rule on [-1, 1] (exact for the cubic element integrands)
_GX = np.array([np.sqrt(0.6), 0.0, -np.sqrt(0.6)])
_GW = np.array([5.0 / 9.0, 8.0 / 9.0, 5.0 / 9.0])


def linearInterp1D(x, u, xp):
    """u given at x, linearly interpolated at xp (petgem/mt1d.py:101-133):
    below x.min() the first interval extrapolates, above x.max() the value
    is 0."""
    x = np.asarray(x, dtype=np.float64)
    xp = np.asarray(xp, dtype=np.float64)
    o = np.argsort(x)
    xs, us = x[o], np.asarray(u)[o]
    out = np.zeros(xp.shape, dtype=us.dtype)
    if xs.size < 2:
        return out
    i = np.maximum(np.searchsorted(xs, xp, side="left"), 1)
    ok = i <= xs.size - 1
    i = np.minimum(i, xs.size - 1)
    x0, x1 = xs[i - 1], xs[i]
    xi = (2.0 * xp - x1 - x0) / (x1 - x0)
    val = 0.5 * (1.0 - xi) * us[i - 1] + 0.5 * (1.0 + xi) * us[i]
    out[ok] = val[ok]
    return out


def eval_MT1D(za, zb, za_D, zb_D, sigma0, x0, omega, mu, n_nodes_ref, degree=1, interpolate_at=None,
              return_nodes=False):
    """petgem/mt1d.py:21-76 for linear elements (the only degree the
    reference implements)."""
    if degree != 1:
        raise NotImplementedError("eval_MT1D: only linear elements (degree 1), as in the reference")
    n_el = int(np.ceil((n_nodes_ref - 1) / degree))
    n = n_el * degree + 1
    x = np.linspace(za, zb, n)
    xu, pos = np.unique(np.asarray(x0, dtype=np.float64), return_index=True)
    sig = linearInterp1D(xu, np.asarray(sigma0, dtype=np.float64)[pos], x)
    # element integrals with the 3-point rule: h is signed (nodes run downwards)
    h = x[1:] - x[:-1]
    s0, s1 = sig[:-1], sig[1:]
    m00 = np.zeros(n_el)
    m01 = np.zeros(n_el)
    m11 = np.zeros(n_el)
    for g, w in zip(_GX, _GW):
        n0, n1 = 0.5 * (1.0 - g), 0.5 * (1.0 + g)
        sg = n0 * s0 + n1 * s1
        dl = w * 0.5 * h
        m00 += dl * sg * n0 * n0
        m01 += dl * sg * n0 * n1
        m11 += dl * sg * n1 * n1
    k = 1.0 / h                                  # sum_g w (h/2) (1/(h/2))^2 (1/4) = 1/h
    c = 1j * omega * mu
    diag = np.zeros(n, dtype=np.complex128)
    diag[:-1] += k + c * m00
    diag[1:] += k + c * m11
    off = -k + c * m01                           # (e, e+1) and (e+1, e)
    # essential conditions u(za) = za_D, u(zb) = zb_D (row/column elimination)
    f = np.zeros(n, dtype=np.complex128)
    f[1] -= off[0] * za_D
    f[n - 2] -= off[n - 2] * zb_D
    f[0], f[n - 1] = za_D, zb_D
    diag[0] = diag[n - 1] = 1.0
    ab = np.zeros((3, n), dtype=np.complex128)
    ab[0, 1:] = off                              # super-diagonal
    ab[1] = diag
    ab[2, :-1] = off                             # sub-diagonal
    ab[0, 1] = 0.0                               # row 0 is the identity
    ab[2, 0] = 0.0                               # column 0 eliminated
    ab[0, n - 1] = 0.0                           # column n-1 eliminated
    ab[2, n - 2] = 0.0                           # row n-1 is the identity
    u = solve_banded((1, 1), ab, f)
    if interpolate_at is None:
        return (u, x) if return_nodes else u
    pts = np.asarray(interpolate_at, dtype=np.float64)
    uniq, inv = np.unique(pts.reshape(-1), return_inverse=True)
    sol = linearInterp1D(x, u, uniq)[inv].reshape(pts.shape)
    return (sol, x) if return_nodes else sol


def triangle_rule(degree):
    """Collapsed Gauss-Legendre rule on the triangle (0,0),(1,0),(0,1), exact
    for polynomials of total degree <= degree: (points (n, 2), weights (n,)),
    weights summing to 1/2."""
    m = (degree + 3) // 2          # the collapsed direction carries one degree more
    t, w = np.polynomial.legendre.leggauss(m)
    t = 0.5 * (t + 1.0)
    w = 0.5 * w
    s_, v_ = np.meshgrid(t, t, indexing="ij")
    ws, wv = np.meshgrid(w, w, indexing="ij")
    pts = np.stack([(s_ * (1.0 - v_)).ravel(), v_.ravel()], axis=1)
    return pts, (ws * wv * (1.0 - v_)).ravel()
