"""Oracle: hierarchical H(curl) basis on the reference tetrahedron (numpy).

Test infrastructure only (see ``oracle/__init__.py``).

Restates petgem's ``shape3DETet`` family (petgem/hvfem.py:319-1052), which
implements the orientation-embedded Nedelec (first kind) shape functions of
Fuentes, Keith, Demkowicz & Nagaraj (2015).  Everything here is vectorised
over evaluation points: scalar fields have shape ``(npts,)``, vector fields
``(3, npts)``, gradients of affine coordinates are constant ``(3,)`` vectors.

DOF order per element (hvfem.py:363-463): 6 edges x p functions, then 4 faces
x p(p-1) functions (two families interleaved), then p(p-1)(p-2)/2 bubbles
(three families interleaved).
"""
import functools

import numpy as np

# local vertex pairs of the 6 edges, before orientation (hvfem.py:881-951)
EDGE_VERTS = ((0, 1), (1, 2), (0, 2), (0, 3), (1, 3), (2, 3))
# local vertex triples of the 4 faces, before orientation (hvfem.py:954-1016)
FACE_VERTS = ((0, 1, 2), (0, 1, 3), (1, 2, 3), (0, 2, 3))
# face orientation code -> permutation of the face's vertex triple (hvfem.py:825-878)
FACE_PERM = ((0, 1, 2), (1, 2, 0), (2, 0, 1), (0, 2, 1), (1, 0, 2), (2, 1, 0))
# gradients of the affine coordinates on the reference tet (hvfem.py:1019-1052)
DLAM = (np.array([-1.0, -1.0, -1.0]), np.array([1.0, 0.0, 0.0]),
        np.array([0.0, 1.0, 0.0]), np.array([0.0, 0.0, 1.0]))


def ndof(p):
    """DOFs per element, p(p+2)(p+3)/2 (hvfem.py:48)."""
    return p * (p + 2) * (p + 3) // 2


def legendre_scaled(s, t, n):
    """Shifted, scaled Legendre P_0..P_{n-1}(s; t) (hvfem.py:629-664)."""
    P = [np.ones_like(s)]
    if n >= 2:
        y = 2.0 * s - t
        P.append(y)
        tt = t * t
        for i in range(1, n - 1):
            P.append(((2.0 * i + 1.0) * y * P[i] - i * tt * P[i - 1]) / (i + 1.0))
    return P


def jacobi_scaled(s, t, alpha, n):
    """Shifted, scaled Jacobi P^alpha_0..P^alpha_n(s; t) (hvfem.py:733-788)."""
    P = [np.ones_like(s)]
    if n >= 1:
        y = 2.0 * s - t
        P.append(y + alpha * s)
        tt = t * t
        for j in range(2, n + 1):
            a = 2.0 * j * (j + alpha) * (2.0 * j + alpha - 2.0)
            b = 2.0 * j + alpha - 1.0
            c = (2.0 * j + alpha) * (2.0 * j + alpha - 2.0)
            d = 2.0 * (j + alpha - 1.0) * (j - 1.0) * (2.0 * j + alpha)
            P.append((b * (c * y + alpha * alpha * t) * P[j - 1] - d * tt * P[j - 2]) / a)
    return P


def ijacobi_scaled(s, t, alpha, n):
    """Integrated scaled Jacobi L^alpha_j(s; t), j = 1..n (hvfem.py:667-730).

    Returns lists indexed by order j (index 0 unused): L_j, dL_j/ds (which is
    P^alpha_{j-1}) and dL_j/dt.
    """
    P = jacobi_scaled(s, t, alpha, n)
    L = [None, s * 1.0]
    Ls = [None, P[0]]
    Lt = [None, np.zeros_like(s)]
    tt = t * t
    for j in range(2, n + 1):
        tau = 2.0 * j + alpha
        L.append((j + alpha) / ((tau - 1.0) * tau) * P[j]
                 + alpha / ((tau - 2.0) * tau) * t * P[j - 1]
                 - (j - 1.0) / ((tau - 2.0) * (tau - 1.0)) * tt * P[j - 2])
        Ls.append(P[j - 1])
        Lt.append(-(j - 1.0) * (P[j - 1] + t * P[j - 2]) / (tau - 2.0))
    return L, Ls, Lt


def _outer(vec, scal):
    return vec[:, None] * scal[None, :]


def edge_family(s0, s1, d0, d1, n):
    """Edge ancillary functions E_i = P_i(s1; s0+s1) (s0 d1 - s1 d0), i < n,
    and their curls (i+2) P_i (d0 x d1) (hvfem.py:467-513, Idec=False)."""
    P = legendre_scaled(s1, s0 + s1, n)
    whitney = _outer(d1, s0) - _outer(d0, s1)
    c = np.cross(d0, d1)
    E = [P[i][None, :] * whitney for i in range(n)]
    C = [_outer(c, (i + 2.0) * P[i]) for i in range(n)]
    return E, C


def tri_family(s, d, n):
    """Triangle ancillary functions (hvfem.py:516-566, Idec=False).

    ``s`` = (s0, s1, s2) scalar fields, ``d`` their gradients.  Returns a dict
    keyed by (i, j), i >= 0, j >= 1, i + j <= n - 1, of (value, curl):
    value = E_i(s0, s1) * L^{2i+1}_j(s2; s0+s1+s2).
    """
    E, CE = edge_family(s[0], s[1], d[0], d[1], n - 1)
    t = s[0] + s[1] + s[2]
    dt = d[0] + d[1] + d[2]
    out = {}
    for i in range(0, n - 1):
        L, Ls, Lt = ijacobi_scaled(s[2], t, 2.0 * i + 1.0, n - 1 - i)
        for j in range(1, n - i):
            grad = _outer(d[2], Ls[j]) + _outer(dt, Lt[j])
            val = E[i] * L[j][None, :]
            curl = L[j][None, :] * CE[i] + np.cross(grad, E[i], axis=0)
            out[(i, j)] = (val, curl)
    return out


def shape3d(X, p, eo, fo):
    """H(curl) shape functions and curls at reference points (hvfem.py:319-464).

    X: (npts, 3) reference coordinates; p: order 1..6; eo: 6 edge flags
    (0/1); fo: 4 face codes (0..5).  Returns (N, C), each (3, nd, npts).
    """
    X = np.atleast_2d(np.asarray(X, dtype=np.float64))
    x, y, z = X[:, 0], X[:, 1], X[:, 2]
    lam = (1.0 - x - y - z, x * 1.0, y * 1.0, z * 1.0)
    N, C = [], []
    for e, (a, b) in enumerate(EDGE_VERTS):
        if eo[e]:
            a, b = b, a
        E, CE = edge_family(lam[a], lam[b], DLAM[a], DLAM[b], p)
        N += E
        C += CE
    if p >= 2:
        for f, verts in enumerate(FACE_VERTS):
            v = [verts[k] for k in FACE_PERM[int(fo[f])]]
            fams = []
            for rot in ((0, 1, 2), (1, 2, 0)):
                w = [v[k] for k in rot]
                fams.append(tri_family([lam[k] for k in w], [DLAM[k] for k in w], p))
            for k in range(1, p):
                for r in range(0, k):
                    for F in fams:
                        val, curl = F[(r, k - r)]
                        N.append(val)
                        C.append(curl)
    if p >= 3:
        fams = []
        for f in range(3):
            abcd = [(f + k) % 4 for k in range(4)]
            abc, dv = abcd[:3], abcd[3]
            T = tri_family([lam[k] for k in abc], [DLAM[k] for k in abc], p - 1)
            blend = {k: ijacobi_scaled(lam[dv], 1.0, 2.0 * k, p - 1 - k) for k in range(1, p - 1)}
            fams.append((T, dv, blend))
        for j in range(2, p):
            for k in range(1, j):
                for r in range(0, k):
                    q = j - k
                    for T, dv, blend in fams:
                        L, Ls, _ = blend[k]
                        val, curl = T[(r, k - r)]
                        N.append(val * L[q][None, :])
                        C.append(L[q][None, :] * curl
                                 + np.cross(_outer(DLAM[dv], Ls[q]), val, axis=0))
    N = np.stack(N, axis=1)
    C = np.stack(C, axis=1)
    assert N.shape[1] == ndof(p)
    return N, C


@functools.lru_cache(maxsize=None)
def tet_rule(degree):
    """Quadrature on the reference tet {x,y,z >= 0, x+y+z <= 1}, exact for
    total degree ``degree``: a collapsed (Duffy) Gauss-Legendre product rule.

    petgem integrates with tabulated rules of degree 2p (hvfem.py:1055-1610);
    the elemental integrands are polynomials of degree <= 2p, so any rule exact
    to that degree gives the same matrices up to rounding.
    """
    n = degree // 2 + 2
    g, w = np.polynomial.legendre.leggauss(n)
    g = 0.5 * (g + 1.0)
    w = 0.5 * w
    u, v, s = np.meshgrid(g, g, g, indexing="ij")
    wu, wv, ws = np.meshgrid(w, w, w, indexing="ij")
    pts = np.stack([u, v * (1.0 - u), s * (1.0 - u) * (1.0 - v)], axis=-1).reshape(-1, 3)
    wts = (wu * wv * ws * (1.0 - u) ** 2 * (1.0 - v)).reshape(-1)
    return pts, wts


@functools.lru_cache(maxsize=4096)
def reference_basis_at_rule(p, eo, fo):
    """Basis and curl at the degree-2p rule for one orientation tuple."""
    pts, wts = tet_rule(2 * p)
    N, C = shape3d(pts, p, eo, fo)
    return N, C, wts
