"""Oracle: magnetotelluric (MT) plane-wave right-hand side and impedances.

Test infrastructure only (see ``oracle/__init__.py``).  Restates, with numpy
and scipy.sparse:

* boundary faces and their elements (petgem/mesh.py:128-221),
* the box side of every boundary face (computeFacePlane, mesh.py:324-429),
* the 1-D MT field (eval_MT1D, petgem/mt1d.py:21-191: linear elements,
  3-point Gauss rule, essential conditions by row/column elimination, sparse
  direct solve, the reference's linear interpolation rules),
* the boundary-face integral of the tangential excitation
  (petgem/solver.py:318-512 with hvfem.py:2556-2780),
* computeImpedance (petgem/postprocessing.py:619-688).

The triangle rule is an argument: the reference's own rule (from the golden
fixture) to pin against petgem, or the product's rule to compare kernels.
"""
import numpy as np
import scipy.sparse as sp
import scipy.sparse.linalg as spla

from . import basis, fem

FACE_VERTS = np.array([[0, 1, 2], [0, 1, 3], [1, 2, 3], [0, 2, 3]])        # hvfem.py:2668-2683
NREF = np.array([[0.0, 0.0, -1.0], [0.0, -1.0, 0.0], [1.0, 1.0, 1.0] / np.sqrt(3.0), [-1.0, 0.0, 0.0]])
# e = u * DIRS[polarisation - 1][plane]                                        hvfem.py:2556-2624
DIRS = np.array([[[1, 0, 0], [0, 0, -1], [0, 0, 0], [0, 0, 1], [0, 0, 0], [-1, 0, 0]],
                 [[0, 1, 0], [0, 0, 0], [0, 0, -1], [0, 0, 0], [0, 0, 1], [0, -1, 0]]], dtype=np.float64)


def boundary_faces(elemsF, n_faces):
    """(bFaces ascending, element, local face) of the faces owned by one element."""
    elemsF = np.asarray(elemsF)
    cnt = np.bincount(elemsF.reshape(-1), minlength=n_faces)
    bfaces = np.nonzero(cnt == 1)[0]
    owner = np.full(n_faces, -1, dtype=np.int64)
    local = np.full(n_faces, -1, dtype=np.int64)
    T = elemsF.shape[0]
    # lowest element first (invConnectivity fills in ascending element order)
    for lf in range(4):
        f = elemsF[:, lf]
        m = (cnt[f] == 1)
        owner[f[m]] = np.nonzero(m)[0]
        local[f[m]] = lf
    assert T > 0
    return bfaces, owner[bfaces], local[bfaces]


def face_planes(nodes, facesN, bfaces):
    """computeFacePlane: 0 bottom, 1 left, 2 front, 3 right, 4 back, 5 top."""
    lo, hi = nodes.min(axis=0), nodes.max(axis=0)
    a = np.array([lo[0], lo[1], lo[2]]); b = np.array([hi[0], lo[1], lo[2]])
    c = np.array([lo[0], hi[1], lo[2]]); d = np.array([hi[0], hi[1], lo[2]])
    e = np.array([lo[0], lo[1], hi[2]]); f = np.array([hi[0], lo[1], hi[2]])
    g = np.array([lo[0], hi[1], hi[2]]); h = np.array([hi[0], hi[1], hi[2]])
    normals = [np.cross(a - b, a - c), np.cross(a - c, a - e), np.cross(a - b, a - e),
               np.cross(b - d, b - f), np.cross(d - c, d - h), np.cross(e - f, e - g)]
    base = [a, a, a, b, d, e]
    out = np.empty(len(bfaces), dtype=np.int64)
    for i, fc in enumerate(bfaces):
        cen = np.sum(nodes[facesN[fc]], axis=0) / 3.0
        vals = np.array([np.dot(nv, cen - bp) for nv, bp in zip(normals, base)])
        out[i] = np.nonzero(np.abs(vals) < 1e-13)[0][0]
    return out


def mt1d_field(za, zb, sigma0, x0, omega, mu, n_nodes=10 ** 6, interpolate_at=None):
    """eval_MT1D with degree 1 and u(za) = 1, u(zb) = 0 (mt1d.py:21-76)."""
    n = n_nodes
    x = np.linspace(za, zb, n)
    xu, pos = np.unique(np.asarray(x0, dtype=np.float64), return_index=True)
    # the reference interpolates sigma with its own loop; vectorised here
    # with the same rules (first interval extrapolates, 0 above the last sample)
    o = np.argsort(xu)
    xs, ss = xu[o], np.asarray(sigma0, dtype=np.float64)[pos][o]
    sig = np.zeros(n)
    if xs.size >= 2:
        i = np.maximum(np.searchsorted(xs, x, side="left"), 1)
        ok = i <= xs.size - 1
        i = np.minimum(i, xs.size - 1)
        xi = (2 * x - xs[i] - xs[i - 1]) / (xs[i] - xs[i - 1])
        sig[ok] = (0.5 * (1 - xi) * ss[i - 1] + 0.5 * (1 + xi) * ss[i])[ok]
    gx, gw = np.polynomial.legendre.leggauss(3)
    h = x[1:] - x[:-1]
    rows, cols, mv, kv = [], [], [], []
    e = np.arange(n - 1)
    for a in range(2):
        for b in range(2):
            m = np.zeros(n - 1)
            for g, w in zip(gx, gw):
                N = np.array([0.5 * (1 - g), 0.5 * (1 + g)])
                sg = N[0] * sig[:-1] + N[1] * sig[1:]
                m += w * 0.5 * h * sg * N[a] * N[b]
            rows.append(e + a)
            cols.append(e + b)
            mv.append(m)
            kv.append((1.0 if a == b else -1.0) / h)
    M = sp.coo_matrix((np.concatenate(mv), (np.concatenate(rows), np.concatenate(cols))), shape=(n, n)).tocsr()
    K = sp.coo_matrix((np.concatenate(kv), (np.concatenate(rows), np.concatenate(cols))), shape=(n, n)).tocsr()
    A = (K + 1j * omega * mu * M).tolil()
    f = -A[:, 0].toarray().ravel() * 1.0
    for node, val in ((0, 1.0), (n - 1, 0.0)):
        A[node, :] = 0
        A[:, node] = 0
        A[node, node] = 1
        f[node] = val
    u = spla.spsolve(A.tocsr(), f)
    if interpolate_at is None:
        return u
    pts = np.asarray(interpolate_at, dtype=np.float64)
    uniq, inv = np.unique(pts.reshape(-1), return_inverse=True)
    xo = np.argsort(x)
    xs, us = x[xo], u[xo]
    i = np.maximum(np.searchsorted(xs, uniq, side="left"), 1)
    ok = i <= xs.size - 1
    i = np.minimum(i, xs.size - 1)
    xi = (2 * uniq - xs[i] - xs[i - 1]) / (xs[i] - xs[i - 1])
    val = np.where(ok, 0.5 * (1 - xi) * us[i - 1] + 0.5 * (1 + xi) * us[i], 0.0)
    return val[inv].reshape(pts.shape)


def face_points(coords, lf, rule_pts):
    """Reference-tet points and physical points of the rule on local face lf."""
    ref = np.array([[0.0, 0, 0], [1, 0, 0], [0, 1, 0], [0, 0, 1]])
    fv = FACE_VERTS[lf]
    r3 = ref[fv[0]] + np.outer(rule_pts[:, 0], ref[fv[1]] - ref[fv[0]]) + np.outer(rule_pts[:, 1],
                                                                                   ref[fv[2]] - ref[fv[0]])
    lam = np.stack([1 - r3.sum(1), r3[:, 0], r3[:, 1], r3[:, 2]], axis=1)
    return r3, lam @ coords


class Boundary:
    """Mesh-side data of the MT excitation (oracle)."""

    def __init__(self, nodes, tets, elemsF, facesN, n_faces):
        self.nodes = np.asarray(nodes, dtype=np.float64)
        self.tets = np.asarray(tets)
        self.bfaces, self.belem, self.blocal = boundary_faces(elemsF, n_faces)
        self.planes = face_planes(self.nodes, facesN, self.bfaces)


def mt_field_at_faces(bd, sigma, rule_pts, omega, mu=fem.MU0, n_nodes=10 ** 6):
    """u at the z of every face rule point (solver.py:318-395)."""
    zpts = np.zeros((len(bd.bfaces), len(rule_pts)))
    cz, s4 = [], []
    for i, (e, lf) in enumerate(zip(bd.belem, bd.blocal)):
        coords = bd.nodes[bd.tets[e]]
        _, xyz = face_points(coords, lf, rule_pts)
        zpts[i] = xyz[:, 2]
        if bd.planes[i] == 3:
            cz.append((np.sum(coords[FACE_VERTS[lf]], axis=0) / 3.0)[2])
            s4.append(sigma[e, 0])
    z = bd.nodes[bd.tets][:, :, 2]
    return mt1d_field(z.max(), z.min(), np.asarray(s4), np.asarray(cz), omega, mu, n_nodes, zpts), zpts


def mt_rhs(bd, eo, fo, dofs, ndofs, p, u, rule_pts, rule_w, omega, pol, mu=fem.MU0):
    """b for one polarisation (1 = x, 2 = y): solver.py:397-512."""
    b = np.zeros(ndofs, dtype=np.complex128)
    const = 1j * omega * mu
    for i, (e, lf) in enumerate(zip(bd.belem, bd.blocal)):
        coords = bd.nodes[bd.tets[e]]
        J, iJ = fem.jacobian(coords)
        nv = iJ @ NREF[lf]
        nu = nv / np.linalg.norm(nv)
        fvc = coords[FACE_VERTS[lf]]
        det2 = np.linalg.norm(np.cross(fvc[1] - fvc[0], fvc[2] - fvc[0]))
        d = DIRS[pol - 1][bd.planes[i]]
        r3, _ = face_points(coords, lf, rule_pts)
        contrib = np.zeros(dofs.shape[1], dtype=np.complex128)
        for k in range(len(rule_w)):
            Nref, _ = basis.shape3d(r3[k][None, :], p, tuple(int(v) for v in eo[e]), tuple(int(v) for v in fo[e]))
            Nr = iJ @ Nref[:, :, 0]
            tang = Nr - np.outer(nu, nu @ Nr)          # (n x N) x n
            contrib += rule_w[k] * det2 * (d @ tang) * u[i, k]
        np.add.at(b, dofs[e], contrib * const)
    return b


def impedance(fields, omega, mu):
    """computeImpedance (postprocessing.py:619-688): apparent resistivity,
    phase, tipper and impedance from two polarisations' (R, 6) fields."""
    E1x, E1y, E2x, E2y = fields[0][:, 0], fields[0][:, 1], fields[1][:, 0], fields[1][:, 1]
    H1x, H1y, H1z = fields[0][:, 3], fields[0][:, 4], fields[0][:, 5]
    H2x, H2y, H2z = fields[1][:, 3], fields[1][:, 4], fields[1][:, 5]
    m1 = H2y * H2x * H1y - H2y * H2y * H1x
    m2 = H2x * H2x * H1y - H2y * H2x * H1x
    m3 = E2x * H2x * H1y - H2y * E2x * H1x
    m4 = H2y * E2y * H1y - H2y * H2y * E1y
    m5 = H2x * E2y * H1y - H2y * H2x * E1y
    m6 = H2y * H2x * E1y - E2y * H2y * H1x
    m7 = H2x * H2x * E1y - E2y * H2x * H1x
    d = H1x * m1 - H1y * m2
    Z = [(E1x * m1 - H1y * m3) / d, (H1x * m3 - E1x * m2) / d, (H1x * m4 - H1y * m5) / d, (H1x * m6 - H1y * m7) / d]
    rho = [np.abs(z) ** 2 / (mu * omega) for z in Z]
    phase = [(180.0 / np.pi * np.arctan(-np.imag(z) / np.real(z))) % 360 for z in Z]
    c = H1x * H2y
    t1 = (H2z / H2y - (H1z * H2x) / c) / (1.0 - (H1y * H2x) / c)
    t2 = (H1z - t1 * H1y) / H1x
    return rho, phase, [t2, t1], Z
