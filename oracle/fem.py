"""Oracle: elemental matrices, assembly, PEC, point source and receiver
interpolation (numpy / scipy.sparse).

Test infrastructure only (see ``oracle/__init__.py``).
"""
import numpy as np
import scipy.sparse as sp

from . import basis

MU0 = 4.0 * np.pi * 1e-7          # petgem/solver.py:174


def jacobian(coords):
    """J with rows x1-x0, x2-x0, x3-x0 and its inverse (petgem/hvfem.py:101-119)."""
    c = np.asarray(coords, dtype=np.float64).reshape(4, 3)
    J = c[1:] - c[0]
    return J, np.linalg.inv(J)


def elemental_matrices(eo, fo, J, invJ, p, sigma):
    """Elemental mass M and stiffness K (petgem/hvfem.py:223-316).

    M = det(J) sum_g w_g (invJ N_g)^T diag(sh, sh, sv) (invJ N_g)
    K = det(J) sum_g w_g c_g^T c_g,  c_g = (C_g^T J) / det(J)   (mu_r = 1)
    with the SIGNED det(J), as in the reference.
    """
    N, C, w = basis.reference_basis_at_rule(p, tuple(int(v) for v in eo),
                                            tuple(int(v) for v in fo))
    det = np.linalg.det(J)
    D = np.array([sigma[0], sigma[0], sigma[1]], dtype=np.float64)
    Nr = np.einsum("ab,bjg->ajg", invJ, N)
    M = np.einsum("g,ajg,a,akg->jk", w, Nr, D, Nr) * det
    Cr = np.einsum("ajg,ab->bjg", C, J) / det
    K = np.einsum("g,ajg,akg->jk", w, Cr, Cr) * det
    return M, K


def element_matrices_batch(coords, eo, fo, sigma, p):
    """(M, K) for every element: coords (T,4,3), eo (T,6), fo (T,4), sigma (T,2)."""
    T = coords.shape[0]
    nd = basis.ndof(p)
    M = np.empty((T, nd, nd))
    K = np.empty((T, nd, nd))
    for e in range(T):
        J, iJ = jacobian(coords[e])
        M[e], K[e] = elemental_matrices(eo[e], fo[e], J, iJ, p, sigma[e])
    return M, K


def assemble(M, K, dofs, ndofs, frequency):
    """A = sum_e P_e^T (K_e - i omega mu M_e) P_e as scipy CSR
    (petgem/solver.py:182-235; PETSc ADD_VALUES is restated as COO sum)."""
    omega = 2.0 * np.pi * frequency
    Ae = K - 1j * omega * MU0 * M
    T, nd = dofs.shape
    rows = np.repeat(dofs, nd, axis=1).reshape(-1)
    cols = np.tile(dofs, (1, nd)).reshape(-1)
    A = sp.coo_matrix((Ae.reshape(-1), (rows, cols)), shape=(ndofs, ndofs)).tocsr()
    A.sum_duplicates()
    A.sort_indices()
    return A


def apply_pec(A, b, bnd):
    """PETSc zeroRowsColumns(rows, diag=1) and b[rows] = 0 (solver.py:552-577)."""
    n = A.shape[0]
    keep = np.ones(n)
    keep[np.asarray(bnd, dtype=np.int64)] = 0.0
    Dk = sp.diags(keep)
    A2 = (Dk @ A @ Dk + sp.diags(1.0 - keep)).tocsr()
    A2.sort_indices()
    b2 = np.array(b, dtype=np.complex128, copy=True)
    b2[np.asarray(bnd, dtype=np.int64)] = 0.0
    return A2, b2


def source_rotation(azimuth, dip):
    """Unit dipole direction after azimuth (x-y) and dip (x-z) rotations
    (petgem/hvfem.py:2303-2344)."""
    a = np.deg2rad(azimuth)
    b = np.deg2rad(dip)
    M1 = np.array([[np.cos(a), -np.sin(a), 0.0], [np.sin(a), np.cos(a), 0.0], [0.0, 0.0, 1.0]])
    M2 = np.array([[np.cos(b), 0.0, -np.sin(b)], [0.0, 1.0, 0.0], [np.sin(b), 0.0, np.cos(b)]])
    return (M1 @ M2) @ np.array([1.0, 0.0, 0.0])


def xyz_to_reference(coords, pts):
    """Reference coordinates of physical points in one tet
    (petgem/hvfem.py:2347-2490): solve J^T xi = x - x0."""
    J, _ = jacobian(coords)
    c = np.asarray(coords).reshape(4, 3)
    return np.linalg.solve(J.T, (np.atleast_2d(pts) - c[0]).T).T


def basis_at(coords, eo, fo, p, xi):
    """Physical basis and curl at reference points (petgem/hvfem.py:2493-2553).

    Returns (N, C), each (3, nd, npts): N = invJ N_ref, C = J^T C_ref / det(J^T).
    """
    J, iJ = jacobian(coords)
    Nref, Cref = basis.shape3d(xi, p, eo, fo)
    N = np.einsum("ab,bjg->ajg", iJ, Nref)
    C = np.einsum("ba,bjg->ajg", J, Cref) / np.linalg.det(J.T)
    return N, C


def locate(nodes, elemsN, pts, tol=1e-12):
    """Index of the first (lowest-index) tet containing each point, -1 if none.

    Restates the brute-force point location of scipy's
    ``Delaunay.find_simplex(bruteforce=True, tol=1e-12)`` on the mesh's own
    connectivity (petgem/preprocessing.py:414-425, postprocessing.py:532-539).
    """
    c = nodes[elemsN]                                  # (T,4,3)
    J = c[:, 1:] - c[:, :1]                            # (T,3,3) rows = edges
    out = np.full(len(pts), -1, dtype=np.int64)
    for i, x in enumerate(np.atleast_2d(pts)):
        rhs = (x - c[:, 0])[:, :, None]
        xi = np.linalg.solve(np.transpose(J, (0, 2, 1)), rhs)[:, :, 0]
        lam = np.concatenate([1.0 - xi.sum(1, keepdims=True), xi], axis=1)
        ok = np.all((lam >= -tol) & (lam <= 1.0 + tol), axis=1)
        hit = np.nonzero(ok)[0]
        if len(hit):
            out[i] = hit[0]
    return out


def source_vector(nodes, elemsN, eo, fo, dofs, ndofs, p, src):
    """Point-dipole RHS b (petgem/solver.py:247-316, preprocessing.py:404-464).

    src: dict with position, azimuth, dip, current, length, frequency.
    """
    pos = np.asarray(src["position"], dtype=np.float64)
    e = int(locate(nodes, elemsN, pos[None, :])[0])
    if e < 0:
        raise ValueError("source outside the mesh")
    coords = nodes[elemsN[e]]
    rot = source_rotation(src["azimuth"], src["dip"])
    IL = src["current"] * src["length"]
    field = rot[0] * np.array([IL, 0, 0]) + rot[1] * np.array([0, IL, 0]) + rot[2] * np.array([0, 0, IL])
    xi = xyz_to_reference(coords, pos)
    N, _ = basis_at(coords, eo[e], fo[e], p, xi)
    omega = 2.0 * np.pi * src["frequency"]
    contrib = (field @ N[:, :, 0]) * (1j * omega * MU0)
    b = np.zeros(ndofs, dtype=np.complex128)
    np.add.at(b, dofs[e], contrib)
    return b, e


def interpolate_fields(x, nodes, elemsN, eo, fo, dofs, p, pts, frequency):
    """E and H = curl E / (i omega mu) at receivers (postprocessing.py:479-616).

    Receivers outside the mesh are dropped, as in the reference.  Returns
    (fields (R',6) complex128, element index per kept receiver).
    """
    el = locate(nodes, elemsN, pts)
    keep = el >= 0
    pts = np.atleast_2d(pts)[keep]
    el = el[keep]
    F = np.zeros((len(pts), 6), dtype=np.complex128)
    for i, (e, xpt) in enumerate(zip(el, pts)):
        coords = nodes[elemsN[e]]
        xi = xyz_to_reference(coords, xpt)
        N, C = basis_at(coords, eo[e], fo[e], p, xi)
        xe = x[dofs[e]]
        F[i, :3] = N[:, :, 0] @ xe
        F[i, 3:] = C[:, :, 0] @ xe
    F[:, 3:] /= 1j * 2.0 * np.pi * frequency * MU0
    return F, el


def node_fields(x, nodes, elemsN, eo, fo, dofs, p, frequency, scale=0.9999):
    """Nodal E and H for visualisation (petgem/postprocessing.py:173-260):
    per element, E and curl E at the vertices pulled towards the centroid by
    `scale`; summed per node in element order, divided by the number of
    elements sharing the node; H = curl E / (i omega mu)."""
    nn = nodes.shape[0]
    acc = np.zeros((nn, 6), dtype=np.complex128)
    cnt = np.zeros(nn)
    for e in range(elemsN.shape[0]):
        coords = nodes[elemsN[e]]
        cen = coords.sum(axis=0) / 4.0
        pts = cen + (coords - cen) * scale
        xi = xyz_to_reference(coords, pts)
        N, C = basis_at(coords, eo[e], fo[e], p, xi)
        xe = x[dofs[e]]
        for k in range(4):
            acc[elemsN[e, k], :3] += N[:, :, k] @ xe
            acc[elemsN[e, k], 3:] += C[:, :, k] @ xe
            cnt[elemsN[e, k]] += 1
    acc /= cnt[:, None]
    acc[:, 3:] /= 1j * 2.0 * np.pi * frequency * MU0
    return acc
