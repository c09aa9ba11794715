"""Oracle: the discrete gradient of the order-p H1 space (p <= 3) into the
H(curl) space, on the CPU.

Test infrastructure only (see ``oracle/__init__.py``): the checker of
``pg_gradient_map``, never part of the product.

petgem has no counterpart: it leaves preconditioning to PETSc
(petgem/solver.py:584-594).  The map is pinned by its defining properties
instead of by petgem output: every column is exactly representable in
petgem's basis (the local projection residual is rounding), and the
curl-curl matrix petgem assembles annihilates it (K G = 0,
petgem/hvfem.py:223-316 for K).

Column order: mesh vertices; then (p >= 2) lambda_a lambda_b per edge; then
(p = 3) lambda_a lambda_b (lambda_b - lambda_a) per edge, (a, b) oriented by
the element's edge flag like petgem's edge functions (hvfem.py:881-951), and
lambda_a lambda_b lambda_c per face.  With vector=True (p >= 2) the vector P1
fields lambda_v e_d follow, 3 columns per vertex: they are also exactly
representable for p >= 2, by the reference projection of lambda_v e_k
combined with the element's Jacobian (covariant pull-back).  A row is taken
from the lowest-index element that holds its DOF.  Columns with an entry in a
PEC row are dropped.
"""
import functools

import numpy as np
import scipy.sparse as sp

from . import basis


def n_local(p):
    """H1 functions per element: 4 (p = 1), 10 (p = 2), 20 (p = 3)."""
    return {1: 4, 2: 10, 3: 20}[p]


def _local_gradients(pts, p, eo):
    """Reference gradients (3, W, npts) of the element's H1 functions."""
    x, y, z = pts[:, 0], pts[:, 1], pts[:, 2]
    lam = (1.0 - x - y - z, x, y, z)
    D = basis.DLAM
    one = np.ones_like(x)
    out = [np.outer(D[i], one) for i in range(4)]
    if p >= 2:
        for a, b in basis.EDGE_VERTS:
            out.append(np.outer(D[b], lam[a]) + np.outer(D[a], lam[b]))
    if p == 3:
        for e, (a, b) in enumerate(basis.EDGE_VERTS):
            if eo[e]:
                a, b = b, a
            g = np.outer(D[b], lam[a]) + np.outer(D[a], lam[b])
            out.append(g * (lam[b] - lam[a])[None, :] + np.outer(D[b] - D[a], lam[a] * lam[b]))
        for a, b, c in basis.FACE_VERTS:
            out.append(np.outer(D[a], lam[b] * lam[c]) + np.outer(D[b], lam[a] * lam[c])
                       + np.outer(D[c], lam[a] * lam[b]))
    return np.stack(out, axis=1)


@functools.lru_cache(maxsize=4096)
def local_coefficients(p, eo, fo):
    """C (nd, W): grad(phi_q) = sum_i C[i, q] N_i on the reference element, by
    exact L2 projection; entries at or below 1e-8 of their column's largest
    are set to 0 (for p <= 3 a coefficient is either >= 0.1 or rounding
    below 1e-11 of an exact zero).  Returns (C, max residual of the representation)."""
    pts, wts = basis.tet_rule(2 * p + 2)
    N, _ = basis.shape3d(pts, p, eo, fo)
    G = _local_gradients(pts, p, eo)
    M = np.einsum("dip,djp,p->ij", N, N, wts)
    R = np.einsum("dip,dqp,p->iq", N, G, wts)
    C = np.linalg.solve(M, R)
    res = float(np.abs(np.einsum("dip,iq->dqp", N, C) - G).max())
    mx = np.abs(C).max(axis=0, keepdims=True)
    C = np.where(np.abs(C) <= 1e-8 * mx, 0.0, C)
    return C, res


@functools.lru_cache(maxsize=4096)
def local_vector_coefficients(p, eo, fo):
    """C (nd, 12): lambda_v e_k = sum_i C[i, 3 v + k] N_i on the reference
    element (p >= 2), cut like local_coefficients; and the largest residual."""
    pts, wts = basis.tet_rule(2 * p + 2)
    N, _ = basis.shape3d(pts, p, eo, fo)
    x, y, z = pts[:, 0], pts[:, 1], pts[:, 2]
    lam = (1.0 - x - y - z, x, y, z)
    F = np.zeros((3, 12, len(wts)))
    for v in range(4):
        for k in range(3):
            F[k, 3 * v + k] = lam[v]
    M = np.einsum("dip,djp,p->ij", N, N, wts)
    R = np.einsum("dip,dqp,p->iq", N, F, wts)
    C = np.linalg.solve(M, R)
    res = float(np.abs(np.einsum("dip,iq->dqp", N, C) - F).max())
    mx = np.abs(C).max(axis=0, keepdims=True)
    C = np.where(np.abs(C) <= 1e-8 * mx, 0.0, C)
    return C, res


def gradient_map(tets, elemsE, elemsF, eo, fo, dofs, n_dofs, n_nodes, p, pec=None, vector=False, nodes=None):
    """G as scipy CSR (n_dofs x n_cols, float64) and the largest local
    representation residual over the orientation tuples used.  vector=True
    (p >= 2, nodes given) appends the vector P1 columns."""
    tets = np.asarray(tets, dtype=np.int64)
    elemsE = np.asarray(elemsE, dtype=np.int64)
    elemsF = np.asarray(elemsF, dtype=np.int64)
    dofs = np.asarray(dofs, dtype=np.int64)
    T, nd = dofs.shape
    W = n_local(p)
    nE = int(elemsE.max()) + 1
    nF = int(elemsF.max()) + 1
    n_cols = n_nodes + (nE if p >= 2 else 0) + (nE + nF if p == 3 else 0)
    gid = [tets]
    if p >= 2:
        gid.append(n_nodes + elemsE)
    if p == 3:
        gid += [n_nodes + nE + elemsE, n_nodes + 2 * nE + elemsF]
    gid = np.concatenate(gid, axis=1)                     # (T, W)
    keys = [tuple(int(v) for v in eo[e]) + tuple(int(v) for v in fo[e]) for e in range(T)]
    uniq = {}
    tuple_of = np.empty(T, dtype=np.int64)
    for e, k in enumerate(keys):
        tuple_of[e] = uniq.setdefault(k, len(uniq))
    tabs = np.empty((len(uniq), nd, W))
    worst = 0.0
    for k, u in uniq.items():
        C, res = local_coefficients(p, k[:6], k[6:])
        tabs[u] = C
        worst = max(worst, res)
    flat = dofs.reshape(-1)
    rows, first = np.unique(flat, return_index=True)
    el, i = first // nd, first % nd
    vals = tabs[tuple_of[el], i, :]                       # (n_rows, W)
    cols = gid[el, :]
    r = np.repeat(rows, W)
    c = cols.reshape(-1)
    v = vals.reshape(-1)
    if vector:
        if p < 2 or nodes is None:
            raise ValueError("vector columns need p >= 2 and the nodes")
        tv = np.empty((len(uniq), nd, 12))
        for k, u in uniq.items():
            Cv, res = local_vector_coefficients(p, k[:6], k[6:])
            tv[u] = Cv
            worst = max(worst, res)
        X = np.asarray(nodes, dtype=np.float64)[tets[el]]            # (n_rows, 4, 3)
        J = np.transpose(X[:, 1:, :] - X[:, :1, :], (0, 2, 1))       # J[d, k] = x_{k+1,d} - x_{0,d}
        cref = tv[tuple_of[el], i, :].reshape(-1, 4, 3)               # (n_rows, v, k)
        cphys = np.einsum("rvk,rdk->rvd", cref, J).reshape(-1, 12)    # (n_rows, 3 v + d)
        vcols = n_cols + 3 * np.repeat(tets[el], 3, axis=1) + np.tile(np.arange(3), 4)[None, :]
        r = np.concatenate([r, np.repeat(rows, 12)])
        c = np.concatenate([c, vcols.reshape(-1)])
        v = np.concatenate([v, cphys.reshape(-1)])
        n_cols += 3 * n_nodes
    keep = v != 0.0
    G = sp.csr_matrix((v[keep], (r[keep], c[keep])), shape=(n_dofs, n_cols))
    if pec is not None and len(pec):
        touched = np.unique(G[np.asarray(pec, dtype=np.int64)].indices)
        mask = np.ones(n_cols)
        mask[touched] = 0.0
        G = (G @ sp.diags(mask)).tocsr()
        G.eliminate_zeros()
    G.sort_indices()
    return G, worst
