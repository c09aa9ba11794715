"""Oracle: receiver-misfit gradient with respect to log10 conductivity.

Test infrastructure only (see ``oracle/__init__.py``).  petgem has no
adjoint; this restates the gradient from the reference's own forward model
(elemental matrices petgem/hvfem.py:223-316, assembly solver.py:182-235, PEC
solver.py:552-577, point source solver.py:247-316, receiver interpolation
postprocessing.py:566-614) with a direct solve:

    A(m) u = b,  A = sum_e P_e^T (K_e - i w mu M_e(sigma_e)) P_e, PEC applied
    E = G u (E part of the receiver interpolation),  r = E - d
    phi(m) = sum |r|^2,  m_e = log10 sigma_e (sigma_h, sigma_v scaled together)
    A lambda = G^T conj(r), lambda[PEC] = 0
    dphi/dm_e = 2 Re(lambda_e^T (-i w mu ln10 M_e) u_e)
              = -2 w mu ln10 Im(lambda_e^T M_e u_e)

and central finite differences of phi for the check.
"""
import numpy as np

from . import fem, solve, topology


class Problem:
    """Mesh-derived data of the oracle forward model (computed once)."""

    def __init__(self, nodes, tets, p, source, receivers):
        self.nodes = np.asarray(nodes, dtype=np.float64)
        self.tets = np.asarray(tets, dtype=np.int64)
        self.p = p
        self.source = source
        self.receivers = np.atleast_2d(np.asarray(receivers, dtype=np.float64))
        eE, eN = topology.compute_edges(self.tets)
        eF, fN = topology.compute_faces(self.tets)
        fE = topology.compute_faces_edges(eF, eE, fN.shape[0])
        self.eo, self.fo = topology.element_orientation(self.tets, eE, eN, eF, fE)
        self.dofs, de, df, dv, self.N = topology.compute_connectivity_dofs(eE, eF, p)
        _, bF, _ = topology.compute_boundary_faces(eF, fN)
        bE = topology.compute_boundary_edges(fE, bF)
        _, self.bnd = topology.compute_boundaries(self.dofs, de, df, bE, bF, p)
        self.coords = self.nodes[self.tets]
        # receiver interpolation operator G (3R x N), E part
        el = fem.locate(self.nodes, self.tets, self.receivers)
        self.rx_elem = el
        rows, cols, vals = [], [], []
        for r, e in enumerate(el):
            if e < 0:
                continue
            xi = fem.xyz_to_reference(self.coords[e], self.receivers[r])
            Nb, _ = fem.basis_at(self.coords[e], self.eo[e], self.fo[e], p, xi)
            for c in range(3):
                rows += [3 * r + c] * len(self.dofs[e])
                cols += list(self.dofs[e])
                vals += list(Nb[c, :, 0])
        import scipy.sparse as sp
        self.G = sp.csr_matrix((vals, (rows, cols)), shape=(3 * len(el), self.N))

    def sigma(self, m):
        s = 10.0 ** np.asarray(m, dtype=np.float64)
        return np.stack([s, s], axis=1)

    def forward(self, m):
        """(phi-ready E (R,3) complex, u, A with PEC, M per element)."""
        M, K = fem.element_matrices_batch(self.coords, self.eo, self.fo, self.sigma(m), self.p)
        A = fem.assemble(M, K, self.dofs, self.N, self.source["frequency"])
        b, _ = fem.source_vector(self.nodes, self.tets, self.eo, self.fo, self.dofs, self.N, self.p, self.source)
        A, b = fem.apply_pec(A, b, self.bnd)
        u = solve.direct(A, b)
        E = (self.G @ u).reshape(-1, 3)
        return E, u, A, M


def misfit(prob, m, d_obs):
    E, *_ = prob.forward(m)
    return float(np.sum(np.abs(E - d_obs) ** 2))


def gradient(prob, m, d_obs):
    """Adjoint gradient dphi/dm (T,) and phi."""
    E, u, A, M = prob.forward(m)
    r = E - d_obs
    rhs = prob.G.T @ np.conj(r).reshape(-1)
    rhs[np.asarray(prob.bnd, dtype=np.int64)] = 0.0
    lam = solve.direct(A, rhs)
    w = 2.0 * np.pi * prob.source["frequency"]
    ue = u[prob.dofs]                       # (T, nd)
    le = lam[prob.dofs]
    q = np.einsum("tj,tjk,tk->t", le, M, ue)
    g = -2.0 * w * fem.MU0 * np.log(10.0) * np.imag(q)
    return g, float(np.sum(np.abs(r) ** 2))


def fd_gradient(prob, m, d_obs, elems, h=1e-6):
    """Central finite differences of phi at the given elements."""
    m = np.asarray(m, dtype=np.float64)
    out = np.empty(len(elems))
    for i, e in enumerate(elems):
        mp = m.copy()
        mp[e] += h
        mm = m.copy()
        mm[e] -= h
        out[i] = (misfit(prob, mp, d_obs) - misfit(prob, mm, d_obs)) / (2.0 * h)
    return out
