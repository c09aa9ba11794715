"""Gradient of a receiver misfit with respect to log10 conductivity.

petgem has no adjoint; this is the inversion building block of the GB300
path.  For m_e = log10 sigma_e (horizontal and vertical conductivity scaled
together) and receivers E = G u (the E part of the receiver interpolation,
petgem/postprocessing.py:566-614):

    A(m) u = b                       forward solve (PEC applied)
    phi(m) = sum_r,c |E_rc - d_rc|^2
    A lambda = G^T conj(E - d)       adjoint solve (A is complex symmetric,
                                     so A^T = A; PEC rows of the RHS zeroed)
    dphi/dm_e = 2 ln(10) Im(lambda_e^T (-omega mu M_e) u_e)

The right-hand side G^T conj(E - d) is ``pg_receiver_adjoint`` and the
per-element contraction is ``pg_element_mass_bilinear``; both run in
libpetgem_gb300.so.  ``receiver_misfit`` wraps the pair as a
torch.autograd.Function, so ``phi.backward()`` fills ``m.grad``.
"""
import math

import numpy as np
import torch

from .engine import SolveInfo


class ReceiverMisfit:
    """phi(m) for one DeviceMesh, one point source and fixed receivers / data.

    d_obs: complex [R, 3] observed E at the receivers (rows of receivers that
    fall outside the mesh are ignored, as petgem drops such receivers)."""

    def __init__(self, mesh, source, receivers, d_obs, rtol=1e-10, ksp="cocg", precision="fp64", max_it=100000,
                 precond="block"):
        self.mesh = mesh
        self.source = dict(source)
        self.freq = float(source["frequency"])
        self.receivers = np.atleast_2d(np.asarray(receivers, dtype=np.float64))
        self.d = torch.as_tensor(np.asarray(d_obs, dtype=np.complex128), device=mesh.device).reshape(-1, 3)
        if self.d.shape[0] != self.receivers.shape[0]:
            raise ValueError("d_obs needs one row per receiver")
        self.src_elem = mesh.locate_source(self.source)
        if int(self.src_elem.item()) < 0:
            raise ValueError("source outside the mesh")
        self.opts = dict(rtol=rtol, ksp=ksp, precision=precision, max_it=max_it, precond=precond)
        self.last_info = []

    def _sigma(self, m):
        s = torch.pow(10.0, m.to(torch.float64))
        return torch.stack([s, s], dim=1).contiguous()

    def _solve(self, vals, rhs):
        x, info = self.mesh.solve(vals, rhs, raise_on_fail=True, **self.opts)
        self.last_info.append(info)
        return x

    def evaluate(self, m):
        """phi and the state the gradient needs."""
        mesh = self.mesh
        sigma = self._sigma(m)
        coef = mesh.element_coefficients(sigma, self.freq)
        vals = mesh.assemble(sigma, self.freq, coef=coef, pec=True)
        b = torch.zeros(mesh.N, dtype=torch.complex128, device=mesh.device)
        mesh.source_rhs(self.source, self.src_elem, b)
        mesh.pec_rhs(b)
        u = self._solve(vals, b)
        F, keep = mesh.receiver_fields(u, self.receivers, self.freq)
        r = F[:, :3] - self.d[keep]
        phi = torch.sum(r.real ** 2 + r.imag ** 2)
        return phi, (coef, vals, u, r, keep)

    def gradient(self, state):
        """dphi/dm (float64 [T]) from evaluate()'s state: one adjoint solve."""
        mesh = self.mesh
        coef, vals, u, r, keep = state
        w = torch.zeros((self.receivers.shape[0], 3), dtype=torch.complex128, device=mesh.device)
        w[keep] = torch.conj(r)
        rhs = mesh.receiver_adjoint(w, self.receivers)
        mesh.pec_rhs(rhs)
        lam = self._solve(vals, rhs)
        q = mesh.element_mass_bilinear(coef, u, lam)
        return 2.0 * math.log(10.0) * q.imag

    def value_and_gradient(self, m):
        phi, st = self.evaluate(m)
        return phi, self.gradient(st)


class _MisfitFunction(torch.autograd.Function):
    @staticmethod
    def forward(ctx, m, problem):
        phi, state = problem.evaluate(m.detach())
        ctx.problem = problem
        ctx.state = state
        return phi

    @staticmethod
    def backward(ctx, grad_phi):
        g = ctx.problem.gradient(ctx.state)
        ctx.state = None
        return grad_phi * g, None


def receiver_misfit(m, problem):
    """phi(m) as a differentiable torch scalar; m float64 [T] on the mesh's device."""
    return _MisfitFunction.apply(m, problem)


__all__ = ["ReceiverMisfit", "receiver_misfit", "SolveInfo"]
