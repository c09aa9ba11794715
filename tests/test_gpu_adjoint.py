"""GPU receiver-misfit gradient (adjoint solve + per-element contraction)
against the oracle's adjoint and central finite differences of the oracle
forward model (golden), against GPU finite differences, and the transpose /
bilinear-form identities of its two kernels."""
import json

import numpy as np
import pytest
import torch

from oracle import adjoint as oadj
from oracle import fem
from tests.helpers import load, rel_norm

pytestmark = pytest.mark.gpu

GRAD_TOL = 1e-6     # normwise, against the oracle gradient and golden central differences


def _setup(rtol=1e-12):
    from petgem_gb300.adjoint import ReceiverMisfit
    from petgem_gb300.engine import DeviceMesh
    g = load("adjoint_n4.npz")
    mesh = DeviceMesh(g["nodes"], g["tets"], int(g["p"]))
    prob = ReceiverMisfit(mesh, json.loads(str(g["src"])), g["receivers"], g["d_obs"], rtol=rtol)
    return g, mesh, prob


def test_gradient_vs_oracle_and_finite_differences():
    from petgem_gb300.adjoint import receiver_misfit
    g, mesh, prob = _setup()
    m = torch.tensor(g["m0"], dtype=torch.float64, device=mesh.device, requires_grad=True)
    phi = receiver_misfit(m, prob)
    phi.backward()
    assert abs(phi.item() - float(g["phi"])) <= 1e-8 * float(g["phi"])
    grad = m.grad.cpu().numpy()
    assert rel_norm(grad, g["grad"]) < GRAD_TOL
    assert rel_norm(grad[g["fd_elems"]], g["fd_grad"]) < GRAD_TOL
    assert all(i.status == 0 for i in prob.last_info)


def test_gradient_vs_gpu_finite_differences():
    g, mesh, prob = _setup()
    m0 = torch.tensor(g["m0"], dtype=torch.float64, device=mesh.device)
    _, grad = prob.value_and_gradient(m0)
    h = 1e-4
    for e in g["fd_elems"][:3]:
        mp, mm = m0.clone(), m0.clone()
        mp[e] += h
        mm[e] -= h
        fd = (prob.evaluate(mp)[0] - prob.evaluate(mm)[0]).item() / (2 * h)
        assert abs(fd - grad[e].item()) <= 1e-5 * abs(grad).max().item()


def test_directional_derivative_over_all_elements():
    """grad . v against central differences of phi along a seeded random
    direction v that moves every element at once (a check whose size does
    not depend on which elements happen to be picked)."""
    g, mesh, prob = _setup(rtol=1e-12)
    m0 = torch.tensor(g["m0"], dtype=torch.float64, device=mesh.device)
    _, grad = prob.value_and_gradient(m0)
    v = torch.as_tensor(np.random.default_rng(8).standard_normal(mesh.T), device=mesh.device)
    dphi = float(torch.dot(grad, v))
    for h in (1e-4, 1e-5):
        fd = (prob.evaluate(m0 + h * v)[0] - prob.evaluate(m0 - h * v)[0]).item() / (2 * h)
        assert abs(fd - dphi) <= 1e-5 * abs(dphi), (h, fd, dphi)


def test_receiver_adjoint_is_the_transpose_of_the_gather():
    g, mesh, prob = _setup()
    rng = np.random.default_rng(11)
    x = torch.as_tensor(rng.standard_normal(mesh.N) + 1j * rng.standard_normal(mesh.N), device=mesh.device)
    R = g["receivers"].shape[0]
    w = torch.as_tensor(rng.standard_normal((R, 3)) + 1j * rng.standard_normal((R, 3)), device=mesh.device)
    F, keep = mesh.receiver_fields(x, g["receivers"], 1.0)
    lhs = torch.sum(F[:, :3] * w[keep])                # w^T (G x)
    gt = mesh.receiver_adjoint(w, g["receivers"])
    rhs = torch.sum(gt * x)                             # (G^T w)^T x
    assert abs((lhs - rhs).item()) <= 1e-12 * abs(lhs.item())


def test_element_mass_bilinear_vs_oracle_matrices():
    g, mesh, prob = _setup()
    rng = np.random.default_rng(12)
    T = mesh.T
    s = 10.0 ** rng.uniform(-2, 0.5, T)
    sigma = np.stack([s, s * rng.uniform(0.3, 1.0, T)], 1)
    f = 2.5
    coef = mesh.element_coefficients(sigma, f)
    x = rng.standard_normal(mesh.N) + 1j * rng.standard_normal(mesh.N)
    y = rng.standard_normal(mesh.N) + 1j * rng.standard_normal(mesh.N)
    out = mesh.element_mass_bilinear(coef, torch.as_tensor(x, device=mesh.device),
                                      torch.as_tensor(y, device=mesh.device)).cpu().numpy()
    prob_o = oadj.Problem(g["nodes"], g["tets"], int(g["p"]), json.loads(str(g["src"])), g["receivers"])
    M, _ = fem.element_matrices_batch(prob_o.coords, prob_o.eo, prob_o.fo, sigma, int(g["p"]))
    dofs = prob_o.dofs
    ref = -2 * np.pi * f * fem.MU0 * np.einsum("tj,tjk,tk->t", y[dofs], M, x[dofs])
    assert rel_norm(out, ref) < 1e-12
