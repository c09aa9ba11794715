"""Oracle receiver-misfit gradient against its committed golden vectors and
against central finite differences of the oracle forward model (CPU)."""
import json

import numpy as np

from oracle import adjoint
from tests.helpers import load, rel_norm


def _problem(g):
    return adjoint.Problem(g["nodes"], g["tets"], int(g["p"]), json.loads(str(g["src"])), g["receivers"])


def test_oracle_adjoint_matches_golden_and_finite_differences():
    g = load("adjoint_n4.npz")
    prob = _problem(g)
    grad, phi = adjoint.gradient(prob, g["m0"], g["d_obs"])
    assert abs(phi - float(g["phi"])) <= 1e-10 * float(g["phi"])
    assert rel_norm(grad, g["grad"]) < 1e-9
    el = g["fd_elems"]
    assert rel_norm(grad[el], g["fd_grad"]) < 1e-6


def test_oracle_finite_differences_converge():
    """Central differences at h and h/10 approach the adjoint gradient O(h^2)."""
    g = load("adjoint_n4.npz")
    prob = _problem(g)
    el = g["fd_elems"][:2]
    e3 = rel_norm(adjoint.fd_gradient(prob, g["m0"], g["d_obs"], el, h=1e-3), g["grad"][el])
    e4 = rel_norm(adjoint.fd_gradient(prob, g["m0"], g["d_obs"], el, h=1e-4), g["grad"][el])
    assert e4 < e3 / 30.0
