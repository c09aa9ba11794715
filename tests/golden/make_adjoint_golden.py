"""Golden vectors for the receiver-misfit gradient (adjoint) tests.

petgem has no adjoint, so the reference point is its forward model: the
oracle's forward model (pinned to petgem's own assembled A and source b by
make_golden.py) solved directly, differentiated by central finite
differences.  Writes adjoint_n4.npz:

* a 4^3 Kuhn box, interior nodes jittered (seed 0), p = 2;
* m = log10 sigma ~ U[-2, 0.5] per element (seed 3); data d = E(m) with 10 %
  complex Gaussian noise relative to each component (seed 4); the gradient
  is taken at m0 = m + 0.05 N(0, 1) (seed 6);
* 25 receivers on z = 0, x-HED at (0, 0, 50) m, 1 Hz;
* the oracle adjoint gradient for every element and central differences
  (h = 1e-5) at the 6 largest-gradient and 6 random elements.

Run from the repository root:  python tests/golden/make_adjoint_golden.py
"""
import json
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

from oracle import adjoint  # noqa: E402
from petgem_gb300 import synthetic  # noqa: E402


def main():
    n, p = 4, 2
    lo, hi = (-1000.0,) * 3, (1000.0,) * 3
    nodes, tets = synthetic.kuhn_box(n, lo, hi)
    nodes = synthetic.jitter_interior(nodes, n, 0.15, 0, lo, hi)
    m = np.random.default_rng(3).uniform(-2.0, 0.5, len(tets))
    g = np.linspace(-800.0, 800.0, 5)
    X, Y = np.meshgrid(g, g, indexing="ij")
    rx = np.stack([X.ravel(), Y.ravel(), np.zeros(25)], axis=1)
    src = {"frequency": 1.0, "position": [0.0, 0.0, 50.0], "azimuth": 0.0, "dip": 0.0, "current": 1.0,
           "length": 1.0}
    prob = adjoint.Problem(nodes, tets, p, src, rx)
    E, *_ = prob.forward(m)
    rng = np.random.default_rng(4)
    d = E * (1.0 + 0.1 * (rng.standard_normal(E.shape) + 1j * rng.standard_normal(E.shape)))
    m0 = m + 0.05 * np.random.default_rng(6).standard_normal(len(m))
    grad, phi = adjoint.gradient(prob, m0, d)
    top = np.argsort(-np.abs(grad))[:6]
    rest = np.setdiff1d(np.arange(len(tets)), top)
    elems = np.concatenate([top, np.random.default_rng(7).choice(rest, 6, replace=False)])
    fd = adjoint.fd_gradient(prob, m0, d, elems, h=1e-5)
    out = os.path.join(os.path.dirname(os.path.abspath(__file__)), "adjoint_n4.npz")
    np.savez_compressed(out, nodes=nodes, tets=tets, p=p, m0=m0, d_obs=d, receivers=rx, src=json.dumps(src),
                        grad=grad, phi=phi, fd_elems=elems, fd_grad=fd, fd_h=1e-5)
    print("wrote", out, "phi", phi, "fd vs adjoint", np.linalg.norm(grad[elems] - fd) / np.linalg.norm(fd))


if __name__ == "__main__":
    main()
