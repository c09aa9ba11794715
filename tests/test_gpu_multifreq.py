"""Several frequencies x several sources in one double-float COCG (one matrix
read per iteration for every column) against one FP64 solve per frequency;
CUDA-graph replay of the iterations against direct launches."""
import numpy as np
import pytest
import torch

from tests.helpers import rel_norm

pytestmark = pytest.mark.gpu


def test_multifrequency_solve_matches_per_frequency_solves():
    from petgem_gb300 import synthetic
    from petgem_gb300.engine import DeviceMesh
    model = synthetic.config1(6)
    m = DeviceMesh(model.nodes, model.tets, 2)
    freqs = [0.25, 0.5, 1.0, 2.0]
    srcs = [dict(model.source), dict(model.source, position=[200.0, -100.0, 50.0])]
    f0 = 1.0
    A0 = m.assemble(model.sigma, f0, pec=True)
    cols, fcol = [], []
    for f in freqs:
        for s in srcs:
            s = dict(s, frequency=f)
            b = torch.zeros(m.N, dtype=torch.complex128, device=m.device)
            m.source_rhs(s, m.locate_source(s), b)
            m.pec_rhs(b)
            cols.append(b)
            fcol.append(f)
    B = torch.stack(cols, 1).contiguous()
    X, info = m.solve_frequencies(A0, f0, B, fcol, rtol=1e-10)
    assert info.status == 0 and max(info.relres_per_rhs) <= 1e-10
    for j, f in enumerate(fcol):
        Af = m.assemble(model.sigma, f, pec=True)
        xj, ij = m.solve(Af, B[:, j].contiguous(), rtol=1e-11, ksp="cocg", max_it=100000)
        assert rel_norm(X[:, j].cpu().numpy(), xj.cpu().numpy()) < 1e-8
        # the true residual of the multi-frequency column against its own operator
        r = B[:, j] - m.spmv(Af, X[:, j].contiguous())
        assert (torch.linalg.norm(r) / torch.linalg.norm(B[:, j])).item() <= 1.01e-10


def test_graph_replay_matches_direct_launches(monkeypatch):
    """The double-float COCG replays its iterations from a captured CUDA graph;
    the result is bit-identical to launching every kernel directly."""
    from petgem_gb300 import synthetic
    from petgem_gb300.engine import DeviceMesh
    model = synthetic.config1(6)
    m = DeviceMesh(model.nodes, model.tets, 2)
    A = m.assemble(model.sigma, 1.0, pec=True)
    b = torch.zeros((m.N, 2), dtype=torch.complex128, device=m.device)
    for j, x in enumerate((0.0, 300.0)):
        s = dict(model.source, position=[x, 0.0, 50.0])
        bj = torch.zeros(m.N, dtype=torch.complex128, device=m.device)
        m.source_rhs(s, m.locate_source(s), bj)
        b[:, j] = bj
    m.pec_rhs(b)
    out = {}
    for g in ("1", "0"):
        monkeypatch.setenv("PG_GRAPHS", g)
        x, info = m.solve(A, b, rtol=1e-10, ksp="cocg", precision="df64", check_every=64)
        assert info.status == 0
        out[g] = (x, info.iterations)
    assert out["1"][1] == out["0"][1]
    assert torch.equal(out["1"][0], out["0"][0])


@pytest.mark.parametrize("p,precision", [(1, "fp64"), (2, "fp64"), (2, "df64"), (2, "mixed"), (3, "df64")])
def test_block_jacobi_matches_diagonal_jacobi(p, precision):
    """Entity block-Jacobi COCG (S A S^T with S = D^-1/2 L^-1 per entity block)
    reaches the same solution as diagonal Jacobi, in fewer iterations for p >= 2."""
    from petgem_gb300 import synthetic
    from petgem_gb300.engine import DeviceMesh
    model = synthetic.config1(5 if p < 3 else 4)
    m = DeviceMesh(model.nodes, model.tets, p)
    A = m.assemble(model.sigma, 1.0, pec=True)
    b = torch.zeros(m.N, dtype=torch.complex128, device=m.device)
    m.source_rhs(model.source, m.locate_source(model.source), b)
    m.pec_rhs(b)
    rtol = 1e-10 if precision != "mixed" else 1e-7
    xb, ib = m.solve(A, b, rtol=rtol, ksp="cocg", precision=precision, max_it=100000, precond="block")
    xj, ij = m.solve(A, b, rtol=rtol, ksp="cocg", precision=precision, max_it=100000, precond="jacobi")
    assert ib.status == 0 and ij.status == 0
    r = b - m.spmv(A, xb)
    assert (torch.linalg.norm(r) / torch.linalg.norm(b)).item() <= 1.01 * rtol
    assert rel_norm(xb.cpu().numpy(), xj.cpu().numpy()) < 1e3 * rtol
    if p >= 2 and precision != "mixed":
        assert ib.iterations < ij.iterations
