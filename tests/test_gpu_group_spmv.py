"""Double-float products of the COCG: every lanes-per-row / unrolling variant
and the entity-group products (rows [R i, R i + R) of one mesh entity share
their columns, R = p; one column step at a time, unrolled, or 4 steps'
loads batched) reach the same solution, and the monitor shows the forced
variant ran."""
import numpy as np
import pytest
import torch

from tests.helpers import rel_norm

pytestmark = pytest.mark.gpu


def _system(p, k):
    from petgem_gb300 import synthetic
    from petgem_gb300.engine import DeviceMesh
    model = synthetic.config1(5 if p == 2 else 4)
    m = DeviceMesh(model.nodes, model.tets, p)
    A = m.assemble(model.sigma, 1.0, pec=True)
    b = torch.zeros((m.N, k), dtype=torch.complex128, device=m.device)
    for j, x in enumerate(np.linspace(-800.0, 800.0, k) if k > 1 else [0.0]):
        s = dict(model.source, position=[float(x), 0.0, 50.0])
        bj = torch.zeros(m.N, dtype=torch.complex128, device=m.device)
        m.source_rhs(s, m.locate_source(s), bj)
        b[:, j] = bj
    m.pec_rhs(b)
    assert bool((torch.linalg.norm(b, dim=0) > 0).all())
    return m, A, (b[:, 0].contiguous() if k == 1 else b)


@pytest.mark.parametrize("p,k,variant", [(2, 1, 202), (2, 1, 204), (2, 1, 208), (2, 1, 212), (2, 1, 214),
                                         (2, 1, 232), (2, 1, 234), (2, 1, 42), (3, 1, 304), (3, 1, 314),
                                         (3, 1, 302), (3, 1, 332), (3, 1, 334), (2, 4, 200), (2, 4, 2),
                                         (3, 8, 300), (2, 4, 250), (2, 16, 250), (3, 8, 350)])
def test_df64_product_variants_agree(p, k, variant, monkeypatch, capfd):
    m, A, b = _system(p, k)
    rtol = 1e-10
    monkeypatch.setenv("PG_KSP_MONITOR", "1")
    monkeypatch.setenv("PG_SPMV_VARIANT", str(variant))
    x, info = m.solve(A, b, rtol=rtol, ksp="cocg", precision="df64", max_it=100000, precond="block")
    err = capfd.readouterr().err
    assert f"SpMV variant {variant} " in err
    assert info.status == 0
    r = b - m.spmv(A, x)
    rr = torch.linalg.norm(r, dim=0) / torch.linalg.norm(b, dim=0)
    assert rr.max().item() <= 1.01 * rtol
    monkeypatch.setenv("PG_SPMV_VARIANT", "41" if k == 1 else "1")
    x0, i0 = m.solve(A, b, rtol=rtol, ksp="cocg", precision="df64", max_it=100000, precond="block")
    assert rel_norm(x.cpu().numpy(), x0.cpu().numpy()) < 1e3 * rtol
    assert abs(info.iterations - i0.iterations) <= 0.05 * i0.iterations + 10


def test_group_variant_needs_checked_groups(monkeypatch, capfd):
    """With diagonal Jacobi the rows are not known to group: a forced group
    variant is ignored."""
    m, A, b = _system(2, 1)
    monkeypatch.setenv("PG_KSP_MONITOR", "1")
    monkeypatch.setenv("PG_SPMV_VARIANT", "204")
    x, info = m.solve(A, b, rtol=1e-9, ksp="cocg", precision="df64", max_it=100000, precond="jacobi")
    err = capfd.readouterr().err
    assert info.status == 0
    assert "SpMV variant 204 " not in err and "SpMV variant " in err
