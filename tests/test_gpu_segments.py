"""Several meshes of different sizes in one double-float COCG
(pg_cocg_segments).  Every system keeps its own scalars and convergence test,
so each solution is the one its own solve reaches; every launch serves all
systems."""
import numpy as np
import pytest
import torch

from tests.helpers import rel_norm

pytestmark = pytest.mark.gpu


def _system(n, seed, k=1, p=2):
    from petgem_gb300 import synthetic
    from petgem_gb300.engine import DeviceMesh
    model = synthetic.config1(n)
    rng = np.random.default_rng(seed)
    sigma = model.sigma * 10.0 ** rng.uniform(-0.3, 0.3, (len(model.sigma), 1))
    m = DeviceMesh(model.nodes, model.tets, p)
    A = m.assemble(sigma, 1.0, pec=True)
    b = torch.zeros((m.N, k), dtype=torch.complex128, device=m.device)
    for j in range(k):
        s = dict(model.source, position=[-300.0 + 200.0 * j, 50.0 * seed, 50.0])
        bj = torch.zeros(m.N, dtype=torch.complex128, device=m.device)
        m.source_rhs(s, m.locate_source(s), bj)
        b[:, j] = bj
    m.pec_rhs(b)
    assert bool((torch.linalg.norm(b, dim=0) > 0).all())
    return m, A, (b[:, 0].contiguous() if k == 1 else b)


def _true_relres(m, A, x, b):
    r = b - m.spmv(A, x)
    if b.ndim == 1:
        return [(torch.linalg.norm(r) / torch.linalg.norm(b)).item()]
    return (torch.linalg.norm(r, dim=0) / torch.linalg.norm(b, dim=0)).tolist()


@pytest.mark.parametrize("k,precond", [(1, "jacobi"), (1, "block"), (4, "block"), (1, "grad"), (4, "grad")])
def test_segments_match_separate_solves(k, precond):
    from petgem_gb300.engine import solve_csr_segments
    sizes = [5, 3, 4]
    systems = [_system(n, seed=j + 1, k=k) for j, n in enumerate(sizes)]
    rtol = 1e-10
    blocks = (2, [(m.nE, m.nF, m.T) for m, _, _ in systems]) if precond == "block" else None
    grads = [m.gradient_map() for m, _, _ in systems] if precond == "grad" else None
    xs, info = solve_csr_segments([(m.rowptr, m.col, A, b) for m, A, b in systems], blocks=blocks, rtol=rtol,
                                  gradients=grads)
    assert info.status == 0
    assert len(info.relres_per_rhs) == len(sizes) and all(len(r) == k for r in info.relres_per_rhs)
    for j, (m, A, b) in enumerate(systems):
        x = xs[j] if k > 1 else xs[j].reshape(-1)
        # each system's own true residual, against its own operator
        rr = _true_relres(m, A, x, b)
        assert max(rr) <= 1.01 * rtol
        assert max(info.relres_per_rhs[j]) <= rtol
        xo, io = m.solve(A, b, rtol=rtol, ksp="cocg", precision="df64", max_it=100000, precond=precond)
        assert rel_norm(x.cpu().numpy(), xo.cpu().numpy()) < 1e3 * rtol
        # the iteration count of each system is its own, close to its separate solve's
        its = max(info.its_per_rhs[j])
        assert abs(its - io.iterations) <= 0.25 * io.iterations + 20, (j, its, io.iterations)
    assert info.iterations == max(max(v) for v in info.its_per_rhs)


def test_segments_column_outside_its_system_is_rejected():
    """A row that references another system's column breaks the
    block-diagonal layout: PG_ERR_ARG before any iteration."""
    from petgem_gb300 import _lib
    from petgem_gb300.engine import concat_systems, solve_csr_segments
    systems = [_system(3, seed=1), _system(3, seed=2)]
    sys_list = [(m.rowptr, m.col, A, b) for m, A, b in systems]
    rowptr, col, vals, b, rows = concat_systems(sys_list)
    assert rows.tolist() == [0, systems[0][0].N, systems[0][0].N + systems[1][0].N]
    bad = col.clone()
    bad[0] = int(rows[1])          # row 0 of system 0 -> a column of system 1 (still < n)
    m0 = systems[0][0]
    with pytest.raises(_lib.PetgemError) as e:
        solve_csr_segments([(m0.rowptr, bad[:m0.nnz], systems[0][1], systems[0][2]), sys_list[1]])
    assert e.value.status == -1


def test_segments_converged_system_stays_put():
    """A system whose b is zero is converged from the start (x = 0) while the
    others iterate."""
    from petgem_gb300.engine import solve_csr_segments
    m1, A1, b1 = _system(4, seed=1)
    m2, A2, b2 = _system(3, seed=2)
    z = torch.zeros_like(b2)
    xs, info = solve_csr_segments([(m1.rowptr, m1.col, A1, b1), (m2.rowptr, m2.col, A2, z)], rtol=1e-9)
    assert info.status == 0
    assert torch.count_nonzero(xs[1]).item() == 0
    assert info.its_per_rhs[1][0] == 0
    assert _true_relres(m1, A1, xs[0], b1)[0] <= 1.01e-9


@pytest.mark.parametrize("k,variant", [(1, 42), (1, 41), (1, 22), (1, 82), (1, 232), (1, 234), (4, 2), (4, 1),
                                       (4, 200)])
def test_segments_product_variants_agree(k, variant, monkeypatch, capfd):
    """Every product shape of the several-systems solve (rows, entity groups
    with batched loads, several RHS) reaches the same solutions; the monitor
    shows the forced shape ran."""
    from petgem_gb300.engine import solve_csr_segments
    systems = [_system(n, seed=j + 1, k=k) for j, n in enumerate((4, 3))]
    blocks = (2, [(m.nE, m.nF, m.T) for m, _, _ in systems])
    sysl = [(m.rowptr, m.col, A, b) for m, A, b in systems]
    monkeypatch.setenv("PG_KSP_MONITOR", "1")
    monkeypatch.setenv("PG_SPMV_VARIANT", str(variant))
    xs, info = solve_csr_segments(sysl, blocks=blocks, rtol=1e-10)
    assert f"SpMV variant {variant} " in capfd.readouterr().err
    monkeypatch.setenv("PG_SPMV_VARIANT", "42" if k == 1 else "2")
    x0, i0 = solve_csr_segments(sysl, blocks=blocks, rtol=1e-10)
    assert info.status == 0 and i0.status == 0
    for j, (m, A, b) in enumerate(systems):
        x = xs[j] if k > 1 else xs[j].reshape(-1)
        assert max(_true_relres(m, A, x, b)) <= 1.01e-10
        assert rel_norm(xs[j].cpu().numpy(), x0[j].cpu().numpy()) < 1e-7
