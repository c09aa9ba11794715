"""GMRES with entity block-Jacobi (PETSc -pc_type bjacobi, one block per
edge / face / element; right preconditioning A M^-1, M^-1 = A_aa^-1) against
GMRES with diagonal Jacobi and against COCG: the same solution, the true
residual at rtol, fewer iterations than diagonal Jacobi for p >= 2."""
import pytest
import torch

from tests.helpers import rel_norm

pytestmark = pytest.mark.gpu


def _system(p, n):
    from petgem_gb300 import synthetic
    from petgem_gb300.engine import DeviceMesh
    model = synthetic.config1(n)
    m = DeviceMesh(model.nodes, model.tets, p)
    A = m.assemble(model.sigma, 1.0, pec=True)
    b = torch.zeros((m.N, 2), dtype=torch.complex128, device=m.device)
    for j, x in enumerate((-300.0, 300.0)):
        s = dict(model.source, position=[x, 0.0, 50.0])
        bj = torch.zeros(m.N, dtype=torch.complex128, device=m.device)
        m.source_rhs(s, m.locate_source(s), bj)
        b[:, j] = bj
    m.pec_rhs(b)
    assert bool((torch.linalg.norm(b, dim=0) > 0).all())
    return m, A, b


@pytest.mark.parametrize("p,n,precision", [(1, 5, "fp64"), (2, 4, "fp64"), (2, 4, "mixed"), (3, 3, "fp64")])
def test_gmres_block_jacobi(p, n, precision):
    m, A, b = _system(p, n)
    rtol = 1e-9 if precision == "fp64" else 1e-7
    kw = dict(rtol=rtol, ksp="gmres", precision=precision, max_it=200000, restart=30)
    xb, ib = m.solve(A, b, precond="block", **kw)
    xj, ij = m.solve(A, b, precond="jacobi", **kw)
    assert ib.status == 0 and ij.status == 0
    r = b - m.spmv(A, xb)
    rr = torch.linalg.norm(r, dim=0) / torch.linalg.norm(b, dim=0)
    assert rr.max().item() <= 1.01 * rtol
    assert rel_norm(xb.cpu().numpy(), xj.cpu().numpy()) < 1e3 * rtol
    xc, ic = m.solve(A, b, rtol=1e-10, ksp="cocg", max_it=200000, precond="block")
    assert rel_norm(xb.cpu().numpy(), xc.cpu().numpy()) < 1e3 * rtol
    if p >= 2:
        assert ib.iterations < ij.iterations


def test_gmres_block_counts_must_match():
    """Entity counts that do not add up to the matrix size: PG_ERR_ARG."""
    from petgem_gb300 import _lib
    from petgem_gb300.engine import solve_csr
    m, A, b = _system(2, 3)
    with pytest.raises(_lib.PetgemError) as e:
        solve_csr(m.rowptr, m.col, A, b, ksp="gmres", blocks=(2, m.nE + 1, m.nF, m.T))
    assert e.value.status == -1


@pytest.mark.parametrize("precond", ["jacobi", "block"])
def test_gmres_graph_replay_is_bit_identical(precond, monkeypatch):
    """Restart cycles replayed from a captured CUDA graph give the iterates of
    direct launches, bit for bit (several restarts, 1 and 4 RHS)."""
    from petgem_gb300 import synthetic
    from petgem_gb300.engine import DeviceMesh
    mdl = synthetic.csem_two_layer(4, 2, block=False)
    m = DeviceMesh(mdl.nodes, mdl.tets, 2)
    vals = m.assemble(mdl.sigma, 1.0, pec=True)
    bs = []
    for x0 in (-500.0, 0.0, 250.0, 600.0):
        b, _ = m.source_vector(dict(mdl.source, position=[x0, 20.0, 50.0]))
        m.pec_rhs(b)
        bs.append(b)
    for rhs in (bs[0], torch.stack(bs, 1).contiguous()):
        monkeypatch.setenv("PG_GRAPHS", "1")
        xg, ig = m.solve(vals, rhs, rtol=1e-9, ksp="gmres", restart=10, precond=precond, max_it=5000)
        monkeypatch.setenv("PG_GRAPHS", "0")
        xd, idd = m.solve(vals, rhs, rtol=1e-9, ksp="gmres", restart=10, precond=precond, max_it=5000)
        assert ig.restarts >= 3 and ig.iterations == idd.iterations
        assert torch.equal(xg, xd)
