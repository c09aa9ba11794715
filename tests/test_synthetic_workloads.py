"""The seeded synthetic workloads (no GPU): Kuhn-split boxes with every tet
positively oriented (petgem scales M and K by the signed det(J)), the counts
of the metric's meshes, and each workload's seeded parameters."""
import numpy as np

from petgem_gb300 import synthetic


def test_kuhn_counts_and_orientation():
    for n in (2, 5):
        nodes, tets = synthetic.kuhn_box(n)
        assert nodes.shape == ((n + 1) ** 3, 3) and tets.shape == (6 * n ** 3, 4)
        assert np.all(synthetic.signed_volumes(nodes, tets) > 0)
        # the tets fill the box exactly
        assert abs(synthetic.signed_volumes(nodes, tets).sum() / 2000.0 ** 3 - 1.0) < 1e-12


def test_config1_jitter_keeps_orientation_and_boundary():
    m = synthetic.config1(6)
    assert np.all(synthetic.signed_volumes(m.nodes, m.tets) > 0)
    on_box = np.any(np.isclose(np.abs(m.nodes), 1000.0), axis=1)
    plain, _ = synthetic.kuhn_box(6)
    assert np.array_equal(m.nodes[on_box], plain[on_box])          # boundary nodes stay on the box
    assert not np.array_equal(m.nodes[~on_box], plain[~on_box])    # interior nodes move
    assert m.sigma.min() >= 0.01 - 1e-12 and m.sigma.max() <= 3.3 + 1e-12
    assert m.receivers.shape == (100, 3)
    assert np.array_equal(m.sigma, synthetic.config1(6).sigma)     # seeded


def test_config3_log_conductivity():
    m = synthetic.config3(4)
    assert m.m.shape == (m.tets.shape[0],)
    assert m.m.min() >= -2.0 and m.m.max() <= 0.5
    assert np.allclose(m.sigma[:, 0], 10.0 ** m.m) and np.array_equal(m.sigma[:, 0], m.sigma[:, 1])
    assert np.array_equal(m.m, synthetic.config3(4).m)


def test_config2_sources_and_extra_meshes():
    m = synthetic.config2(4)
    assert m.frequencies == [0.25, 0.5, 1.0, 2.0] and len(m.sources) == 64
    for n in synthetic.config2_extra_sizes()[:2]:
        e = synthetic.config2_extra(n)
        assert e.tets.shape[0] == 6 * n ** 3
        assert set(np.unique(e.sigma)) <= {1.0, 3.3}
