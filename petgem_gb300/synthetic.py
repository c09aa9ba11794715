"""Seeded synthetic meshes and models for the benchmark workloads.

No public dataset is involved: every workload is a box split into n^3 cubes,
each cube into 6 Kuhn tetrahedra, with analytic or seeded conductivities.
All tetrahedra are generated with positive orientation, because petgem
scales M and K by the signed det(J) (petgem/hvfem.py:265,313-314).
"""
import itertools

import numpy as np


def kuhn_box(n, lo=(-1000.0, -1000.0, -1000.0), hi=(1000.0, 1000.0, 1000.0)):
    """Nodes (x fastest) and positively oriented Kuhn tets, cube by cube."""
    lo = np.asarray(lo, dtype=np.float64)
    hi = np.asarray(hi, dtype=np.float64)
    ax = [np.linspace(lo[d], hi[d], n + 1) for d in range(3)]
    Z, Y, X = np.meshgrid(ax[2], ax[1], ax[0], indexing="ij")
    nodes = np.stack([X.ravel(), Y.ravel(), Z.ravel()], axis=1)
    k, j, i = [a.ravel() for a in np.meshgrid(np.arange(n), np.arange(n), np.arange(n), indexing="ij")]

    def vid(di, dj, dk):
        return (i + di) + (n + 1) * ((j + dj) + (n + 1) * (k + dk))

    tets = []
    for perm in itertools.permutations(range(3)):
        step = np.zeros(3, dtype=np.int64)
        corner = [vid(0, 0, 0)]
        for a in perm[:2]:
            step[a] = 1
            corner.append(vid(*step))
        corner.append(vid(1, 1, 1))
        inv = sum(1 for x in range(3) for y in range(x + 1, 3) if perm[x] > perm[y])
        if inv % 2:                      # odd permutation -> negative volume
            corner[1], corner[2] = corner[2], corner[1]
        tets.append(np.stack(corner, axis=1))
    tets = np.stack(tets, axis=1).reshape(-1, 4)     # cube-major: 6 tets per cube
    return nodes, tets.astype(np.int64)


def signed_volumes(nodes, tets):
    c = nodes[tets]
    return np.linalg.det(c[:, 1:] - c[:, :1]) / 6.0


def jitter_interior(nodes, n, frac, seed, lo, hi):
    """Move interior nodes by U(-frac*h, frac*h) per axis; boundary nodes fixed."""
    lo = np.asarray(lo, dtype=np.float64)
    hi = np.asarray(hi, dtype=np.float64)
    h = (hi - lo) / n
    rng = np.random.default_rng(seed)
    d = rng.uniform(-1.0, 1.0, size=nodes.shape) * frac * h
    eps = 1e-9 * h
    interior = np.all((nodes > lo + eps) & (nodes < hi - eps), axis=1)
    out = nodes.copy()
    out[interior] += d[interior]
    return out


class Model:
    """A forward-modelling workload: mesh, conductivity, source, receivers."""

    def __init__(self, name, nodes, tets, sigma, p, source, receivers, physical=None):
        self.name = name
        self.nodes = nodes
        self.tets = tets
        self.sigma = sigma            # (T, 2) horizontal, vertical
        self.p = p
        self.source = source          # dict: frequency, position, azimuth, dip, current, length
        self.receivers = receivers    # (R, 3)
        self.physical = physical


def _hed(x=0.0, y=0.0, z=50.0, f=1.0):
    return {"frequency": f, "position": [x, y, z], "azimuth": 0.0, "dip": 0.0, "current": 1.0, "length": 1.0}


def csem_two_layer(n, p, block=True, f=1.0):
    """Seawater 3.3 S/m above z=0, sediment 1.0 S/m below, optional 0.01 S/m
    400x400x100 m block centred at (0,0,-300); x-HED at (0,0,50); 20
    receivers on z=0, x in [-800, 800]."""
    nodes, tets = kuhn_box(n)
    cen = nodes[tets].mean(axis=1)
    s = np.where(cen[:, 2] > 0.0, 3.3, 1.0)
    if block:
        blk = (np.abs(cen[:, 0]) <= 200.0) & (np.abs(cen[:, 1]) <= 200.0) & (cen[:, 2] >= -350.0) & (cen[:, 2] <= -250.0)
        s[blk] = 0.01
    sigma = np.stack([s, s], axis=1)
    rx = np.stack([np.linspace(-800.0, 800.0, 20), np.zeros(20), np.zeros(20)], axis=1)
    return Model(f"csem_two_layer_n{n}_p{p}", nodes, tets, sigma, p, _hed(f=f), rx)


def config0():
    """Plain FP64 CSEM, p=1, 16^3 cubes x 6 tets (24,576 tets)."""
    m = csem_two_layer(16, 1, block=True)
    m.name = "csem_p1_16cubed"
    return m


def config1(n=32):
    """Mixed-precision CSEM, p=2, 32^3 cubes x 6 tets (196,608 tets); interior
    nodes jittered by U(+-0.15h) (seed 0); per-element sigma log-uniform in
    [0.01, 3.3] S/m (seed 1); HED at (0,0,50) 1 Hz; 10x10 receivers on z=0
    spanning [-800, 800]^2."""
    lo, hi = (-1000.0,) * 3, (1000.0,) * 3
    nodes, tets = kuhn_box(n, lo, hi)
    nodes = jitter_interior(nodes, n, 0.15, 0, lo, hi)
    rng = np.random.default_rng(1)
    s = 10.0 ** rng.uniform(np.log10(0.01), np.log10(3.3), size=len(tets))
    sigma = np.stack([s, s], axis=1)
    g = np.linspace(-800.0, 800.0, 10)
    X, Y = np.meshgrid(g, g, indexing="ij")
    rx = np.stack([X.ravel(), Y.ravel(), np.zeros(100)], axis=1)
    return Model(f"csem_p2_{n}cubed_jitter", nodes, tets, sigma, 2, _hed(), rx)


def config2_sources(count=64, x_max=800.0):
    """`count` x-directed HEDs at z = 50 m, x evenly spaced in [-x_max, x_max].
    The batched workload's nominal line, x in [-1600, 1600], runs past the
    [-1000, 1000] m box, where a source cannot be located (petgem raises); the
    line is therefore kept inside the box, over the receivers' span."""
    return [_hed(x=float(x)) for x in np.linspace(-x_max, x_max, count)]


def config2(n=24):
    """Batched CSEM, p=2, n^3 cubes over [-1000, 1000]^3: two-layer model
    (3.3 S/m above z=0, 1.0 S/m below); 64 x-HEDs at z = 50 m (config2_sources)
    at 0.25, 0.5, 1 and 2 Hz; the receivers of config0 (20 on z=0)."""
    m = csem_two_layer(n, 2, block=False)
    m.name = f"csem_p2_{n}cubed_batched"
    m.frequencies = [0.25, 0.5, 1.0, 2.0]
    m.sources = config2_sources()
    return m


def config2_extra_sizes(count=8, lo=8, hi=20, seed=2):
    """Cubes per axis of the batched workload's extra independent meshes:
    `count` sizes drawn uniformly from lo..hi (seed 2)."""
    rng = np.random.default_rng(seed)
    return [int(v) for v in rng.integers(lo, hi + 1, size=count)]


def config2_extra(n):
    """One extra mesh of the batched workload: the two-layer model of config2
    on n^3 cubes."""
    m = csem_two_layer(n, 2, block=False)
    m.name = f"csem_p2_{n}cubed_extra"
    return m


def config3(n=24):
    """Adjoint gradient workload, p=2: n^3 cubes x 6 tets over [-1000, 1000]^3;
    per-element m_e = log10 sigma_e ~ U[-2, 0.5] (seed 3), sigma_h = sigma_v;
    HED at (0,0,50) 1 Hz; 10x10 receivers on z=0 spanning [-800, 800]^2.
    The model's `m` holds the log-conductivities."""
    nodes, tets = kuhn_box(n)
    m = np.random.default_rng(3).uniform(-2.0, 0.5, len(tets))
    s = 10.0 ** m
    g = np.linspace(-800.0, 800.0, 10)
    X, Y = np.meshgrid(g, g, indexing="ij")
    rx = np.stack([X.ravel(), Y.ravel(), np.zeros(100)], axis=1)
    model = Model(f"adjoint_p2_{n}cubed", nodes, tets, np.stack([s, s], axis=1), 2, _hed(), rx)
    model.m = m
    return model


def config4(n=40, seed=5):
    """MT, p=3, n^3 cubes over [-5000, 5000]^2 x [-5000, 2000] m: air 1e-8 S/m
    above z=0, 0.1 S/m for -1000 <= z <= 0, 0.01 S/m below, and three
    ellipsoids (centres and semi-axes 200-800 m, conductivity log-uniform in
    [0.001, 1] S/m, seeded); 2 polarisations at 0.1 and 1 Hz; 20 x 20
    receivers on the surface."""
    lo, hi = (-5000.0, -5000.0, -5000.0), (5000.0, 5000.0, 2000.0)
    nodes, tets = kuhn_box(n, lo, hi)
    cen = nodes[tets].mean(axis=1)
    s = np.where(cen[:, 2] > 0.0, 1e-8, np.where(cen[:, 2] >= -1000.0, 0.1, 0.01))
    rng = np.random.default_rng(seed)
    for _ in range(3):
        c = np.array([rng.uniform(-3000, 3000), rng.uniform(-3000, 3000), rng.uniform(-3500, -800)])
        ax = rng.uniform(200.0, 800.0, 3)
        inside = (((cen - c) / ax) ** 2).sum(axis=1) <= 1.0
        s[inside] = 10.0 ** rng.uniform(-3.0, 0.0)
    g = np.linspace(-4000.0, 4000.0, 20)
    X, Y = np.meshgrid(g, g, indexing="ij")
    rx = np.stack([X.ravel(), Y.ravel(), np.full(400, -1.0)], axis=1)
    m = Model(f"mt_p3_{n}cubed", nodes, tets, np.stack([s, s], axis=1), 3, None, rx)
    m.frequencies = [0.1, 1.0]
    m.polarizations = ["x", "y"]
    return m
