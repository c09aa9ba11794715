"""Nodal E/H for visualisation: GPU node averaging against the oracle
restatement of petgem's postprocessing loop, and the VTK file written from it."""
import numpy as np
import pytest
import torch

from oracle import fem, topology
from tests.helpers import load_test_mesh, rel_norm

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("p", [1, 2])
def test_node_fields_vs_oracle(p, tmp_path):
    from petgem_gb300 import vtk
    from petgem_gb300.engine import DeviceMesh
    pts, tets, phys = load_test_mesh()
    sel = tets[:1500]                      # a connected subset keeps the oracle loop short
    used = np.unique(sel)
    remap = -np.ones(len(pts), dtype=np.int64)
    remap[used] = np.arange(len(used))
    pts2, tets2 = pts[used], remap[sel]
    m = DeviceMesh(pts2, tets2, p)
    rng = np.random.default_rng(p)
    x = rng.standard_normal(m.N) + 1j * rng.standard_normal(m.N)
    F = m.node_fields(torch.as_tensor(x, device=m.device), 2.0).cpu().numpy()
    eE, eN = topology.compute_edges(tets2)
    eF, fN = topology.compute_faces(tets2)
    fE = topology.compute_faces_edges(eF, eE, fN.shape[0])
    eo, fo = topology.element_orientation(tets2, eE, eN, eF, fE)
    dofs, _, _, _, _ = topology.compute_connectivity_dofs(eE, eF, p)
    Fo = fem.node_fields(x, pts2, tets2, eo, fo, dofs, p, 2.0)
    assert rel_norm(F[:, :3], Fo[:, :3]) < 1e-12
    assert rel_norm(F[:, 3:], Fo[:, 3:]) < 1e-12
    path = tmp_path / "f.vtk"
    vtk.write(path, pts2, tets2, {"Ex_real": F[:, 0].real}, {"sigma_horizontal": np.ones(len(tets2))})
    p2, t2, fields = vtk.read(path)
    assert np.array_equal(p2, pts2) and np.array_equal(t2, tets2)
    assert np.array_equal(fields["Ex_real"], F[:, 0].real)


def test_node_fields_vs_reference_loop_golden():
    """pg_node_fields against petgem's own VTK nodal loop
    (postprocessing.py:172-261; tests/golden/make_node_fields_golden.py)."""
    from petgem_gb300.engine import DeviceMesh
    from tests.helpers import load
    g = load("node_fields.npz")
    cases = [(g["n3_points"], g["n3_tets"], 2, g["n3_x"], g["n3_frequency"], g["n3_fields"])]
    for p in (1, 3):
        cases.append((g["tm_points"], g["tm_tets"], p, g[f"tm_p{p}_x"], g["tm_frequency"], g[f"tm_p{p}_fields"]))
    for pts, tets, p, x, f, ref in cases:
        m = DeviceMesh(pts, tets, p)
        F = m.node_fields(torch.as_tensor(x, device=m.device), float(f)).cpu().numpy()
        assert rel_norm(F[:, :3], ref[:, :3]) < 1e-12, p
        assert rel_norm(F[:, 3:], ref[:, 3:]) < 1e-12, p
