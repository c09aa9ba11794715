"""Legacy VTK writer: layout and round trip (CPU)."""
import numpy as np

from petgem_gb300 import vtk


def test_vtk_round_trip_and_header(tmp_path):
    from petgem_gb300 import synthetic
    nodes, tets = synthetic.kuhn_box(2)
    rng = np.random.default_rng(0)
    pd = {"csem_Ex_real": rng.standard_normal(len(nodes)), "csem_Ex_imag": rng.standard_normal(len(nodes))}
    cd = {"sigma_horizontal": rng.uniform(0.1, 1.0, len(tets))}
    path = tmp_path / "m.vtk"
    vtk.write(path, nodes, tets, pd, cd)
    head = open(path, "rb").read(200).split(b"\n")
    assert head[0] == b"# vtk DataFile Version 4.2" and head[2] == b"BINARY"
    assert head[3] == b"DATASET UNSTRUCTURED_GRID" and head[4] == f"POINTS {len(nodes)} double".encode()
    p2, t2, fields = vtk.read(path)
    assert np.array_equal(p2, nodes) and np.array_equal(t2, tets)
    for k, v in {**pd, **cd}.items():
        assert np.array_equal(fields[k], v)
