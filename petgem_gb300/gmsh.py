"""Minimal reader for gmsh 2.x ASCII meshes (tetrahedra + physical tags).

petgem reads the mesh with meshio (petgem/preprocessing.py:78-81) and uses
``mesh.points`` and the first cell block, which must be the tetrahedra.
meshio is not available here, so this reader returns the same arrays:
node coordinates in file order and 0-based tetrahedron connectivity with the
gmsh physical tag of each tet.
"""
import numpy as np


class GmshMesh:
    def __init__(self, points, tets, physical):
        self.points = points          # (nNodes, 3) float64
        self.tets = tets              # (nElems, 4) int64, 0-based
        self.physical = physical      # (nElems,) int64 gmsh physical tag


def read(path):
    with open(path, "r") as f:
        lines = f.read().split("\n")
    pos = {ln.strip(): i for i, ln in enumerate(lines) if ln.startswith("$")}
    if "$MeshFormat" in pos:
        ver = lines[pos["$MeshFormat"] + 1].split()[0]
        if not ver.startswith("2"):
            raise ValueError(f"{path}: gmsh format {ver} not supported (need 2.x ASCII)")
    i = pos["$Nodes"]
    nn = int(lines[i + 1])
    rows = np.array([ln.split() for ln in lines[i + 2:i + 2 + nn]], dtype=np.float64)
    tags = rows[:, 0].astype(np.int64)
    points = np.ascontiguousarray(rows[:, 1:4])
    tag_to_index = {int(t): k for k, t in enumerate(tags)}
    i = pos["$Elements"]
    ne = int(lines[i + 1])
    tets, phys = [], []
    for ln in lines[i + 2:i + 2 + ne]:
        v = ln.split()
        if int(v[1]) != 4:
            continue
        ntags = int(v[2])
        phys.append(int(v[3]) if ntags > 0 else 0)
        tets.append([tag_to_index[int(x)] for x in v[3 + ntags:3 + ntags + 4]])
    return GmshMesh(points, np.asarray(tets, dtype=np.int64), np.asarray(phys, dtype=np.int64))


def write(path, points, tets, physical=None):
    """Write a gmsh 2.2 ASCII file with tetrahedra (type 4) and physical tags."""
    points = np.asarray(points, dtype=np.float64)
    tets = np.asarray(tets, dtype=np.int64)
    phys = np.ones(len(tets), dtype=np.int64) if physical is None else np.asarray(physical, dtype=np.int64)
    with open(path, "w") as f:
        f.write("$MeshFormat\n2.2 0 8\n$EndMeshFormat\n$Nodes\n%d\n" % len(points))
        for i, (x, y, z) in enumerate(points):
            f.write("%d %.17g %.17g %.17g\n" % (i + 1, x, y, z))
        f.write("$EndNodes\n$Elements\n%d\n" % len(tets))
        for i, (t, ph) in enumerate(zip(tets, phys)):
            f.write("%d 4 2 %d %d %d %d %d %d\n" % (i + 1, ph, ph, t[0] + 1, t[1] + 1, t[2] + 1, t[3] + 1))
        f.write("$EndElements\n")
