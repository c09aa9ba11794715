"""Legacy VTK unstructured-grid writer (binary) for the nodal fields.

petgem writes its optional visualisation file with meshio
(petgem/postprocessing.py:262-336): tetrahedra, cell data sigma_horizontal /
sigma_vertical, and one point-data array per field component, real and
imaginary parts apart.  meshio is not available here, so this writes the same
content in the legacy VTK binary layout (big-endian, as the format requires),
which VTK and ParaView read.
"""
import numpy as np


def write(path, points, tets, point_data=None, cell_data=None):
    points = np.ascontiguousarray(points, dtype=np.float64)
    tets = np.ascontiguousarray(tets, dtype=np.int64)
    n, T = points.shape[0], tets.shape[0]
    with open(path, "wb") as f:
        def line(s):
            f.write((s + "\n").encode("ascii"))
        line("# vtk DataFile Version 4.2")
        line("petgem_gb300 nodal fields")
        line("BINARY")
        line("DATASET UNSTRUCTURED_GRID")
        line(f"POINTS {n} double")
        f.write(points.astype(">f8").tobytes())
        line("")
        line(f"CELLS {T} {5 * T}")
        cells = np.concatenate([np.full((T, 1), 4, dtype=np.int64), tets], axis=1)
        f.write(cells.astype(">i4").tobytes())
        line("")
        line(f"CELL_TYPES {T}")
        f.write(np.full(T, 10, dtype=">i4").tobytes())      # VTK_TETRA
        line("")
        for kind, count, data in (("CELL_DATA", T, cell_data), ("POINT_DATA", n, point_data)):
            if not data:
                continue
            line(f"{kind} {count}")
            line(f"FIELD FieldData {len(data)}")
            for name, arr in data.items():
                a = np.ascontiguousarray(arr, dtype=np.float64).reshape(count, -1)
                line(f"{name} {a.shape[1]} {count} double")
                f.write(a.astype(">f8").tobytes())
                line("")


def read(path):
    """Points, tets and the FIELD arrays of a file written by write() (for tests)."""
    raw = open(path, "rb").read()
    pos = 0

    def next_line():
        nonlocal pos
        e = raw.index(b"\n", pos)
        s = raw[pos:e].decode("ascii")
        pos = e + 1
        return s

    def take(dtype, count):
        nonlocal pos
        a = np.frombuffer(raw[pos:pos + count * np.dtype(dtype).itemsize], dtype=dtype)
        pos += count * np.dtype(dtype).itemsize
        return a
    for _ in range(4):
        next_line()
    n = int(next_line().split()[1])
    pts = take(">f8", 3 * n).reshape(n, 3).astype(np.float64)
    next_line()
    T = int(next_line().split()[1])
    cells = take(">i4", 5 * T).reshape(T, 5)[:, 1:].astype(np.int64)
    next_line()
    next_line()
    take(">i4", T)
    next_line()
    fields = {}
    while pos < len(raw):
        hdr = next_line()
        if not hdr:
            continue
        kind, count = hdr.split()
        nf = int(next_line().split()[2])
        for _ in range(nf):
            name, comp, cnt, _dt = next_line().split()
            fields[name] = take(">f8", int(comp) * int(cnt)).astype(np.float64)
            next_line()
    return pts, cells, fields
