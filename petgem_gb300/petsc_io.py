"""PETSc binary files: the scratch format petgem's stages exchange.

petgem's Preprocessing writes the mesh, DOF maps and model as PETSc binary
matrices / vectors (petgem/preprocessing.py, parallel.py:65-140), its Solver
reads them and writes the solutions x{i}.dat, and its Postprocessing reads
those back.  Reading and writing the same files lets either side of a mixed
run be petgem's own code: petgem's preprocessing can feed this solver, and
this solver's solutions can feed petgem's postprocessing.

Layout (big-endian, PETSc built with complex scalars and 32-bit indices):

* vector: int32 classid 1211214, int32 n, then n complex128 values;
* matrix (AIJ; dense matrices are written this way too, every row full):
  int32 classid 1211216, int32 rows, int32 cols, int32 nnz, int32 [rows] row
  lengths, int32 [nnz] column indices, complex128 [nnz] values.  A header
  with nnz = -1 marks PETSc's native dense layout (values row by row), which
  is read as well.
"""
import numpy as np

VEC_CLASSID = 1211214
MAT_CLASSID = 1211216
_I4 = np.dtype(">i4")
_C16 = np.dtype(">c16")


def write_vec(path, x):
    x = np.asarray(x).reshape(-1)
    with open(path, "wb") as f:
        f.write(np.array([VEC_CLASSID, x.size], dtype=_I4).tobytes())
        f.write(x.astype(_C16).tobytes())


def read_vec(path):
    raw = open(path, "rb").read()
    cid, n = np.frombuffer(raw[:8], dtype=_I4)
    if cid != VEC_CLASSID:
        raise ValueError(f"{path}: not a PETSc binary vector (classid {cid})")
    return np.frombuffer(raw[8:8 + 16 * n], dtype=_C16).astype(np.complex128)


def write_mat(path, rowptr, col, vals, shape):
    """AIJ matrix from CSR arrays."""
    rowptr = np.asarray(rowptr, dtype=np.int64)
    col = np.asarray(col)
    vals = np.asarray(vals).reshape(-1)
    m, n = shape
    with open(path, "wb") as f:
        f.write(np.array([MAT_CLASSID, m, n, col.size], dtype=_I4).tobytes())
        f.write(np.diff(rowptr).astype(_I4).tobytes())
        f.write(col.astype(_I4).tobytes())
        f.write(vals.astype(_C16).tobytes())


def write_dense(path, a):
    """A dense 2-D array the way petgem writes its scratch matrices (AIJ
    layout with every row full)."""
    a = np.atleast_2d(np.asarray(a))
    m, n = a.shape
    rowptr = np.arange(m + 1, dtype=np.int64) * n
    col = np.tile(np.arange(n, dtype=np.int32), m)
    write_mat(path, rowptr, col, a.reshape(-1), (m, n))


def read_mat(path):
    """(rowptr int64, col int32, vals complex128, (rows, cols))."""
    raw = open(path, "rb").read()
    cid, m, n, nz = np.frombuffer(raw[:16], dtype=_I4)
    if cid != MAT_CLASSID:
        raise ValueError(f"{path}: not a PETSc binary matrix (classid {cid})")
    off = 16
    if nz == -1:                                   # native dense layout
        vals = np.frombuffer(raw[off:off + 16 * m * n], dtype=_C16).astype(np.complex128)
        rowptr = np.arange(m + 1, dtype=np.int64) * n
        col = np.tile(np.arange(n, dtype=np.int32), m)
        return rowptr, col, vals, (int(m), int(n))
    lens = np.frombuffer(raw[off:off + 4 * m], dtype=_I4).astype(np.int64)
    off += 4 * m
    col = np.frombuffer(raw[off:off + 4 * nz], dtype=_I4).astype(np.int32)
    off += 4 * nz
    vals = np.frombuffer(raw[off:off + 16 * nz], dtype=_C16).astype(np.complex128)
    rowptr = np.concatenate([[0], np.cumsum(lens)])
    return rowptr, col, vals, (int(m), int(n))


def read_dense(path):
    """A matrix file with full rows as a dense (rows, cols) complex array."""
    rowptr, col, vals, (m, n) = read_mat(path)
    if vals.size != m * n:
        raise ValueError(f"{path}: not a dense matrix ({vals.size} of {m * n} entries stored)")
    out = np.zeros((m, n), dtype=np.complex128)
    out[np.repeat(np.arange(m), np.diff(rowptr)), col] = vals
    return out


def read_petgem_scratch(directory):
    """Mesh and model from petgem's preprocessing scratch files: nodes
    (n_nodes, 3) rebuilt from nodes.dat (per-element coordinates) and
    meshConnectivity.dat, tets (T, 4), sigma (T, 2) from
    conductivityModel.dat (petgem/preprocessing.py:88-285)."""
    import os
    coords = read_dense(os.path.join(directory, "nodes.dat")).real
    tets = np.rint(read_dense(os.path.join(directory, "meshConnectivity.dat")).real).astype(np.int64)
    sigma = read_dense(os.path.join(directory, "conductivityModel.dat")).real
    nodes = np.zeros((int(tets.max()) + 1, 3))
    nodes[tets.reshape(-1)] = coords.reshape(-1, 3)
    return nodes, tets, sigma
