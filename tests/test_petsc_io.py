"""PETSc binary scratch files: petgem's own test fixtures read back (a solved
system: the residual of the stored solution is small), round trips, and a
petgem-style scratch directory read into a mesh."""
import os

import numpy as np
import pytest
import scipy.sparse as sp

from petgem_gb300 import petsc_io

FIX = os.path.join(os.path.dirname(__file__), "golden")


def test_vector_and_matrix_round_trip(tmp_path):
    rng = np.random.default_rng(0)
    x = rng.standard_normal(37) + 1j * rng.standard_normal(37)
    petsc_io.write_vec(tmp_path / "x.dat", x)
    assert np.array_equal(petsc_io.read_vec(tmp_path / "x.dat"), x)
    A = sp.random(20, 20, density=0.2, random_state=1, format="csr") + 1j * sp.eye(20)
    A.sort_indices()
    petsc_io.write_mat(tmp_path / "A.dat", A.indptr, A.indices, A.data, A.shape)
    rp, col, vals, shape = petsc_io.read_mat(tmp_path / "A.dat")
    assert shape == (20, 20)
    assert np.array_equal(rp, A.indptr) and np.array_equal(col, A.indices) and np.array_equal(vals, A.data)
    D = rng.standard_normal((5, 12))
    petsc_io.write_dense(tmp_path / "D.dat", D)
    assert np.array_equal(petsc_io.read_dense(tmp_path / "D.dat").real, D)


def test_file_layout_is_big_endian_petsc():
    """Byte layout: classid, sizes and values big-endian (PETSc's binary viewer)."""
    x = np.array([1.0 + 2.0j])
    path = os.path.join(os.path.dirname(__file__), "_tmp_vec.dat")
    try:
        petsc_io.write_vec(path, x)
        raw = open(path, "rb").read()
    finally:
        os.remove(path)
    assert raw[:8] == np.array([1211214, 1], dtype=">i4").tobytes()
    assert raw[8:] == np.array([1.0, 2.0], dtype=">f8").tobytes()


def test_petgem_scratch_round_trip(tmp_path):
    from petgem_gb300 import synthetic
    nodes, tets = synthetic.kuhn_box(2)
    sigma = np.stack([np.arange(len(tets)) + 1.0, np.ones(len(tets))], 1)
    petsc_io.write_dense(tmp_path / "nodes.dat", nodes[tets].reshape(len(tets), 12))
    petsc_io.write_dense(tmp_path / "meshConnectivity.dat", tets)
    petsc_io.write_dense(tmp_path / "conductivityModel.dat", sigma)
    n2, t2, s2 = petsc_io.read_petgem_scratch(str(tmp_path))
    assert np.array_equal(t2, tets) and np.array_equal(n2, nodes) and np.array_equal(s2, sigma)


def test_reads_petgem_fixture_system():
    """petgem's tests/test_petsc.py system (matrix-A / vector-b / vector-x,
    x the zero initial guess): sizes from the headers, a direct solve of the
    decoded system leaves a rounding-level residual, the PEC rows are unit."""
    import scipy.sparse.linalg as spla
    paths = [os.path.join(FIX, f) for f in ("petgem_matrix-A.dat", "petgem_vector-b.dat", "petgem_vector-x.dat")]
    rp, col, vals, shape = petsc_io.read_mat(paths[0])
    A = sp.csr_matrix((vals, col, rp), shape=shape)
    b = petsc_io.read_vec(paths[1])
    x0 = petsc_io.read_vec(paths[2])
    assert shape == (4184, 4184) and A.nnz == 49931 and b.size == x0.size == 4184
    assert not np.any(x0)
    x = spla.spsolve(A.tocsc(), b)
    assert np.linalg.norm(A @ x - b) <= 1e-10 * np.linalg.norm(b)
    assert vals[0] == 1.0 and rp[1] - rp[0] == 1
