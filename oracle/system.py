"""Oracle: a whole CSEM forward system on the CPU, as petgem's Solver builds it.

Test infrastructure only (see ``oracle/__init__.py``): used by ``tests/`` and
by the CPU-baseline leg of ``bench.py`` as the checker and the timed CPU
path, never by the product.

The steps follow petgem/solver.py in order:

* topology and DOF numbering: ``mesh.computeEdges/Faces/FacesEdges``
  (petgem/mesh.py:18-125) and ``hvfem.computeConnectivityDOFS``
  (petgem/hvfem.py:15-98), restated in ``oracle.topology``;
* elemental matrices per element (petgem/solver.py:182-235,
  hvfem.py:223-316), spread over processes started with ``spawn`` (safe
  after a CUDA context exists in the parent);
* global assembly as a COO sum (PETSc ADD_VALUES);
* PEC: ``zeroRowsColumns(boundaries, diag=1)`` and ``b[boundaries] = 0``
  (petgem/solver.py:552-577, mesh.py:149-321);
* the point-dipole right-hand side (petgem/solver.py:247-316).
"""
import multiprocessing as mp

import numpy as np

from . import fem, topology


def _mk_chunk(args):
    coords, eo, fo, sigma, p = args
    return fem.element_matrices_batch(coords, eo, fo, sigma, p)


def element_matrices(coords, eo, fo, sigma, p, processes=None, pool=None):
    """(M, K) f64 [T, nd, nd] for every element, over `processes` spawn workers."""
    T = coords.shape[0]
    processes = processes or mp.cpu_count() or 1
    if processes <= 1 or T < 2048:
        return fem.element_matrices_batch(coords, eo, fo, sigma, p)
    parts = np.array_split(np.arange(T), processes * 4)
    jobs = [(coords[i], eo[i], fo[i], sigma[i], p) for i in parts]
    own = pool is None
    if own:
        pool = mp.get_context("spawn").Pool(processes)
    try:
        res = pool.map(_mk_chunk, jobs)
    finally:
        if own:
            pool.close()
            pool.join()
    return np.concatenate([r[0] for r in res]), np.concatenate([r[1] for r in res])


def mesh_maps(nodes, tets, p):
    """Topology, orientation, DOF map and PEC DOFs of a tetrahedral mesh."""
    eE, eN = topology.compute_edges(tets)
    eF, fN = topology.compute_faces(tets)
    fE = topology.compute_faces_edges(eF, eE, fN.shape[0])
    eo, fo = topology.element_orientation(tets, eE, eN, eF, fE)
    dofs, de, df, dv, N = topology.compute_connectivity_dofs(eE, eF, p)
    _, bF, _ = topology.compute_boundary_faces(eF, fN)
    bE = topology.compute_boundary_edges(fE, bF)
    _, bnd = topology.compute_boundaries(dofs, de, df, bE, bF, p)
    return {"elemsE": eE, "elemsF": eF, "eo": eo, "fo": fo, "dofs": dofs, "N": N, "bnd": bnd}


def csem_system(nodes, tets, sigma, p, src, processes=None, pec=True, pool=None):
    """A (scipy CSR, PEC applied when pec) and b of a CSEM model; returns a
    dict with A, b, the maps of ``mesh_maps`` and the source element."""
    mm = mesh_maps(nodes, tets, p)
    M, K = element_matrices(nodes[tets], mm["eo"], mm["fo"], sigma, p, processes, pool)
    A = fem.assemble(M, K, mm["dofs"], mm["N"], src["frequency"])
    del M, K
    b, se = fem.source_vector(nodes, tets, mm["eo"], mm["fo"], mm["dofs"], mm["N"], p, src)
    if pec:
        A, b = pec_in_pattern(A, b, mm["bnd"])
    return dict(mm, A=A, b=b, src_elem=se)


def pec_in_pattern(A, b, bnd):
    """zeroRowsColumns(rows, diag=1) and b[rows] = 0 (petgem/solver.py:552-577)
    on a copy of A that keeps every stored entry, as PETSc's AIJ matrix does
    (zeroed entries stay in the pattern; ``fem.apply_pec`` drops them)."""
    A = A.tocsr(copy=True)
    flag = np.zeros(A.shape[0], dtype=bool)
    flag[np.asarray(bnd, dtype=np.int64)] = True
    rows = np.repeat(np.arange(A.shape[0]), np.diff(A.indptr))
    hit = flag[rows] | flag[A.indices]
    A.data[hit] = 0.0
    A.data[hit & (rows == A.indices)] = 1.0
    b = np.array(b, dtype=np.complex128, copy=True)
    b[flag] = 0.0
    return A, b


def receiver_fields(sysd, x, nodes, tets, p, receivers, frequency):
    """E and H at the receivers inside the mesh (petgem/postprocessing.py:479-616)."""
    return fem.interpolate_fields(x, nodes, tets, sysd["eo"], sysd["fo"], sysd["dofs"], p, receivers, frequency)
