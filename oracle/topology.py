"""Oracle: mesh topology, DOF numbering and PEC boundary DOFs (numpy).

Test infrastructure only (see ``oracle/__init__.py``).  Integer results must
be bit-exact against petgem; each function cites the reference it restates.
"""
import numpy as np

# local edge -> local vertex pair (petgem/mesh.py:27-32)
EDGE_LOCAL = ((0, 1), (1, 2), (0, 2), (0, 3), (1, 3), (2, 3))
# local face -> local vertex triple (petgem/mesh.py:68-71)
FACE_LOCAL = ((0, 1, 2), (0, 1, 3), (1, 2, 3), (0, 2, 3))
# local face -> its three local edges, in the order petgem stores them (mesh.py:116-123)
FACE_EDGES_LOCAL = ((0, 1, 2), (0, 4, 3), (1, 5, 4), (2, 5, 3))


def _unique_rows_first(rows):
    """Rank rows by lexicographic order of their sorted entries.

    Returns (first_index, inverse) like ``np.unique(..., return_index=True,
    return_inverse=True)`` on the row-sorted array, which is what petgem's
    ``deleteDuplicateRows``/``findUniqueRows`` do (petgem/vectors.py:15-64):
    ids are lexicographic ranks, ``first_index`` is the first occurrence.
    """
    key = np.sort(rows, axis=1)
    order = np.lexsort(key.T[::-1])          # stable: ties keep input order
    ks = key[order]
    new = np.ones(len(ks), dtype=bool)
    new[1:] = np.any(ks[1:] != ks[:-1], axis=1)
    gid = np.cumsum(new) - 1
    inverse = np.empty(len(rows), dtype=np.int64)
    inverse[order] = gid
    first = order[new]
    return first, inverse


def compute_edges(elemsN):
    """elemsE (T,6) and sorted edgesNodes (nE,2) (petgem/mesh.py:18-53)."""
    elemsN = np.asarray(elemsN, dtype=np.int64)
    T = elemsN.shape[0]
    pairs = np.stack([elemsN[:, list(e)] for e in EDGE_LOCAL], axis=1).reshape(-1, 2)
    first, inv = _unique_rows_first(pairs)
    edgesNodes = np.sort(pairs[first], axis=1)
    return inv.reshape(T, 6), edgesNodes


def compute_faces(elemsN):
    """elemsF (T,4) and facesN (nF,3) in first-seen vertex order (mesh.py:56-89)."""
    elemsN = np.asarray(elemsN, dtype=np.int64)
    T = elemsN.shape[0]
    tri = np.stack([elemsN[:, list(f)] for f in FACE_LOCAL], axis=1).reshape(-1, 3)
    first, inv = _unique_rows_first(tri)
    return inv.reshape(T, 4), tri[first]


def compute_faces_edges(elemsF, elemsE, nFaces):
    """facesE (nF,3): each face's edges in the local order of the lowest-index
    element that contains it (petgem/mesh.py:92-125 with vectors.py:81-132)."""
    elemsF = np.asarray(elemsF, dtype=np.int64)
    elemsE = np.asarray(elemsE, dtype=np.int64)
    T = elemsF.shape[0]
    face = elemsF.reshape(-1)
    elem = np.repeat(np.arange(T), 4)
    loc = np.tile(np.arange(4), T)
    order = np.lexsort((elem, face))
    fs = face[order]
    first = np.ones(len(fs), dtype=bool)
    first[1:] = fs[1:] != fs[:-1]
    owner = elem[order][first]
    lf = loc[order][first]
    fel = np.asarray(FACE_EDGES_LOCAL)[lf]               # (nF,3) local edge ids
    facesE = np.take_along_axis(elemsE[owner], fel, axis=1)
    assert facesE.shape[0] == nFaces
    return facesE


def compute_connectivity_dofs(elemsE, elemsF, p):
    """DOF numbering (petgem/hvfem.py:15-98): edge block, face block, volume block.

    Returns (dofs (T,nd), dof_edges (nE,p), dof_faces (nF,p(p-1)),
    dof_volume (T,p(p-1)(p-2)/2), total_num_dofs).
    """
    elemsE = np.asarray(elemsE, dtype=np.int64)
    elemsF = np.asarray(elemsF, dtype=np.int64)
    T = elemsE.shape[0]
    nE = int(elemsE.max()) + 1
    nF = int(elemsF.max()) + 1
    de, df, dv = p, p * (p - 1), p * (p - 1) * (p - 2) // 2
    dof_edges = np.arange(nE * de, dtype=np.int64).reshape(nE, de)
    dof_faces = (nE * de + np.arange(nF * df, dtype=np.int64)).reshape(nF, df)
    dof_volume = (nE * de + nF * df + np.arange(T * dv, dtype=np.int64)).reshape(T, dv)
    dofs = np.concatenate([dof_edges[elemsE].reshape(T, 6 * de),
                           dof_faces[elemsF].reshape(T, 4 * df),
                           dof_volume], axis=1)
    total = int(dofs.max()) + 1
    return dofs, dof_edges, dof_faces, dof_volume, total


def compute_boundary_faces(elemsF, facesN):
    """Faces owned by exactly one element, ascending (petgem/mesh.py:149-221).

    Returns (bfacesN (3,nB), bFaces (nB,), nB).
    """
    counts = np.bincount(np.asarray(elemsF).reshape(-1), minlength=facesN.shape[0])
    bFaces = np.nonzero(counts == 1)[0]
    return np.ascontiguousarray(facesN[bFaces].T), bFaces, len(bFaces)


def compute_boundary_edges(facesE, bFaces):
    """Edges lying on boundary faces, ascending id (petgem/mesh.py:224-277)."""
    return np.unique(np.asarray(facesE)[bFaces].reshape(-1))


def compute_boundaries(dofs, dof_edges, dof_faces, bEdges, bFaces, p):
    """(inner dofs, boundary dofs) in petgem's order (petgem/mesh.py:280-321)."""
    b_e = dof_edges[bEdges].reshape(-1)
    b_f = dof_faces[bFaces].reshape(-1) if dof_faces.size else np.zeros(0, np.int64)
    bnd = np.concatenate([b_e, b_f])
    total = int(dofs.max()) + 1
    inner = np.setdiff1d(np.arange(total), bnd)
    return inner, bnd


def element_orientation(elemsN, elemsE, edgesNodes, elemsF, facesE):
    """Edge flags (T,6) and face codes (T,4) for every element, vectorised
    restatement of petgem/hvfem.py:122-220 (computeElementOrientation)."""
    elemsN = np.asarray(elemsN, dtype=np.int64)
    T = elemsN.shape[0]
    eo = np.zeros((T, 6), dtype=np.int64)
    for i, (a, b) in enumerate(EDGE_LOCAL):
        g = edgesNodes[elemsE[:, i]]
        eo[:, i] = ((elemsN[:, a] == g[:, 1]) & (elemsN[:, b] == g[:, 0])).astype(np.int64)
    fo = np.zeros((T, 4), dtype=np.int64)
    code = {12: 0, 31: 1, 23: 2, 32: 3, 13: 4, 21: 5}
    for i, le in enumerate(FACE_EDGES_LOCAL):
        gf = facesE[elemsF[:, i]]                    # (T,3) global edges of this face
        e0 = elemsE[:, le[0]]
        e1 = elemsE[:, le[1]]
        k1 = np.zeros(T, dtype=np.int64)
        k2 = np.zeros(T, dtype=np.int64)
        for k in range(3):
            k1 = np.where(e0 == gf[:, k], k + 1, k1)
            k2 = np.where(e1 == gf[:, k], k + 1, k2)
        sel = k1 * 10 + k2
        out = np.zeros(T, dtype=np.int64)
        for s, c in code.items():
            out[sel == s] = c
        fo[:, i] = out
    return eo, fo
