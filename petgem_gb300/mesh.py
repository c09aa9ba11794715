"""Drop-in counterparts of petgem's mesh-topology functions (petgem/mesh.py).

Same names, arguments and return layouts as the reference; numbering is
bit-exact with petgem and is computed on the GPU (libpetgem_gb300.so).
Host numpy only converts inputs and outputs.
"""
import numpy as np
import torch

from . import _lib
from .engine import _p, _s, _ws

_dev = "cuda:0"


def _i32(a):
    return torch.as_tensor(np.ascontiguousarray(a), device=_dev).to(torch.int32).contiguous()


def _np(t):
    return t.cpu().numpy().astype(np.int64)


def _topology(elemsN):
    en = _i32(elemsN)
    T = en.shape[0]
    nn = int(en.max().item()) + 1
    i32 = dict(dtype=torch.int32, device=_dev)
    eE = torch.empty((T, 6), **i32)
    eF = torch.empty((T, 4), **i32)
    edgesNodes = torch.empty((6 * T, 2), **i32)
    facesN = torch.empty((4 * T, 3), **i32)
    facesE = torch.empty((4 * T, 3), **i32)
    fnel = torch.empty(4 * T, **i32)
    counts = torch.zeros(2, dtype=torch.int64, device=_dev)
    status = torch.zeros(1, **i32)
    ws = _ws(_lib.query("pg_topology_workspace_bytes", T), torch.device(_dev))
    _lib.call("pg_topology", _p(en), T, max(nn, 4), _p(eE), _p(eF), _p(edgesNodes), _p(facesN), _p(facesE), _p(fnel),
              _p(counts), _p(status), _p(ws), ws.numel(), _s())
    nE, nF = [int(v) for v in counts.cpu().tolist()]
    return eE, eF, edgesNodes[:nE], facesN[:nF], facesE[:nF], fnel[:nF]


def _select_equal(values, target):
    n = values.numel()
    out = torch.empty(max(n, 1), dtype=torch.int32, device=_dev)
    cnt = torch.zeros(1, dtype=torch.int64, device=_dev)
    ws = _ws(_lib.query("pg_select_workspace_bytes", n), torch.device(_dev))
    _lib.call("pg_select_equal", _p(values), n, int(target), _p(out), _p(cnt), _p(ws), ws.numel(), _s())
    return out[:int(cnt.item())]


def computeEdges(elemsN, nElems):
    """petgem/mesh.py:18 -> (elemsE (T,6), edgesNodes (nE,2) sorted)."""
    eE, _, eN, _, _, _ = _topology(np.asarray(elemsN)[:nElems])
    return _np(eE), _np(eN)


def computeFaces(elemsN, nElems):
    """petgem/mesh.py:56 -> (elemsF (T,4), facesN (nF,3) first-seen vertex order)."""
    _, eF, _, fN, _, _ = _topology(np.asarray(elemsN)[:nElems])
    return _np(eF), _np(fN)


def computeFacesEdges(elemsF, elemsE, nFaces, nElems):
    """petgem/mesh.py:92: each face's edges, in the local order of the
    lowest-index element that contains it."""
    eF = _i32(np.asarray(elemsF)[:nElems])
    eE = _i32(np.asarray(elemsE)[:nElems])
    facesE = torch.empty((nFaces, 3), dtype=torch.int32, device=_dev)
    owner = torch.empty(nFaces, dtype=torch.int32, device=_dev)
    st = torch.zeros(1, dtype=torch.int32, device=_dev)
    _lib.call("pg_faces_edges", _p(eF), _p(eE), eF.shape[0], nFaces, _p(facesE), _p(owner), _p(st), _s())
    if int(st.item()) != 0:
        raise _lib.PetgemError("pg_faces_edges", int(st.item()), "face index out of range")
    return _np(facesE)


def computeBoundaryFaces(elemsF, facesN):
    """petgem/mesh.py:149 -> (bfacesN (3,nB), bFaces (nB,), nB): faces owned by exactly one element."""
    facesN = np.asarray(facesN)
    eF = _i32(elemsF)
    nF = facesN.shape[0]
    cnt = torch.empty(nF, dtype=torch.int32, device=_dev)
    _lib.call("pg_face_counts", _p(eF), eF.shape[0], nF, _p(cnt), _s())
    bFaces = _np(_select_equal(cnt, 1))
    return np.ascontiguousarray(facesN[bFaces].T), bFaces, len(bFaces)


def computeBoundaryEdges(edgesN, bfacesN):
    """petgem/mesh.py:224: ids (ascending) of the edges lying on boundary faces."""
    edgesN = np.asarray(edgesN)
    bf = np.asarray(bfacesN).T
    pairs = np.concatenate([bf[:, [0, 1]], bf[:, [1, 2]], bf[:, [2, 0]]])
    pairs = np.sort(pairs, axis=1)
    eN = _i32(edgesN)
    pr = _i32(pairs)
    flags = torch.empty(eN.shape[0], dtype=torch.int32, device=_dev)
    _lib.call("pg_flag_edges_of_pairs", _p(eN), eN.shape[0], _p(pr), pr.shape[0], _p(flags), _s())
    return _np(_select_equal(flags, 1))


def computeBoundaries(dof_connectivity, dof_edges, dof_faces, bEdges, bFaces, Nord):
    """petgem/mesh.py:280 -> (inner dofs, boundary dofs): boundary = edge DOFs
    of boundary edges then face DOFs of boundary faces (index gathers)."""
    b_e = np.asarray(dof_edges)[np.asarray(bEdges)].reshape(-1)
    df = np.asarray(dof_faces)
    b_f = df[np.asarray(bFaces)].reshape(-1) if df.size else np.zeros(0, np.int64)
    bnd = np.concatenate([b_e, b_f]).astype(np.int64)
    total = int(np.max(dof_connectivity)) + 1
    mark = torch.zeros(total, dtype=torch.int32, device=_dev)
    if bnd.size:
        mark[torch.as_tensor(bnd, device=_dev)] = 1
    inner = _np(_select_equal(mark, 0))
    return inner, bnd
