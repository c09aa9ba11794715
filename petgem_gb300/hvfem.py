"""Drop-in counterparts of petgem's ``hvfem`` entry points (petgem/hvfem.py).

Same names, argument meanings and return layouts as the reference; the
computation runs on the GPU through libpetgem_gb300.so.  Where petgem prints
and calls ``exit(-1)`` these raise ``PetgemError``/``ValueError``.

Batched siblings (``*_batched``) take and return device tensors for whole
meshes; the single-element functions wrap them with T = 1 and return numpy.
"""
import numpy as np
import torch

from . import kernels
from ._lib import PetgemError
from .engine import source_field

_dev = "cuda:0"


def _nd(p):
    return p * (p + 2) * (p + 3) // 2


def computeConnectivityDOFS(elemsE, elemsF, Nord):
    """petgem/hvfem.py:15 -> (dof_connectivity, dof_edges, dof_faces, dof_volume, total_num_dofs)."""
    from . import _lib
    from .engine import _p, _s
    if not 1 <= int(Nord) <= 6:
        raise ValueError("Nord must be 1..6")
    p = int(Nord)
    eE = torch.as_tensor(np.ascontiguousarray(elemsE), device=_dev).to(torch.int32).contiguous()
    eF = torch.as_tensor(np.ascontiguousarray(elemsF), device=_dev).to(torch.int32).contiguous()
    T = eE.shape[0]
    nE = int(eE.max().item()) + 1
    nF = int(eF.max().item()) + 1
    dofs = torch.empty((T, _nd(p)), dtype=torch.int32, device=_dev)
    _lib.call("pg_connectivity_dofs", _p(eE), _p(eF), T, nE, nF, p, _p(dofs), _s())
    de, df, dv = p, p * (p - 1), p * (p - 1) * (p - 2) // 2
    dof_edges = np.arange(nE * de, dtype=np.int64).reshape(nE, de)
    dof_faces = (nE * de + np.arange(nF * df, dtype=np.int64)).reshape(nF, df)
    dof_volume = (nE * de + nF * df + np.arange(T * dv, dtype=np.int64)).reshape(T, dv)
    d = dofs.cpu().numpy().astype(np.int64)
    return d, dof_edges, dof_faces, dof_volume, int(d.max()) + 1


def computeJacobian(eleNodes):
    """petgem/hvfem.py:101: J with rows x1-x0, x2-x0, x3-x0 and inv(J) (3x3 host helper)."""
    c = np.asarray(eleNodes, dtype=np.float64).reshape(4, 3)
    J = c[1:] - c[0]
    return J, np.linalg.inv(J)


def computeElementOrientation(edgesEle, nodesEle, edgesNodesEle, globalEdgesInFace):
    """petgem/hvfem.py:122 for one element -> (edge flags (6,), face codes (4,)).

    Runs the batched GPU kernel on a one-element mesh whose global edge and
    face tables are the element's own.
    """
    from . import _lib
    from .engine import _p, _s
    elemsN = torch.tensor([[0, 1, 2, 3]], dtype=torch.int32, device=_dev)
    nodes_local = np.asarray(nodesEle, dtype=np.int64).reshape(4)
    # express everything in local ids: node k of the element is local node k
    g2l = {int(g): k for k, g in enumerate(nodes_local)}
    en = np.asarray(edgesNodesEle, dtype=np.int64).reshape(6, 2)
    edgesNodes = torch.tensor([[g2l[int(a)], g2l[int(b)]] for a, b in en], dtype=torch.int32, device=_dev)
    eids = np.asarray(edgesEle, dtype=np.int64).reshape(6)
    e2l = {int(g): k for k, g in enumerate(eids)}
    fe = np.asarray(globalEdgesInFace, dtype=np.int64).reshape(4, 3)
    facesE = torch.tensor([[e2l[int(v)] for v in row] for row in fe], dtype=torch.int32, device=_dev)
    elemsE = torch.arange(6, dtype=torch.int32, device=_dev).view(1, 6)
    elemsF = torch.arange(4, dtype=torch.int32, device=_dev).view(1, 4)
    # nodes of the element's local edges must match their local numbering
    eo = torch.empty((1, 6), dtype=torch.int8, device=_dev)
    fo = torch.empty((1, 4), dtype=torch.int8, device=_dev)
    _lib.call("pg_element_orientation", _p(elemsN), _p(elemsE), _p(edgesNodes), _p(elemsF), _p(facesE), 1, _p(eo),
              _p(fo), _s())
    return eo[0].cpu().numpy().astype(np.int64), fo[0].cpu().numpy().astype(np.int64)


def computeElementalMatrices(edge_orientation, face_orientation, jacobian, invjacob, Nord, sigmaEle):
    """petgem/hvfem.py:223 for one element -> (Me, Ke) (nd x nd float64).

    The element is rebuilt from the Jacobian (x0 = 0, x_i = J[i-1]); invjacob
    is recomputed on the device, as the batched kernel works from vertices.
    """
    J = np.asarray(jacobian, dtype=np.float64).reshape(3, 3)
    coords = np.vstack([np.zeros(3), J]).reshape(1, 4, 3)
    M, K = computeElementalMatricesBatched(coords, np.asarray(edge_orientation).reshape(1, 6),
                                           np.asarray(face_orientation).reshape(1, 4),
                                           np.asarray(sigmaEle, dtype=np.float64).reshape(1, 2), int(Nord))
    return M[0].cpu().numpy(), K[0].cpu().numpy()


def computeElementalMatricesBatched(coords, eo, fo, sigma, p):
    """Batched sibling: coords (T,4,3), eo (T,6), fo (T,4), sigma (T,2) -> device (M, K) (T,nd,nd) f64."""
    T = coords.shape[0]
    nodes = torch.as_tensor(np.ascontiguousarray(coords, dtype=np.float64).reshape(-1, 3), device=_dev)
    elemsN = torch.arange(4 * T, dtype=torch.int32, device=_dev).view(T, 4)
    eo_t = torch.as_tensor(np.ascontiguousarray(eo), device=_dev).to(torch.int8).contiguous()
    fo_t = torch.as_tensor(np.ascontiguousarray(fo), device=_dev).to(torch.int8).contiguous()
    sig = torch.as_tensor(np.ascontiguousarray(sigma, dtype=np.float64), device=_dev).contiguous()
    tup, codes = kernels.orientation_tuples(eo_t, fo_t)
    tabs = kernels.tuple_tables(codes, p)
    return kernels.elemental_matrices(nodes, elemsN, sig, tup, tabs, p)


def computeSourceVectorRotation(azimuth, dip):
    """petgem/hvfem.py:2303: unit dipole direction after azimuth / dip rotations."""
    return source_field({"azimuth": azimuth, "dip": dip, "current": 1.0, "length": 1.0})


def computeBasisFunctions(edge_orientation, face_orientation, jacobian, invjacob, Nord, points):
    """petgem/hvfem.py:2493 -> (basis (3, nd, npts), curl_basis (3, nd, npts)) in the physical element.

    Evaluated on the GPU by the receiver-gather kernel applied to unit
    solution vectors (one per basis function).
    """
    from .engine import DeviceMesh
    p = int(Nord)
    nd = _nd(p)
    J = np.asarray(jacobian, dtype=np.float64).reshape(3, 3)
    coords = np.vstack([np.zeros(3), J])
    X = np.atleast_2d(np.asarray(points, dtype=np.float64))
    phys = X @ J                                  # x = x0 + J^T xi  (x0 = 0)
    m = DeviceMesh(coords, np.array([[0, 1, 2, 3]]), p, device=_dev, pattern=False)
    m.eo.copy_(torch.as_tensor(np.asarray(edge_orientation).reshape(1, 6), dtype=torch.int8))
    m.fo.copy_(torch.as_tensor(np.asarray(face_orientation).reshape(1, 4), dtype=torch.int8))
    m.dofs.copy_(torch.arange(nd, dtype=torch.int32).view(1, nd))
    basis = np.zeros((3, nd, len(X)))
    curl = np.zeros((3, nd, len(X)))
    omu = 1.0
    for j in range(nd):
        x = torch.zeros(nd, dtype=torch.complex128, device=_dev)
        x[j] = 1.0
        F, keep = _gather_at(m, x, phys, omu)
        basis[:, j, :] = F[:, :3].real.T
        curl[:, j, :] = (F[:, 3:] * 1j).real.T         # H = curl / (i w mu) with w mu = 1
    return basis, curl


def _gather_at(m, x, pts, omega_mu):
    from . import _lib
    from .engine import _p, _s
    pts_t = torch.as_tensor(np.ascontiguousarray(pts), device=_dev)
    elem = torch.zeros(pts_t.shape[0], dtype=torch.int32, device=_dev)
    F = torch.empty((pts_t.shape[0], 6), dtype=torch.complex128, device=_dev)
    _lib.call("pg_gather_fields", _p(x), _p(m.nodes), _p(m.elemsN), _p(m.eo), _p(m.fo), _p(m.dofs), m.p, _p(pts_t),
              _p(elem), pts_t.shape[0], omega_mu, _p(F), _s())
    return F.cpu().numpy(), None


def tetrahedronXYZToXiEtaZeta(eleNodes, points):
    """petgem/hvfem.py:2347: reference coordinates of physical points (host helper)."""
    c = np.asarray(eleNodes, dtype=np.float64).reshape(4, 3)
    J = c[1:] - c[0]
    pts = np.asarray(points, dtype=np.float64)
    out = np.linalg.solve(J.T, (np.atleast_2d(pts) - c[0]).T).T
    return out[0] if pts.ndim == 1 else out


__all__ = ["computeConnectivityDOFS", "computeJacobian", "computeElementOrientation", "computeElementalMatrices",
           "computeElementalMatricesBatched", "computeSourceVectorRotation", "computeBasisFunctions",
           "tetrahedronXYZToXiEtaZeta", "PetgemError"]
