"""Tensor-level wrappers over the C ABI (device tensors in, device tensors out).

torch provides device memory and the current CUDA stream; every computation
runs in ``libpetgem_gb300.so``.  All functions require CUDA tensors and raise
``PetgemError`` on a failed status.
"""
import ctypes

import torch

from . import _lib

_u8 = torch.uint8


def _ptr(t):
    return ctypes.c_void_p(t.data_ptr()) if t is not None else ctypes.c_void_p(0)


def _stream():
    return ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)


def _check_cuda(*ts):
    for t in ts:
        if t is not None and not t.is_cuda:
            raise ValueError("petgem_gb300 kernels need CUDA tensors")
        if t is not None and not t.is_contiguous():
            raise ValueError("petgem_gb300 kernels need contiguous tensors")


def ndof(p):
    return p * (p + 2) * (p + 3) // 2


def workspace(nbytes, device):
    return torch.empty(max(int(nbytes), 1), dtype=_u8, device=device)


def orientation_tuples(eo, fo):
    """Distinct orientation tuples: returns (tuple_of_elem int32 [T], codes int32 [U])."""
    _check_cuda(eo, fo)
    T = eo.shape[0]
    dev = eo.device
    tup = torch.empty(T, dtype=torch.int32, device=dev)
    codes = torch.empty(min(T, 64 * 1296), dtype=torch.int32, device=dev)
    n = torch.zeros(1, dtype=torch.int64, device=dev)
    ws = workspace(_lib.query("pg_tuples_workspace_bytes", T), dev)
    _lib.call("pg_orientation_tuples", _ptr(eo), _ptr(fo), T, _ptr(tup), _ptr(codes), _ptr(n), _ptr(ws),
              ws.numel(), _stream())
    U = int(n.item())
    return tup, codes[:U].clone()


def tuple_tables(codes, p):
    """Reference-space moment tables, f64 [U, 12, nd(nd+1)/2]."""
    _check_cuda(codes)
    U = codes.shape[0]
    per = _lib.query("pg_table_doubles", p)
    tab = torch.empty(U * per, dtype=torch.float64, device=codes.device)
    _lib.call("pg_tuple_tables", _ptr(codes), U, p, _ptr(tab), _stream())
    nd = ndof(p)
    return tab.view(U, 12, nd * (nd + 1) // 2)


def elemental_matrices(nodes, elemsN, sigma, tuple_of_elem, tables, p):
    """Batched elemental (M, K), each f64 [T, nd, nd] (signed det(J) scaling)."""
    _check_cuda(nodes, elemsN, sigma, tuple_of_elem, tables)
    T = elemsN.shape[0]
    nd = ndof(p)
    dev = nodes.device
    M = torch.empty((T, nd, nd), dtype=torch.float64, device=dev)
    K = torch.empty((T, nd, nd), dtype=torch.float64, device=dev)
    st = torch.zeros(1, dtype=torch.int32, device=dev)
    _lib.call("pg_elemental_matrices", _ptr(nodes), _ptr(elemsN), _ptr(sigma), _ptr(tuple_of_elem), _ptr(tables),
              T, p, _ptr(M), _ptr(K), _ptr(st), _stream())
    s = int(st.item())
    if s != 0:
        raise _lib.PetgemError("pg_elemental_matrices", s, "degenerate element (det(J) == 0 or non-finite)")
    return M, K
