"""The allocation-free entry point pg_select_equal_noalloc, called through the
C ABI, against pg_select_equal (which takes a caller-allocated workspace).

pg_select_equal_noalloc exists for callers that cannot allocate device
memory: its scratch is a static device array inside the library, so the call
itself allocates nothing.  The results are integer indices, so they must be
identical; two calls in a row check that no state from the first call leaks
into the second (the static scratch keeps its contents between calls).
This file is named so that pytest collects it last."""
import ctypes

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


def _select(lib, values, target, noalloc):
    dev = values.device
    n = values.numel()
    out = torch.full((n,), -7, dtype=torch.int32, device=dev)
    cnt = torch.full((1,), -7, dtype=torch.int64, device=dev)
    s = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    P = lambda t: ctypes.c_void_p(t.data_ptr())
    if noalloc:
        st = lib.pg_select_equal_noalloc(P(values), n, int(target), P(out), P(cnt), s)
    else:
        nbytes = lib.pg_select_workspace_bytes(n)
        ws = torch.empty(nbytes, dtype=torch.uint8, device=dev)
        st = lib.pg_select_equal(P(values), n, int(target), P(out), P(cnt), P(ws), nbytes, s)
    assert st == 0, lib.pg_last_error()
    torch.cuda.synchronize()
    k = int(cnt.item())
    return out[:k].cpu().numpy()


def test_noalloc_matches_workspace_version_twice():
    from petgem_gb300 import _lib
    lib = _lib.load()
    assert lib.pg_select_equal_noalloc_max_n() == 262144
    rng = np.random.default_rng(11)
    dev = torch.device("cuda:0")
    cases = [(rng.integers(0, 3, 200_000), 1), (rng.integers(0, 5, 262_144), 4)]
    for vals, target in cases:                           # two calls in a row, different sizes and data
        v = torch.as_tensor(vals.astype(np.int32), device=dev)
        a = _select(lib, v, target, noalloc=True)
        b = _select(lib, v, target, noalloc=False)
        assert np.array_equal(a, b)
        assert np.array_equal(a, np.nonzero(vals == target)[0])


def test_noalloc_rejects_sizes_beyond_the_limit():
    from petgem_gb300 import _lib
    lib = _lib.load()
    n = lib.pg_select_equal_noalloc_max_n() + 1
    # the size check happens before any pointer is touched: the buffers are never accessed
    dummy = torch.zeros(1, dtype=torch.int32, device="cuda:0")
    cnt = torch.zeros(1, dtype=torch.int64, device="cuda:0")
    P = lambda t: ctypes.c_void_p(t.data_ptr())
    st = lib.pg_select_equal_noalloc(P(dummy), n, 0, P(dummy), P(cnt), ctypes.c_void_p(0))
    assert st == -1
    assert b"static scratch limit" in lib.pg_last_error()
