"""The C-ABI library loads and exports every function include/petgem_gb300.h
declares (no GPU needed: nothing is called except pure host queries)."""
import os
import re

from petgem_gb300 import _build, _lib

HEADER = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "include", "petgem_gb300.h")


def declared_functions():
    text = open(HEADER).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    names = re.findall(r"\b(pg_[a-z0-9_]+)\s*\(", text)
    return sorted(set(names))


def test_header_declares_functions():
    names = declared_functions()
    assert "pg_gmres" in names and "pg_topology" in names and len(names) >= 25


def test_library_exports_every_declared_symbol():
    lib = _lib.load()
    missing = [n for n in declared_functions() if not hasattr(lib, n)]
    assert not missing, missing


def test_ctypes_signatures_cover_header():
    assert set(declared_functions()) == set(_lib.SIGNATURES)


def test_host_queries():
    lib = _lib.load()
    assert lib.pg_abi_version() == 4
    assert _lib.query("pg_table_doubles", 2) == 12 * 20 * 21 // 2
    assert _lib.query("pg_table_doubles", 7) == 0
    assert _lib.query("pg_pattern_local_entities", 1) == 6
    assert _lib.query("pg_pattern_local_entities", 3) == 11
    o = _lib.GmresOpts()
    lib.pg_gmres_default_opts(o)
    assert o.restart == 30 and abs(o.rtol - 1e-8) < 1e-20 and o.precision == 0


def test_noalloc_limit_matches_header_and_select_workspace():
    """The allocation-free select's limit is the header's PG_NOALLOC_MAX_N,
    and the workspace formula its static scratch is sized by is the one
    pg_select_workspace_bytes reports (one compile-time function in
    csrc/pg_sort.cuh): 2 int32 arrays + one int64 partial per 2,048 + 512."""
    lib = _lib.load()
    m = re.search(r"#define\s+PG_NOALLOC_MAX_N\s+(\d+)", open(HEADER).read())
    n = int(m.group(1))
    assert _lib.query("pg_select_equal_noalloc_max_n") == n
    a256 = lambda b: (b + 255) // 256 * 256
    for k in (1, 2047, 2048, 2049, 100_000, n):
        assert _lib.query("pg_select_workspace_bytes", k) == 2 * a256(4 * k) + a256(8 * max(1, -(-k // 2048))) + 512


def test_library_is_in_tree():
    assert os.path.dirname(_lib.library_path()) == os.path.dirname(os.path.abspath(_build.__file__))


def test_solver_argument_checks_on_host():
    """Size queries and argument checks of the solvers run on the host,
    before any device call: bad shapes return 0 bytes / PG_ERR_ARG."""
    import ctypes

    import numpy as np
    lib = _lib.load()
    P = ctypes.c_void_p
    co = _lib.CocgOpts()
    lib.pg_cocg_default_opts(ctypes.byref(co))
    co.precision = 2
    rows = np.array([0, 10, 30], dtype=np.int64)
    rp = P(rows.ctypes.data)
    ok = lib.pg_cocg_segments_workspace_bytes(30, 300, 4, rp, 2, P(0), ctypes.byref(co))
    assert ok > 0
    bad = np.array([0, 10, 29], dtype=np.int64)          # does not end at n
    assert lib.pg_cocg_segments_workspace_bytes(30, 300, 4, P(bad.ctypes.data), 2, P(0), ctypes.byref(co)) == 0
    down = np.array([0, 20, 10, 30], dtype=np.int64)     # falls
    assert lib.pg_cocg_segments_workspace_bytes(30, 300, 1, P(down.ctypes.data), 3, P(0), ctypes.byref(co)) == 0
    assert lib.pg_cocg_segments_workspace_bytes(30, 300, 3, rp, 2, P(0), ctypes.byref(co)) == 0   # k not 2^i
    # block-Jacobi needs per-system entity counts that add up to each system's rows (p = 2: 2 per edge / face)
    co.block_p = 2
    assert lib.pg_cocg_segments_workspace_bytes(30, 300, 1, rp, 2, P(0), ctypes.byref(co)) == 0
    ents = np.array([3, 2, 0, 5, 5, 0], dtype=np.int64)
    assert lib.pg_cocg_segments_workspace_bytes(30, 300, 1, rp, 2, P(ents.ctypes.data), ctypes.byref(co)) > ok // 4
    ents_bad = np.array([4, 2, 0, 5, 5, 0], dtype=np.int64)
    assert lib.pg_cocg_segments_workspace_bytes(30, 300, 1, rp, 2, P(ents_bad.ctypes.data), ctypes.byref(co)) == 0
    # pg_cocg_segments only runs the double-float form: checked before the device is touched
    co.precision = 0
    res = _lib.GmresResult()
    st = lib.pg_cocg_segments(P(8), P(8), P(8), 30, 300, rp, 2, P(0), P(8), P(8), 1, ctypes.byref(co),
                              ctypes.byref(res), P(0), P(0), P(8), 1 << 20, P(0))
    assert st == -1
    # GMRES block-Jacobi entity counts must add up to n
    go = _lib.GmresOpts()
    lib.pg_gmres_default_opts(ctypes.byref(go))
    plain = lib.pg_gmres_workspace_bytes(30, 300, 1, ctypes.byref(go))
    go.block_p, go.block_edges, go.block_faces, go.block_volumes = 2, 5, 10, 0
    assert lib.pg_gmres_workspace_bytes(30, 300, 1, ctypes.byref(go)) > plain
    go.block_faces = 11
    st = lib.pg_gmres(P(8), P(8), P(8), 30, 300, P(8), P(8), 1, ctypes.byref(go), ctypes.byref(res), P(0), P(8),
                      1 << 30, P(0))
    assert st == -1
