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
    assert lib.pg_abi_version() == 2
    assert _lib.query("pg_table_doubles", 2) == 12 * 20 * 21 // 2
    assert _lib.query("pg_table_doubles", 7) == 0
    assert _lib.query("pg_pattern_local_entities", 1) == 6
    assert _lib.query("pg_pattern_local_entities", 3) == 11
    o = _lib.GmresOpts()
    lib.pg_gmres_default_opts(o)
    assert o.restart == 30 and abs(o.rtol - 1e-8) < 1e-20 and o.precision == 0


def test_library_is_in_tree():
    assert os.path.dirname(_lib.library_path()) == os.path.dirname(os.path.abspath(_build.__file__))
