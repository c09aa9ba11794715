"""Build oracle/_ref/libpg_cpu.so (test / measurement infrastructure): the
CPU baselines of the Krylov solve, COCG (oracle/csrc/cpu_cocg.c) and petgem's
restarted GMRES(m) + Jacobi (oracle/csrc/cpu_gmres.c), gcc -O3 -fopenmp,
plain C11 (no architecture-specific flags, so it builds on x86_64 and
aarch64 alike)."""
import os
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
SRCS = [os.path.join(HERE, "csrc", f) for f in ("cpu_cocg.c", "cpu_gmres.c")]
OUT = os.path.join(HERE, "_ref", "libpg_cpu.so")


def build(force=False):
    os.makedirs(os.path.dirname(OUT), exist_ok=True)
    if not force and os.path.exists(OUT) and all(os.path.getmtime(OUT) >= os.path.getmtime(s) for s in SRCS):
        return OUT
    cmd = ["gcc", "-O3", "-std=c11", "-fopenmp", "-fPIC", "-shared", *SRCS, "-o", OUT, "-lm"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("gcc failed for the CPU baseline solvers:\n" + r.stderr)
    return OUT


def load():
    import ctypes
    lib = ctypes.CDLL(build())
    P, I64, D = ctypes.c_void_p, ctypes.c_int64, ctypes.c_double
    lib.pg_cpu_cocg.restype = ctypes.c_int
    lib.pg_cpu_cocg.argtypes = [I64, P, P, P, P, P, I64, D, P, P]
    lib.pg_cpu_gmres.restype = ctypes.c_int
    lib.pg_cpu_gmres.argtypes = [I64, P, P, P, P, P, ctypes.c_int, I64, D, ctypes.c_int, P, P]
    return lib


def cocg(rowptr, col, vals, b, max_it, rtol):
    """(x, iterations, relres, status) of the CPU COCG on numpy CSR arrays."""
    import ctypes
    import numpy as np
    lib = load()
    rowptr = np.ascontiguousarray(rowptr, dtype=np.int64)
    col = np.ascontiguousarray(col, dtype=np.int32)
    vals = np.ascontiguousarray(vals, dtype=np.complex128)
    b = np.ascontiguousarray(b, dtype=np.complex128)
    x = np.zeros_like(b)
    its = ctypes.c_int64(0)
    rel = ctypes.c_double(0.0)
    st = lib.pg_cpu_cocg(len(b), rowptr.ctypes.data, col.ctypes.data, vals.ctypes.data, b.ctypes.data,
                         x.ctypes.data, int(max_it), float(rtol), ctypes.byref(its), ctypes.byref(rel))
    return x, int(its.value), float(rel.value), int(st)


def gmres(rowptr, col, vals, b, restart, max_it, rtol, reorth=False):
    """(x, iterations, relres, status) of the CPU GMRES(restart) + Jacobi on
    numpy CSR arrays (status 0 converged, 1 max_it, 2 breakdown)."""
    import ctypes
    import numpy as np
    lib = load()
    rowptr = np.ascontiguousarray(rowptr, dtype=np.int64)
    col = np.ascontiguousarray(col, dtype=np.int32)
    vals = np.ascontiguousarray(vals, dtype=np.complex128)
    b = np.ascontiguousarray(b, dtype=np.complex128)
    x = np.zeros_like(b)
    its = ctypes.c_int64(0)
    rel = ctypes.c_double(0.0)
    st = lib.pg_cpu_gmres(len(b), rowptr.ctypes.data, col.ctypes.data, vals.ctypes.data, b.ctypes.data,
                          x.ctypes.data, int(restart), int(max_it), float(rtol), int(bool(reorth)),
                          ctypes.byref(its), ctypes.byref(rel))
    return x, int(its.value), float(rel.value), int(st)
