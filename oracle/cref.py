"""ctypes driver for the C oracle (``oracle/bss_oracle.c``).

TEST INFRASTRUCTURE ONLY: used by tests/ to check results and by bench.py as the
timed CPU baseline (BlockStructuredSolvers.jl src/cpu.jl:30-50 ->
src/backbone_cpu.jl:5-33 restated in C).  Builds into ``oracle/_build/``.

LAPACK/BLAS: the function pointers of scipy.linalg.cython_lapack /
cython_blas (dpotrf/dtrsm/dgemm, spotrf/strsm/sgemm), which wrap the OpenBLAS
that scipy ships, are registered with the C code.  This mirrors the reference,
whose CPU path calls OpenBLAS through Julia's LinearAlgebra.
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD = os.path.join(HERE, "_build")
SO = os.path.join(BUILD, "libbss_oracle.so")
SRC = os.path.join(HERE, "bss_oracle.c")

_lib = None


def build(force: bool = False) -> str:
    os.makedirs(BUILD, exist_ok=True)
    if force or not os.path.exists(SO) or os.path.getmtime(SO) < os.path.getmtime(SRC):
        tmp = SO + ".tmp%d" % os.getpid()
        subprocess.check_call(["gcc", "-O2", "-fPIC", "-shared", "-o", tmp, SRC, "-lm", "-lpthread"])
        os.replace(tmp, SO)
    return SO


def _capsule_ptr(mod, name):
    cap = mod.__pyx_capi__[name]
    get_name = ctypes.pythonapi.PyCapsule_GetName
    get_name.restype = ctypes.c_char_p
    get_name.argtypes = [ctypes.py_object]
    get_ptr = ctypes.pythonapi.PyCapsule_GetPointer
    get_ptr.restype = ctypes.c_void_p
    get_ptr.argtypes = [ctypes.py_object, ctypes.c_char_p]
    return get_ptr(cap, get_name(cap))


def lib(use_blas: bool = True):
    """Load (building if needed) the oracle library; registers scipy's
    LAPACK/BLAS unless ``use_blas`` is False (plain C loops then)."""
    global _lib
    if _lib is None:
        L = ctypes.CDLL(build())
        dp = ctypes.POINTER(ctypes.c_double)
        fp = ctypes.POINTER(ctypes.c_float)
        L.bsso_set_blas.argtypes = [ctypes.c_void_p] * 6
        L.bsso_factorize_d.argtypes = [ctypes.c_int64, ctypes.c_int, dp, dp]
        L.bsso_factorize_d.restype = ctypes.c_int64
        L.bsso_solve_d.argtypes = [ctypes.c_int64, ctypes.c_int, ctypes.c_int, dp, dp, dp]
        L.bsso_factorize_s.argtypes = [ctypes.c_int64, ctypes.c_int, fp, fp]
        L.bsso_factorize_s.restype = ctypes.c_int64
        L.bsso_solve_s.argtypes = [ctypes.c_int64, ctypes.c_int, ctypes.c_int, fp, fp, fp]
        L.bsso_solve_many_d.argtypes = [ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p,
                                        ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
                                        ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int]
        _lib = L
    if use_blas:
        import scipy.linalg.cython_blas as cb
        import scipy.linalg.cython_lapack as cl
        _lib.bsso_set_blas(_capsule_ptr(cl, "dpotrf"), _capsule_ptr(cb, "dtrsm"),
                           _capsule_ptr(cb, "dgemm"), _capsule_ptr(cl, "spotrf"),
                           _capsule_ptr(cb, "strsm"), _capsule_ptr(cb, "sgemm"))
    else:
        _lib.bsso_set_blas(None, None, None, None, None, None)
    return _lib


def blas_backend_name() -> str:
    try:
        import scipy
        cfg = scipy.show_config(mode="dicts")
        return str(cfg["Build Dependencies"]["blas"]["name"])
    except Exception:  # pragma: no cover
        return "unknown"


def set_blas_threads(nthreads: int) -> bool:
    """Best-effort: set the thread count of scipy's bundled OpenBLAS."""
    try:
        import scipy
        libdir = os.path.join(os.path.dirname(os.path.dirname(scipy.__file__)), "scipy.libs")
        for f in sorted(os.listdir(libdir)):
            if "openblas" in f:
                L = ctypes.CDLL(os.path.join(libdir, f))
                for sym in ("scipy_openblas_set_num_threads64_", "scipy_openblas_set_num_threads",
                            "openblas_set_num_threads64_", "openblas_set_num_threads"):
                    fn = getattr(L, sym, None)
                    if fn is not None:
                        fn.argtypes = [ctypes.c_int]
                        fn(int(nthreads))
                        return True
    except Exception:
        pass
    return False


def solve(A_stor: np.ndarray, B_stor: np.ndarray, d_stor: np.ndarray, use_blas: bool = True):
    """factorize! + solve! (cpu.jl) in place on Julia-column-major storage
    arrays: A (N,n,n), B (N-1,n,n), d (N,k,n).  dtype float64 or float32.
    Returns the 1-based index of the first non-SPD block, or 0."""
    L = lib(use_blas)
    N, n, _ = A_stor.shape
    k = d_stor.shape[1]
    assert A_stor.flags.c_contiguous and B_stor.flags.c_contiguous and d_stor.flags.c_contiguous
    if A_stor.dtype == np.float64:
        p = ctypes.POINTER(ctypes.c_double)
        fac, sol = L.bsso_factorize_d, L.bsso_solve_d
    else:
        p = ctypes.POINTER(ctypes.c_float)
        fac, sol = L.bsso_factorize_s, L.bsso_solve_s
    Bp = B_stor.ctypes.data_as(p) if B_stor.size else A_stor.ctypes.data_as(p)
    info = fac(N, n, A_stor.ctypes.data_as(p), Bp)
    if info:
        return int(info)
    sol(N, n, k, A_stor.ctypes.data_as(p), Bp, d_stor.ctypes.data_as(p))
    return 0


def solve_math(A, B, d, dtype=np.float64, use_blas: bool = True):
    """Convenience on math blocks (N,n,n), (N-1,n,n), (N,n,k); returns x (N,n,k)."""
    from oracle.oracle import from_storage, to_storage
    As = to_storage(np.asarray(A, dtype))
    Bs = to_storage(np.asarray(B, dtype)) if len(B) else np.zeros((0, A.shape[1], A.shape[1]), dtype)
    ds = to_storage(np.asarray(d, dtype))
    info = solve(As, Bs, ds, use_blas)
    if info:
        raise np.linalg.LinAlgError(f"block {info} not SPD")
    return from_storage(ds)


def solve_many(systems, nthreads: int):
    """Independent systems [(A_stor, B_stor, d_stor), ...] (float64, Julia
    storage), factor+solve in place with ``nthreads`` workers."""
    L = lib(True)
    ns = len(systems)
    Ns = np.array([s[0].shape[0] for s in systems], np.int64)
    nsz = np.array([s[0].shape[1] for s in systems], np.int32)
    ks = np.array([s[2].shape[1] for s in systems], np.int32)
    Ap = (ctypes.c_void_p * ns)(*[s[0].ctypes.data for s in systems])
    Bp = (ctypes.c_void_p * ns)(*[(s[1].ctypes.data if s[1].size else s[0].ctypes.data) for s in systems])
    dp = (ctypes.c_void_p * ns)(*[s[2].ctypes.data for s in systems])
    info = np.zeros(ns, np.int64)
    L.bsso_solve_many_d(ns, Ns.ctypes.data, nsz.ctypes.data, ks.ctypes.data, ctypes.addressof(Ap),
                        ctypes.addressof(Bp), ctypes.addressof(dp), info.ctypes.data, int(nthreads))
    return info
