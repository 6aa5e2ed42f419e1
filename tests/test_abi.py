"""CPU tests of the C ABI library (no compute calls that need a GPU):
the library loads, exports every entry point include/bss.h declares, its
host-side planner is bit-exact with the reference planner restatement, and
argument/GPU errors come back as status codes."""
import ctypes
import os
import re

import pytest

from oracle import oracle as O

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def lib():
    from blockstructuredsolvers_gb300 import _lib, build
    if not os.path.exists(_lib.LIB_PATH):
        build.build()
    return _lib.load()


def _declared():
    src = open(os.path.join(ROOT, "include", "bss.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(bss_[a-z0-9_]+)\s*\(", src)))


def test_header_declares_core_entry_points():
    names = _declared()
    for need in ("bss_create_batched", "bss_factorize", "bss_solve", "bss_destroy", "bss_create_seq"):
        assert need in names


def test_library_exports_every_declared_symbol(lib):
    from blockstructuredsolvers_gb300 import _lib
    for name in _declared():
        assert hasattr(lib, name), name
    assert set(_lib.EXPORTS) == set(_declared())


def test_version_string(lib):
    assert b"sm_103a" in lib.bss_version()


def test_default_options(lib):
    from blockstructuredsolvers_gb300 import _lib
    o = _lib.default_options()
    assert o.precision == _lib.BSS_PRECISION_PLAIN and o.plan == _lib.BSS_PLAN_AUTO
    assert o.max_refine == 10 and abs(o.tol - 1e-12) < 1e-30


def test_plan_reference_bit_exact(lib):
    from blockstructuredsolvers_gb300 import _lib
    for N in list(range(1, 2500)) + [5000, 16384, 65536, 100003]:
        got = _lib.plan_reference(N)
        want = O.reference_plan(N)
        assert got == (list(want[0]), want[1]), N


def test_argument_errors(lib):
    from blockstructuredsolvers_gb300 import _lib
    h = ctypes.c_void_p()
    assert lib.bss_create_batched(0, 4, 1, _lib.BSS_F64, None, None, ctypes.byref(h)) == _lib.BSS_ERR_ARG
    assert lib.bss_create_batched(10, 4, 0, _lib.BSS_F64, None, None, ctypes.byref(h)) == _lib.BSS_ERR_ARG
    assert lib.bss_create_batched(10, 4, 1, 7, None, None, ctypes.byref(h)) == _lib.BSS_ERR_ARG
    assert lib.bss_create_batched(10, 4000, 1, _lib.BSS_F64, None, None,
                                  ctypes.byref(h)) == _lib.BSS_ERR_UNSUPPORTED
    o = _lib.default_options()
    o.precision = _lib.BSS_PRECISION_MIXED
    assert lib.bss_create_batched(10, 4, 1, _lib.BSS_F32, None, ctypes.byref(o),
                                  ctypes.byref(h)) == _lib.BSS_ERR_ARG
    assert b"mixed" in lib.bss_last_error_string()
    assert lib.bss_factorize(None) == _lib.BSS_ERR_ARG
    assert lib.bss_solve(None) == _lib.BSS_ERR_ARG


def test_no_gpu_is_an_error_not_a_fallback(lib):
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    from blockstructuredsolvers_gb300 import _lib
    h = ctypes.c_void_p()
    rc = lib.bss_create_batched(50, 8, 1, _lib.BSS_F64, None, None, ctypes.byref(h))
    assert rc in (_lib.BSS_ERR_CUDA, _lib.BSS_ERR_OOM)
    assert not h.value


def test_csr_nnz_host_only():
    """bss_csr_nnz is host arithmetic (no GPU needed): n^2 (3N - 2) entries,
    -1 for empty shapes."""
    from blockstructuredsolvers_gb300 import _lib
    L = _lib.load()
    for N, n in [(1, 4), (2, 3), (16384, 64), (100, 32)]:
        assert L.bss_csr_nnz(N, n) == n * n * (3 * N - 2)
    assert L.bss_csr_nnz(0, 4) == -1 and L.bss_csr_nnz(4, 0) == -1
