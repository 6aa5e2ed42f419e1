"""ctypes binding of the C ABI declared in ``include/bss.h``.

The library is the in-tree ``libbss_gb300.so`` built by ``build.py`` for
sm_103a.  There is no fallback: if the library is missing or fails to load,
``load()`` raises.
"""
from __future__ import annotations

import ctypes
import os

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libbss_gb300.so")

BSS_OK = 0
BSS_FACTOR_FMA_CHAIN = 1
BSS_FACTOR_WIDE_L2 = 2
BSS_UPLOAD_FULL = 0
BSS_UPLOAD_UPPER = 1
BSS_ERR_ARG = 1
BSS_ERR_OOM = 2
BSS_ERR_CUDA = 3
BSS_ERR_NOT_SPD = 4
BSS_ERR_TIMEOUT = 5
BSS_ERR_UNSUPPORTED = 6
BSS_ERR_STATE = 7
BSS_ERR_NOT_CONVERGED = 8

BSS_F32 = 0
BSS_F64 = 1
BSS_PRECISION_PLAIN = 0
BSS_PRECISION_MIXED = 1
BSS_PLAN_AUTO = 0
BSS_PLAN_REFERENCE = 1
BSS_NOALLOC_SCRATCH_BYTES = 8 << 20

# every entry point include/bss.h declares
EXPORTS = (
    "bss_default_options", "bss_create_batched", "bss_create_seq", "bss_destroy",
    "bss_get_tensors", "bss_get_dims", "bss_upload", "bss_download", "bss_factorize", "bss_solve", "bss_synchronize",
    "bss_get_info", "bss_last_error_string", "bss_plan_reference", "bss_residual",
    "bss_factorize_levels", "bss_get_level", "bss_factor_solve_noalloc", "bss_kernel_launches",
    "bss_version", "bss_batch_create", "bss_batch_destroy", "bss_batch_get_tensors", "bss_batch_get_dims",
    "bss_batch_factorize", "bss_batch_solve", "bss_batch_synchronize", "bss_batch_get_info",
    "bss_kf_build", "bss_server_default_options", "bss_server_create", "bss_server_destroy", "bss_server_submit",
    "bss_server_submit_kalman", "bss_server_submit_rhs", "bss_server_wait", "bss_server_poll",
    "bss_server_release", "bss_server_get_stats", "bss_server_reset_stats",
    "bss_autotune", "bss_autotune_lookup", "bss_autotune_clear", "bss_autotune_save", "bss_autotune_load",
    "bss_cpu_create", "bss_cpu_destroy", "bss_cpu_get_tensors", "bss_cpu_factorize", "bss_cpu_solve",
    "bss_cpu_failed_block", "bss_tc_selftest", "bss_diag_wide_occupancy", "bss_diag_residual",
    "bss_diag_wait_timeout", "bss_diag_fma_peak", "bss_diag_set_factor_variant", "bss_diag_get_factor_variant",
    "bss_refalgo_create", "bss_refalgo_destroy", "bss_refalgo_get_tensors", "bss_refalgo_get_dims",
    "bss_refalgo_factorize", "bss_refalgo_solve",
    "bss_csr_nnz", "bss_csr_assemble", "bss_spchol_create", "bss_spchol_destroy", "bss_spchol_get_tensors",
    "bss_spchol_get_csr", "bss_spchol_get_dims", "bss_spchol_analyze", "bss_spchol_factorize", "bss_spchol_solve",
)


class Options(ctypes.Structure):
    _fields_ = [
        ("precision", ctypes.c_int32),
        ("plan", ctypes.c_int32),
        ("max_refine", ctypes.c_int32),
        ("target_partitions", ctypes.c_int32),
        ("seq_cutoff", ctypes.c_int32),
        ("use_graphs", ctypes.c_int32),
        ("tol", ctypes.c_double),
        ("chain_blocks", ctypes.c_int32),
        ("coarsest_fp64", ctypes.c_int32),
    ]


class ServerOptions(ctypes.Structure):
    _fields_ = [
        ("hbm_budget_bytes", ctypes.c_int64),
        ("streams", ctypes.c_int32),
        ("max_inflight", ctypes.c_int32),
        ("precision", ctypes.c_int32),
        ("max_refine", ctypes.c_int32),
        ("tol", ctypes.c_double),
    ]


class RequestInfo(ctypes.Structure):
    _fields_ = [
        ("status", ctypes.c_int32),
        ("refine_steps", ctypes.c_int32),
        ("rel_residual", ctypes.c_double),
        ("latency_ms", ctypes.c_double),
        ("queue_ms", ctypes.c_double),
        ("factor_id", ctypes.c_uint64),
    ]


class ServerStats(ctypes.Structure):
    _fields_ = [
        ("submitted", ctypes.c_int64),
        ("completed", ctypes.c_int64),
        ("failed", ctypes.c_int64),
        ("evictions", ctypes.c_int64),
        ("resident_factors", ctypes.c_int64),
        ("bytes_in_use", ctypes.c_int64),
        ("bytes_peak", ctypes.c_int64),
        ("p50_ms", ctypes.c_double),
        ("p99_ms", ctypes.c_double),
        ("mean_ms", ctypes.c_double),
        ("max_ms", ctypes.c_double),
        ("busy_s", ctypes.c_double),
    ]


class TuneEntry(ctypes.Structure):
    _fields_ = [
        ("n", ctypes.c_int32),
        ("dtype", ctypes.c_int32),
        ("precision", ctypes.c_int32),
        ("wave_mult_x4", ctypes.c_int32),
        ("seq_cutoff", ctypes.c_int32),
        ("chain_blocks", ctypes.c_int32),
        ("single_ms", ctypes.c_double),
        ("batch_ms", ctypes.c_double),
        ("factor_variant", ctypes.c_int32),
    ]


class Info(ctypes.Structure):
    _fields_ = [
        ("failed_block", ctypes.c_int64),
        ("failed_level", ctypes.c_int32),
        ("refine_steps", ctypes.c_int32),
        ("rel_residual", ctypes.c_double),
        ("levels", ctypes.c_int32),
        ("coarsest_blocks", ctypes.c_int64),
    ]


class BSSError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"[bss error {code}] {msg}")
        self.code = code


class NotSPDError(BSSError):
    pass


_lib = None


def load(path: str | None = None):
    """Load libbss_gb300.so (raises OSError when it is not built)."""
    global _lib
    if _lib is not None and path is None:
        return _lib
    p = path or LIB_PATH
    if not os.path.exists(p):
        raise OSError(f"{p} not found: run blockstructuredsolvers_gb300/build.py (or __graft_entry__.build())")
    L = ctypes.CDLL(p)
    vp = ctypes.c_void_p
    i64 = ctypes.c_int64
    i32 = ctypes.c_int32
    L.bss_default_options.argtypes = [ctypes.POINTER(Options)]
    L.bss_default_options.restype = None
    L.bss_create_batched.argtypes = [i64, i64, i64, i32, vp, ctypes.POINTER(Options), ctypes.POINTER(vp)]
    L.bss_create_seq.argtypes = [i64, i64, i64, i32, vp, ctypes.POINTER(vp)]
    L.bss_destroy.argtypes = [vp]
    L.bss_get_tensors.argtypes = [vp, ctypes.POINTER(vp), ctypes.POINTER(vp), ctypes.POINTER(vp)]
    L.bss_get_dims.argtypes = [vp, ctypes.POINTER(i64), ctypes.POINTER(i64), ctypes.POINTER(i64),
                               ctypes.POINTER(i32)]
    L.bss_upload.argtypes = [vp, vp, vp, vp, i32, ctypes.POINTER(i64)]
    L.bss_download.argtypes = [vp, vp]
    L.bss_factorize.argtypes = [vp]
    L.bss_solve.argtypes = [vp]
    L.bss_synchronize.argtypes = [vp]
    L.bss_get_info.argtypes = [vp, ctypes.POINTER(Info)]
    L.bss_last_error_string.argtypes = []
    L.bss_last_error_string.restype = ctypes.c_char_p
    L.bss_plan_reference.argtypes = [i64, ctypes.POINTER(i64), i32, ctypes.POINTER(i32), ctypes.POINTER(i64)]
    L.bss_residual.argtypes = [i64, i64, i64, i32, vp, vp, vp, vp, vp, ctypes.POINTER(ctypes.c_double)]
    L.bss_factorize_levels.argtypes = [vp, i32]
    L.bss_get_level.argtypes = [vp, i32, ctypes.POINTER(i64), ctypes.POINTER(i64), ctypes.POINTER(vp),
                                ctypes.POINTER(vp), ctypes.POINTER(vp), ctypes.POINTER(i32)]
    L.bss_factor_solve_noalloc.argtypes = [i64, i64, i64, i32, vp, vp, vp, vp]
    L.bss_kernel_launches.argtypes = []
    L.bss_kernel_launches.restype = ctypes.c_int64
    L.bss_version.argtypes = []
    L.bss_version.restype = ctypes.c_char_p
    pi64 = ctypes.POINTER(i64)
    L.bss_batch_create.argtypes = [i32, pi64, pi64, pi64, i32, vp, ctypes.POINTER(Options), ctypes.POINTER(vp)]
    L.bss_batch_destroy.argtypes = [vp]
    L.bss_batch_get_tensors.argtypes = [vp, i32, ctypes.POINTER(vp), ctypes.POINTER(vp), ctypes.POINTER(vp)]
    L.bss_batch_get_dims.argtypes = [vp, i32, pi64, pi64, pi64]
    L.bss_batch_factorize.argtypes = [vp]
    L.bss_batch_solve.argtypes = [vp]
    L.bss_batch_synchronize.argtypes = [vp]
    L.bss_batch_get_info.argtypes = [vp, i32, ctypes.POINTER(Info)]
    L.bss_kf_build.argtypes = [i64, i64, i64, i64] + [vp] * 10 + [vp]
    L.bss_server_default_options.argtypes = [ctypes.POINTER(ServerOptions)]
    L.bss_server_default_options.restype = None
    u64 = ctypes.c_uint64
    pu64 = ctypes.POINTER(u64)
    L.bss_server_create.argtypes = [ctypes.POINTER(ServerOptions), ctypes.POINTER(vp)]
    L.bss_server_destroy.argtypes = [vp]
    L.bss_server_submit.argtypes = [vp, i64, i64, i64, vp, vp, vp, i32, vp, pu64, pu64]
    L.bss_server_submit_kalman.argtypes = [vp, i64, i64, i64, i64, vp, vp, vp, vp, vp, vp, vp, i32, vp, pu64, pu64]
    L.bss_server_submit_rhs.argtypes = [vp, u64, vp, vp, pu64]
    L.bss_server_wait.argtypes = [vp, u64, ctypes.POINTER(RequestInfo)]
    L.bss_server_poll.argtypes = [vp, u64, ctypes.POINTER(i32)]
    L.bss_server_release.argtypes = [vp, u64]
    L.bss_server_get_stats.argtypes = [vp, ctypes.POINTER(ServerStats)]
    L.bss_server_reset_stats.argtypes = [vp]
    L.bss_autotune.argtypes = [i64, i32, i32, i64, ctypes.POINTER(TuneEntry)]
    L.bss_autotune_lookup.argtypes = [i64, i32, i32, ctypes.POINTER(TuneEntry)]
    L.bss_autotune_clear.argtypes = []
    L.bss_autotune_clear.restype = None
    L.bss_autotune_save.argtypes = [ctypes.c_char_p]
    L.bss_autotune_load.argtypes = [ctypes.c_char_p]
    L.bss_cpu_create.argtypes = [i64, i64, i64, i32, ctypes.POINTER(vp)]
    L.bss_cpu_destroy.argtypes = [vp]
    L.bss_cpu_get_tensors.argtypes = [vp, ctypes.POINTER(vp), ctypes.POINTER(vp), ctypes.POINTER(vp)]
    L.bss_cpu_factorize.argtypes = [vp]
    L.bss_cpu_solve.argtypes = [vp]
    L.bss_cpu_failed_block.argtypes = [vp, ctypes.POINTER(i64)]
    L.bss_tc_selftest.argtypes = [i64, ctypes.POINTER(ctypes.c_double)]
    L.bss_diag_wide_occupancy.argtypes = [ctypes.POINTER(i64)]
    L.bss_diag_residual.argtypes = [i64, i64, i64, i32, vp, vp, vp, vp, vp, vp]
    L.bss_diag_wait_timeout.argtypes = [i64, ctypes.POINTER(i64), ctypes.POINTER(i64)]
    L.bss_diag_fma_peak.argtypes = [i32, ctypes.POINTER(ctypes.c_double)]
    L.bss_diag_set_factor_variant.argtypes = [i32]
    L.bss_diag_get_factor_variant.argtypes = []
    L.bss_diag_get_factor_variant.restype = i32
    L.bss_refalgo_create.argtypes = [i64, i64, i64, i32, vp, ctypes.POINTER(vp)]
    L.bss_refalgo_destroy.argtypes = [vp]
    L.bss_refalgo_get_tensors.argtypes = [vp, ctypes.POINTER(vp), ctypes.POINTER(vp), ctypes.POINTER(vp)]
    L.bss_refalgo_get_dims.argtypes = [vp, ctypes.POINTER(i64), ctypes.POINTER(i64), ctypes.POINTER(i64)]
    L.bss_refalgo_factorize.argtypes = [vp]
    L.bss_refalgo_solve.argtypes = [vp]
    L.bss_csr_nnz.argtypes = [i64, i64]
    L.bss_csr_nnz.restype = i64
    L.bss_csr_assemble.argtypes = [i64, i64, i32, vp, vp, vp, vp, vp, vp]
    L.bss_spchol_create.argtypes = [i64, i64, i64, i32, vp, ctypes.POINTER(vp)]
    L.bss_spchol_destroy.argtypes = [vp]
    L.bss_spchol_get_tensors.argtypes = [vp, ctypes.POINTER(vp), ctypes.POINTER(vp), ctypes.POINTER(vp)]
    L.bss_spchol_get_csr.argtypes = [vp, ctypes.POINTER(vp), ctypes.POINTER(vp), ctypes.POINTER(vp),
                                     ctypes.POINTER(i64)]
    L.bss_spchol_get_dims.argtypes = [vp, ctypes.POINTER(i64), ctypes.POINTER(i64), ctypes.POINTER(i64)]
    L.bss_spchol_analyze.argtypes = [vp]
    L.bss_spchol_factorize.argtypes = [vp]
    L.bss_spchol_solve.argtypes = [vp]
    for name in EXPORTS:
        if name not in ("bss_default_options", "bss_last_error_string", "bss_version", "bss_kernel_launches",
                        "bss_server_default_options", "bss_autotune_clear", "bss_csr_nnz"):
            getattr(L, name).restype = ctypes.c_int
    if path is None:
        _lib = L
    return L


def check(code: int) -> None:
    if code != BSS_OK:
        msg = load().bss_last_error_string().decode(errors="replace")
        if code == BSS_ERR_NOT_SPD:
            raise NotSPDError(code, msg)
        raise BSSError(code, msg)


def default_options() -> Options:
    o = Options()
    load().bss_default_options(ctypes.byref(o))
    return o


def plan_reference(N: int):
    """bss_plan_reference -> ([(N_l, m_l, P_l) finest first], coarsest)."""
    L = load()
    buf = (ctypes.c_int64 * 192)()
    nlev = ctypes.c_int32()
    coarse = ctypes.c_int64()
    check(L.bss_plan_reference(int(N), buf, 64, ctypes.byref(nlev), ctypes.byref(coarse)))
    return [(buf[3 * i], buf[3 * i + 1], buf[3 * i + 2]) for i in range(nlev.value)], coarse.value
