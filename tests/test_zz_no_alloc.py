"""bss_factor_solve_noalloc: the entry point for callers that cannot
allocate device memory (a host runtime whose memory manager owns the device
pool, a fixed-budget server).  It factors and solves in place on the
caller's own buffers with its workspace in the library's static device
array.  Checked through the C ABI against the handle path
(bss_create_batched + bss_factorize + bss_solve) on the same inputs, twice in
a row (the array keeps the previous call's contents), within the tolerances
the other parity tests use.  This file is collected last on purpose."""
import ctypes

import numpy as np
import pytest

from oracle import oracle as O
from tests.gpu_util import download_x, upload

pytestmark = pytest.mark.gpu

TOL = {"f64": 1e-10, "f32": 1e-4}


def _colmajor(a, dt, torch):
    """math blocks (N, r, c) -> contiguous device tensor holding the Julia
    column-major storage (N, c, r) of the same blocks."""
    return torch.from_numpy(np.ascontiguousarray(np.swapaxes(a, 1, 2))).to("cuda", dt).contiguous()


@pytest.mark.parametrize("T", ["f64", "f32"])
def test_noalloc_matches_handle_path_twice(T):
    import torch
    import blockstructuredsolvers_gb300 as bss
    from blockstructuredsolvers_gb300 import _lib
    L = _lib.load()
    dt = torch.float64 if T == "f64" else torch.float32
    code = _lib.BSS_F64 if T == "f64" else _lib.BSS_F32
    for call, (seed, N, n, k) in enumerate([(1, 300, 16, 2), (2, 250, 24, 1)]):
        rng = np.random.default_rng(seed)
        A, B, d = O.gen_shifted_family(rng, N, n, k)
        # existing entry point
        data = bss.initialize_batched(N, n, dt, k=k)
        upload(data, A, B, d)
        bss.factorize_(data)
        bss.solve_(data)
        bss.synchronize(data)
        x_ref = download_x(data, N)
        # the no-allocation entry point on caller-owned buffers
        Ad, Bd, dd = _colmajor(A, dt, torch), _colmajor(B, dt, torch), _colmajor(d, dt, torch)
        torch.cuda.synchronize()
        rc = L.bss_factor_solve_noalloc(N, n, k, code, ctypes.c_void_p(Ad.data_ptr()),
                                        ctypes.c_void_p(Bd.data_ptr()), ctypes.c_void_p(dd.data_ptr()),
                                        ctypes.c_void_p(torch.cuda.current_stream().cuda_stream))
        _lib.check(rc)
        x = np.swapaxes(dd.double().cpu().numpy(), 1, 2)
        err = O.rel_error(x, x_ref)
        assert err <= TOL[T], (call, err)
        assert O.rel_error(x, O.cpu_solve(A, B, d)) <= TOL[T]


def _noalloc(L, _lib, N, n, k, T, A, B, d, torch):
    """one call of the no-allocation entry point on fresh caller-owned
    buffers; B may be None (N = 1) and is then passed as NULL"""
    dt = torch.float64 if T == "f64" else torch.float32
    code = _lib.BSS_F64 if T == "f64" else _lib.BSS_F32
    Ad, dd = _colmajor(A, dt, torch), _colmajor(d, dt, torch)
    Bd = _colmajor(B, dt, torch) if B is not None else None
    torch.cuda.synchronize()
    rc = L.bss_factor_solve_noalloc(N, n, k, code, ctypes.c_void_p(Ad.data_ptr()),
                                    ctypes.c_void_p(Bd.data_ptr() if Bd is not None else None),
                                    ctypes.c_void_p(dd.data_ptr()),
                                    ctypes.c_void_p(torch.cuda.current_stream().cuda_stream))
    _lib.check(rc)
    return np.swapaxes(dd.double().cpu().numpy(), 1, 2)


# paths of the entry point that differ from the two cases above: the wide
# tile-streamed kernels (n > 64; FP32 n <= 128 on the tensor cores), a single
# sequential level (N <= 8), N = 1 with no B buffer, and more right-hand
# sides than one solve pass takes (several column chunks)
@pytest.mark.parametrize("T", ["f64", "f32"])
@pytest.mark.parametrize("seed,N,n,k", [(4, 20, 96, 2), (5, 5, 32, 1), (6, 1, 16, 3), (7, 60, 16, 40)],
                         ids=["wide_n96", "seq_N5", "single_N1", "chunks_k40"])
def test_noalloc_other_paths_twice(T, seed, N, n, k):
    import torch
    import blockstructuredsolvers_gb300 as bss
    from blockstructuredsolvers_gb300 import _lib
    L = _lib.load()
    dt = torch.float64 if T == "f64" else torch.float32
    rng = np.random.default_rng(seed)
    A, B, d = O.gen_shifted_family(rng, N, n, k, diag_shift=2.0 * n, b_scale=0.5)
    data = bss.initialize_batched(N, n, dt, k=k)
    upload(data, A, B, d)
    bss.factorize_(data)
    bss.solve_(data)
    bss.synchronize(data)
    x_ref = download_x(data, N)
    x_cpu = O.cpu_solve(A, B, d)
    for call in range(2):  # the second call runs on the array the first one left behind
        x = _noalloc(L, _lib, N, n, k, T, A, B if N > 1 else None, d, torch)
        assert O.rel_error(x, x_ref) <= TOL[T], (call, O.rel_error(x, x_ref))
        assert O.rel_error(x, x_cpu) <= TOL[T]


def test_noalloc_rejects_out_of_range_sizes():
    """sizes that would not survive the narrowing to the kernels' int
    arguments are rejected before anything runs"""
    import torch
    from blockstructuredsolvers_gb300 import _lib
    L = _lib.load()
    s = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    buf = torch.zeros(16, dtype=torch.float64, device="cuda")
    p = ctypes.c_void_p(buf.data_ptr())
    assert L.bss_factor_solve_noalloc(4, (1 << 32) + 16, 1, _lib.BSS_F64, p, p, p, s) != _lib.BSS_OK
    assert L.bss_factor_solve_noalloc(4, 16, (1 << 31) + 1, _lib.BSS_F64, p, p, p, s) == _lib.BSS_ERR_ARG
    assert L.bss_factor_solve_noalloc(1 << 41, 16, 1, _lib.BSS_F64, p, p, p, s) == _lib.BSS_ERR_ARG
    assert torch.count_nonzero(buf).item() == 0


def test_noalloc_rejects_oversize_and_reports_not_spd():
    import torch
    from blockstructuredsolvers_gb300 import _lib
    L = _lib.load()
    s = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    # workspace of N=100000, n=64 far exceeds the static array: rejected before any work
    big = torch.zeros(16, dtype=torch.float64, device="cuda")
    p = ctypes.c_void_p(big.data_ptr())
    rc = L.bss_factor_solve_noalloc(100000, 64, 1, _lib.BSS_F64, p, p, p, s)
    assert rc == _lib.BSS_ERR_ARG
    assert b"workspace" in L.bss_last_error_string()
    assert torch.count_nonzero(big).item() == 0
    # a non-SPD block is reported
    rng = np.random.default_rng(3)
    A, B, d = O.gen_shifted_family(rng, 60, 8, 1)
    A[17] = -A[17]
    Ad, Bd, dd = (_colmajor(a, torch.float64, torch) for a in (A, B, d))
    rc = L.bss_factor_solve_noalloc(60, 8, 1, _lib.BSS_F64, ctypes.c_void_p(Ad.data_ptr()),
                                    ctypes.c_void_p(Bd.data_ptr()), ctypes.c_void_p(dd.data_ptr()), s)
    assert rc == _lib.BSS_ERR_NOT_SPD
