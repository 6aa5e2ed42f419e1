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
