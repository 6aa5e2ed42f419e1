"""The mixed-precision refinement's residual r = d - T x, computed in
double-float on the FP32 pipe (residual_df_kernel), against an FP64 numpy
residual of the same inputs: elementwise |r - r_np| <= tol (|d| + |T| |x|)
with tol = 2^-42 (measured up to 2^-44.2; FP64 kernel: 2^-48), over block sizes, right-hand-side
counts, signs, zero blocks and magnitudes spread over 2^-30 .. 2^30."""
import ctypes

import numpy as np
import pytest

from oracle import oracle as O

pytestmark = pytest.mark.gpu


def _system(N, n, k, seed):
    rng = np.random.default_rng(seed)
    scale = 2.0 ** rng.integers(-30, 31, size=N)
    A = rng.standard_normal((N, n, n)) * scale[:, None, None]
    B = rng.standard_normal((max(N - 1, 0), n, n)) * scale[:max(N - 1, 0), None, None]
    if N > 3:
        B[1] = 0.0
    x = rng.standard_normal((N, n, k)) * 2.0 ** rng.integers(-10, 11, size=(N, 1, k))
    x[0, 0, 0] = 0.0
    d = O.block_matvec(A, B, x) + rng.standard_normal((N, n, k)) * 1e-9 * np.abs(O.block_matvec(A, B, x)).max()
    return A, B, x, d


def _run(method, A, B, x, d):
    import torch
    from blockstructuredsolvers_gb300 import _lib
    N, n, _ = A.shape
    k = x.shape[2]
    dev = torch.device("cuda")
    cm = lambda v: torch.from_numpy(np.ascontiguousarray(np.swapaxes(v, 1, 2))).to(dev)  # column-major blocks
    At, Bt, xt, dt = cm(A), cm(B) if N > 1 else torch.zeros(1, device=dev, dtype=torch.float64), cm(x), cm(d)
    rt = torch.empty_like(dt)
    L = _lib.load()
    s = ctypes.c_void_p(int(torch.cuda.current_stream().cuda_stream))
    _lib.check(L.bss_diag_residual(N, n, k, method, ctypes.c_void_p(At.data_ptr()), ctypes.c_void_p(Bt.data_ptr()),
                                   ctypes.c_void_p(xt.data_ptr()), ctypes.c_void_p(dt.data_ptr()),
                                   ctypes.c_void_p(rt.data_ptr()), s))
    return np.swapaxes(rt.cpu().numpy(), 1, 2)


@pytest.mark.parametrize("N,n,k", [(1, 16, 1), (2, 64, 1), (37, 64, 3), (300, 64, 1), (50, 128, 2), (20, 16, 5),
                                   (64, 32, 4), (9, 48, 8), (40, 96, 1), (11, 8, 16), (33, 128, 4),
                                   (12, 128, 8), (25, 96, 4)])
def test_double_float_residual_matches_fp64(N, n, k):
    A, B, x, d = _system(N, n, k, seed=N * 1000 + n * 10 + k)
    r_np = d - O.block_matvec(A, B, x)
    bound = np.abs(d) + O.block_matvec(np.abs(A), np.abs(B), np.abs(x))
    r_df = _run(1, A, B, x, d)
    r_64 = _run(0, A, B, x, d)
    err_df = (np.abs(r_df - r_np) / bound).max()
    err_64 = (np.abs(r_64 - r_np) / bound).max()
    print(f"N={N} n={n} k={k}: max err/bound double-float {err_df:.3e} (2^{np.log2(max(err_df, 1e-300)):.1f}), "
          f"fp64 {err_64:.3e}")
    assert err_64 <= 2.0 ** -48
    assert err_df <= 2.0 ** -42
