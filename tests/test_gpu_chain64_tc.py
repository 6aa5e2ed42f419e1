"""The two chain kernels of FP32 factors for 64-wide blocks (33 <= n <= 64:
plain FP32 and every level of the mixed path): the tensor-core kernel
(tcgen05 3xTF32 products; bulk-copied block tiles for even n, plain loads
for odd n, whose blocks are not a multiple of 16 bytes) and the CUDA-core
kernel.  Each is checked against the CPU oracle (<= 1e-4 relative error in
FP32; rel-resid <= 1e-12 and <= 1e-10 error in mixed precision), and their
first-level separator systems against each other."""
import numpy as np
import pytest

from oracle import oracle as O
from tests.gpu_util import download_x, upload

pytestmark = pytest.mark.gpu

VARIANTS = [0, 1]  # 0: tensor-core chain kernel, 1: CUDA-core chain kernel


def _solve(bss, A, B, d, T, variant, **kw):
    from blockstructuredsolvers_gb300 import _lib
    L = _lib.load()
    saved = L.bss_diag_get_factor_variant()
    _lib.check(L.bss_diag_set_factor_variant(variant))
    try:
        N, n, _ = A.shape
        data = bss.initialize_batched(N, n, T, k=d.shape[2], **kw)
        upload(data, A, B, d)
        bss.factorize_(data)
        bss.solve_(data)
        bss.synchronize(data)
        return download_x(data, N), bss.get_info(data)
    finally:
        _lib.check(L.bss_diag_set_factor_variant(saved))


@pytest.mark.parametrize("variant", VARIANTS)
@pytest.mark.parametrize("n", [33, 40, 47, 48, 63, 64])
def test_chain64_variants_fp32_and_mixed(n, variant):
    import torch
    import blockstructuredsolvers_gb300 as bss
    rng = np.random.default_rng(640 + n)
    N, k = 1500, 2
    A, B, d = O.gen_shifted_family(rng, N, n, k)
    x_ref = O.cpu_solve(A, B, d)
    x32, _ = _solve(bss, A, B, d, torch.float32, variant)
    assert O.rel_error(x32, x_ref) <= 1e-4
    xm, info = _solve(bss, A, B, d, torch.float64, variant, precision="mixed")
    assert O.rel_error(xm, x_ref) <= 1e-10
    assert info["rel_residual"] <= 1e-12 and 1 <= info["refine_steps"] <= 3
    assert O.rel_residual(A, B, xm, d) <= 1e-12


def test_separator_system_same_for_both_kernels():
    """The first-level separator system (A'_p = A_s - S_LL - S_RR,
    B'_p = -S_LR) from the tensor-core kernel's products agrees with the
    CUDA-core kernel's to FP32 accuracy."""
    import ctypes
    import torch
    import blockstructuredsolvers_gb300 as bss
    from blockstructuredsolvers_gb300 import _DevView, _lib
    L = _lib.load()
    rng = np.random.default_rng(6464)
    N, n = 2000, 64
    A, B, d = O.gen_shifted_family(rng, N, n, 1)
    outs = []
    saved = L.bss_diag_get_factor_variant()
    for variant in VARIANTS:
        _lib.check(L.bss_diag_set_factor_variant(variant))
        try:
            data = bss.initialize_batched(N, n, torch.float32)
            upload(data, A, B, d)
            _lib.check(L.bss_factorize_levels(data.handle, 1))
            torch.cuda.synchronize()
            Nl, Q = ctypes.c_int64(), ctypes.c_int64()
            pa, pb = ctypes.c_void_p(), ctypes.c_void_p()
            dt = ctypes.c_int32()
            _lib.check(L.bss_get_level(data.handle, 1, ctypes.byref(Nl), ctypes.byref(Q), ctypes.byref(pa),
                                       ctypes.byref(pb), None, ctypes.byref(dt)))
            cnt = Nl.value
            av = torch.as_tensor(_DevView(pa.value, (cnt * n * n,), (4,), "<f4", data), device="cuda")
            bv = torch.as_tensor(_DevView(pb.value, ((cnt - 1) * n * n,), (4,), "<f4", data), device="cuda")
            outs.append((av.double().cpu().numpy(), bv.double().cpu().numpy()))
            del av, bv, data
        finally:
            _lib.check(L.bss_diag_set_factor_variant(saved))
    (a0, b0), (a1, b1) = outs
    assert np.abs(a0 - a1).max() <= 1e-4 * np.abs(a1).max()
    assert np.abs(b0 - b1).max() <= 1e-4 * np.abs(b1).max()


def test_autotuner_picks_a_chain_kernel_and_it_is_used():
    """The tuner times both chain kernels for n = 64 in mixed precision and
    records the faster one; a handle created afterwards factors with it and
    stays correct."""
    import torch
    import blockstructuredsolvers_gb300 as bss
    bss.autotune_clear()
    try:
        e = bss.autotune(64, torch.float64, "mixed", N_probe=4096)
        assert e["factor_variant"] in VARIANTS
        rng = np.random.default_rng(77)
        A, B, d = O.gen_shifted_family(rng, 3000, 64, 1)
        data = bss.initialize_batched(3000, 64, torch.float64, precision="mixed")
        upload(data, A, B, d)
        bss.factorize_(data)
        bss.solve_(data)
        bss.synchronize(data)
        assert O.rel_error(download_x(data, 3000), O.cpu_solve(A, B, d)) <= 1e-10
    finally:
        bss.autotune_clear()
