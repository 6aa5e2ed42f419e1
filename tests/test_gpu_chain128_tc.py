"""The two chain kernels of FP32 factors for wide blocks (65 <= n <= 128:
plain FP32 and every partitioned level of the mixed path): the kernel that
keeps a chain step on chip (tcgen05 3xTF32 products with the factors carried
in shared and tensor memory between steps, one CTA per SM) and the wide
kernel that re-stages its tensor-core operands from L2 per product.  Each is
checked against the CPU oracle (<= 1e-4 relative error in FP32; rel-resid
<= 1e-12 and <= 1e-10 error in mixed precision), and their first-level
separator systems against each other."""
import ctypes

import numpy as np
import pytest

from oracle import oracle as O
from tests.gpu_util import download_x, upload

pytestmark = pytest.mark.gpu

VARIANTS = [0, 2]  # 0: on-chip chain kernel, 2 (BSS_FACTOR_WIDE_L2): L2-staged wide kernel


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
@pytest.mark.parametrize("n", [65, 72, 96, 101, 127, 128])
def test_chain128_variants_fp32_and_mixed(n, variant):
    import torch
    import blockstructuredsolvers_gb300 as bss
    rng = np.random.default_rng(1280 + n)
    N, k = 700, 2
    A, B, d = O.gen_shifted_family(rng, N, n, k)
    x_ref = O.cpu_solve(A, B, d)
    x32, _ = _solve(bss, A, B, d, torch.float32, variant)
    assert O.rel_error(x32, x_ref) <= 1e-4
    xm, info = _solve(bss, A, B, d, torch.float64, variant, precision="mixed")
    assert O.rel_error(xm, x_ref) <= 1e-10
    assert info["rel_residual"] <= 1e-12 and 1 <= info["refine_steps"] <= 3
    assert O.rel_residual(A, B, xm, d) <= 1e-12


def test_chain128_long_chains_mixed():
    """Chains of ~20 blocks (N = 3000 over one CTA per SM), where the
    factors carried on chip from step to step are reused most."""
    import torch
    import blockstructuredsolvers_gb300 as bss
    rng = np.random.default_rng(12800)
    N, n = 3000, 128
    A, B, d = O.gen_shifted_family(rng, N, n, 1)
    xm, info = _solve(bss, A, B, d, torch.float64, 0, precision="mixed")
    assert O.rel_error(xm, O.cpu_solve(A, B, d)) <= 1e-10
    assert info["rel_residual"] <= 1e-12 and 1 <= info["refine_steps"] <= 3


def test_chain128_separator_system_same_for_both_kernels():
    """The first-level separator system (A'_p = A_s - S_LL - S_RR,
    B'_p = -S_LR) from the on-chip kernel agrees with the L2-staged
    kernel's to FP32 accuracy.  The two kernels run different partition
    counts (one and two CTAs per SM), so each is compared with the same
    partition count forced through the plan options."""
    import torch
    import blockstructuredsolvers_gb300 as bss
    from blockstructuredsolvers_gb300 import _DevView, _lib
    L = _lib.load()
    rng = np.random.default_rng(12812)
    N, n = 2500, 128
    A, B, d = O.gen_shifted_family(rng, N, n, 1)
    outs = []
    saved = L.bss_diag_get_factor_variant()
    for variant in VARIANTS:
        _lib.check(L.bss_diag_set_factor_variant(variant))
        try:
            data = bss.initialize_batched(N, n, torch.float32, target_partitions=152)
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
            outs.append((cnt, av.double().cpu().numpy(), bv.double().cpu().numpy()))
            del av, bv, data
        finally:
            _lib.check(L.bss_diag_set_factor_variant(saved))
    (c0, a0, b0), (c1, a1, b1) = outs
    assert c0 == c1
    assert np.abs(a0 - a1).max() <= 1e-4 * np.abs(a1).max()
    assert np.abs(b0 - b1).max() <= 1e-4 * np.abs(b1).max()


def test_autotuner_picks_a_wide_chain_kernel_and_it_is_used():
    """The tuner times both wide chain kernels for n = 128 in mixed
    precision and records the faster one; a handle created afterwards
    factors with it and stays correct."""
    import torch
    import blockstructuredsolvers_gb300 as bss
    bss.autotune_clear()
    try:
        e = bss.autotune(128, torch.float64, "mixed", N_probe=2048)
        assert e["factor_variant"] in VARIANTS
        rng = np.random.default_rng(78)
        A, B, d = O.gen_shifted_family(rng, 1200, 128, 1)
        data = bss.initialize_batched(1200, 128, torch.float64, precision="mixed")
        upload(data, A, B, d)
        bss.factorize_(data)
        bss.solve_(data)
        bss.synchronize(data)
        assert O.rel_error(download_x(data, 1200), O.cpu_solve(A, B, d)) <= 1e-10
    finally:
        bss.autotune_clear()
