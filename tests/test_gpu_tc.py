"""GPU test of the tensor-core (tcgen05, 3xTF32) product of the wide
kernel in isolation: C = X^T Y of FP32 blocks against an FP64 product.
Tolerance: 3xTF32 with FP32 accumulation, relative error <= 1e-5 of max |C|
(FP32 rounding is ~6e-8 per operation; K <= 128 terms)."""
import ctypes

import pytest

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("n", [128, 96, 65, 33, 8])
def test_tc_product_matches_fp64(n):
    import torch
    from blockstructuredsolvers_gb300 import _lib
    assert torch.cuda.is_available()
    err = ctypes.c_double()
    _lib.check(_lib.load().bss_tc_selftest(n, ctypes.byref(err)))
    assert err.value <= 1e-5


@pytest.mark.parametrize("polls", [1 << 10, 1 << 14])
def test_bounded_mbarrier_wait_expires(polls):
    """The tensor-core kernels' wait on their own mbarrier is bounded: on a
    barrier that nothing arrives on (a flag nobody sets) it gives up after
    `polls` polls and reports it, and the context stays usable afterwards."""
    import ctypes
    import numpy as np
    import torch
    import blockstructuredsolvers_gb300 as bss
    from blockstructuredsolvers_gb300 import _lib
    from oracle import oracle as O
    from tests.gpu_util import download_x, upload
    L = _lib.load()
    t, c = ctypes.c_int64(), ctypes.c_int64()
    _lib.check(L.bss_diag_wait_timeout(polls, ctypes.byref(t), ctypes.byref(c)))
    print(f"polls {polls}: expired {t.value}, {c.value} cycles ({c.value / polls:.0f} per poll)")
    assert t.value == 1 and c.value > 0
    rng = np.random.default_rng(4)
    A, B, d = O.gen_shifted_family(rng, 40, 16, 1, diag_shift=16)
    data = bss.initialize_batched(40, 16, torch.float64)
    upload(data, A, B, d)
    bss.factorize_(data)
    bss.solve_(data)
    bss.synchronize(data)
    assert O.rel_error(download_x(data, 40), O.cpu_solve(A, B, d)) <= 1e-10
