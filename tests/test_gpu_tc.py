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
