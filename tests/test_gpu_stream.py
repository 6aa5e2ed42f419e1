"""The streamed solve sweeps of wide blocks (n a multiple of 16 up to 128,
up to 8 right-hand-side columns per pass): every n x n block passes through
a ring of four shared-memory slots fed by bulk copies.  The backward product
splits the columns into shares by right-hand-side groups of four (one group
for k <= 4, two for k = 5 .. 8), so both layouts are checked, in FP32 and
FP64 and in mixed precision, against the CPU oracle."""
import numpy as np
import pytest

from oracle import oracle as O
from tests.gpu_util import download_x, upload

pytestmark = pytest.mark.gpu


def _solve(bss, A, B, d, T, **kw):
    N, n, _ = A.shape
    data = bss.initialize_batched(N, n, T, k=d.shape[2], **kw)
    upload(data, A, B, d)
    bss.factorize_(data)
    bss.solve_(data)
    bss.synchronize(data)
    return download_x(data, N), bss.get_info(data)


@pytest.mark.parametrize("k", [1, 3, 5, 8])
@pytest.mark.parametrize("n", [96, 112, 128])
def test_streamed_sweeps_fp32_fp64(n, k):
    import torch
    import blockstructuredsolvers_gb300 as bss
    rng = np.random.default_rng(1600 + 10 * n + k)
    N = 260
    A, B, d = O.gen_shifted_family(rng, N, n, k)
    x_ref = O.cpu_solve(A, B, d)
    x32, _ = _solve(bss, A, B, d, torch.float32)
    assert O.rel_error(x32, x_ref) <= 1e-4
    x64, _ = _solve(bss, A, B, d, torch.float64)
    assert O.rel_error(x64, x_ref) <= 1e-10


@pytest.mark.parametrize("k", [4, 6])
def test_streamed_sweeps_mixed(k):
    import torch
    import blockstructuredsolvers_gb300 as bss
    rng = np.random.default_rng(1700 + k)
    N, n = 900, 128
    A, B, d = O.gen_shifted_family(rng, N, n, k)
    xm, info = _solve(bss, A, B, d, torch.float64, precision="mixed")
    assert O.rel_error(xm, O.cpu_solve(A, B, d)) <= 1e-10
    assert info["rel_residual"] <= 1e-12 and 1 <= info["refine_steps"] <= 3
    assert O.rel_residual(A, B, xm, d) <= 1e-12
