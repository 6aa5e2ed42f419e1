"""GPU parity of the reference-algorithm comparator (bss_refalgo_*: the
reference's gpu_batched.jl restated over batched cuSOLVER/cuBLAS) against the
oracle's numpy restatement of the same algorithm and the CPU block
Cholesky.  Tolerances: relative error <= 1e-10 (FP64), <= 1e-4 (FP32)."""
import numpy as np
import pytest

from oracle import oracle as O
from tests.gpu_util import download_x, upload

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("N,n,k,T", [(50, 32, 1, "f64"), (100, 32, 1, "f64"), (333, 16, 2, "f64"),
                                     (7, 8, 1, "f64"), (100, 32, 1, "f32"), (64, 64, 3, "f64")])
def test_reference_algorithm_matches_oracle(N, n, k, T):
    import torch
    import blockstructuredsolvers_gb300 as bss
    tdt = torch.float64 if T == "f64" else torch.float32
    rng = np.random.default_rng(N + n)
    A, B, d = O.gen_shifted_family(rng, N, n, k, diag_shift=max(n, 12))
    data = bss.initialize_reference_algorithm(N, n, tdt, k=k)
    upload(data, A, B, d)
    bss.factorize_(data)
    bss.solve_(data)
    torch.cuda.synchronize()
    x = download_x(data, N)
    tol = 1e-10 if T == "f64" else 1e-4
    assert O.rel_error(x, O.cpu_solve(A, B, d)) <= tol
    if T == "f64" and k == 1:
        xr, _, _ = O.batched_reference_solve(A, B, d)
        assert O.rel_error(x, xr) <= 1e-12
