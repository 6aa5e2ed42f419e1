"""GPU parity of the wide-block path (64 < n <= 1024: chain matrices in
global memory, 64 x 64 tiles through shared memory; solves read the blocks
straight from global memory when they cannot be staged) against the oracle.

Tolerances: relative error vs the CPU block Cholesky oracle <= 1e-10 (FP64),
<= 1e-4 (FP32); mixed precision relative residual <= 1e-12.
"""
import numpy as np
import pytest

from oracle import oracle as O
from tests.gpu_util import download_x, upload

pytestmark = pytest.mark.gpu

TOL64 = 1e-10
TOL32 = 1e-4


@pytest.fixture(scope="module")
def bss():
    import torch
    import blockstructuredsolvers_gb300 as bss
    from blockstructuredsolvers_gb300 import _lib
    assert torch.cuda.is_available()
    _lib.load()
    return bss


def _run(bss, A, B, d, T, **kw):
    import torch
    N, n, _ = A.shape
    data = bss.initialize_batched(N, n, T, k=d.shape[2], **kw)
    upload(data, A, B, d)
    bss.factorize_(data)
    bss.solve_(data)
    bss.synchronize(data)
    torch.cuda.synchronize()
    return data, download_x(data, N)


@pytest.mark.parametrize("n", [65, 80, 96, 127, 128, 129, 200])
def test_wide_fp64(bss, n):
    import torch
    rng = np.random.default_rng(100 + n)
    A, B, d = O.gen_shifted_family(rng, 37, n, 2)
    _, x = _run(bss, A, B, d, torch.float64)
    assert O.rel_error(x, O.cpu_solve(A, B, d)) <= TOL64
    assert O.rel_error(x, O.dense_solve(A, B, d)) <= TOL64


@pytest.mark.parametrize("n", [72, 96, 128])
def test_wide_fp32(bss, n):
    import torch
    rng = np.random.default_rng(200 + n)
    A, B, d = O.gen_shifted_family(rng, 45, n, 1, diag_shift=2.0 * n, b_scale=0.5)
    _, x = _run(bss, A, B, d, torch.float32)
    assert O.rel_error(x, O.cpu_solve(A, B, d)) <= TOL32


@pytest.mark.parametrize("n", [96, 128])
def test_wide_mixed_config2_family(bss, n):
    """log-spaced-spectrum generator (lambda over [1, 1e4]) at n = 96, 128:
    FP32 factor + FP64 refinement to 1e-12."""
    import torch
    rng = np.random.default_rng(300 + n)
    A, B, d = O.gen_logspectrum(rng, 150, n, 4)
    data, x = _run(bss, A, B, d, torch.float64, precision="mixed")
    info = bss.get_info(data)
    assert info["rel_residual"] <= 1e-12
    assert O.rel_residual(A, B, x, d) <= 1e-12
    assert O.rel_error(x, O.cpu_solve(A, B, d)) <= 1e-9


@pytest.mark.parametrize("plan", ["auto", "reference"])
def test_wide_partitions_and_reference_plan(bss, plan):
    import torch
    rng = np.random.default_rng(7)
    A, B, d = O.gen_shifted_family(rng, 130, 96, 1)
    _, x = _run(bss, A, B, d, torch.float64, plan=plan)
    assert O.rel_error(x, O.cpu_solve(A, B, d)) <= TOL64


def test_wide_seq_api(bss):
    import torch
    rng = np.random.default_rng(8)
    A, B, d = O.gen_shifted_family(rng, 20, 128, 3)
    data = bss.initialize_seq(20, 128, torch.float64, k=3)
    upload(data, A, B, d)
    bss.factorize_(data)
    bss.solve_(data)
    bss.synchronize(data)
    assert O.rel_error(download_x(data), O.cpu_solve(A, B, d)) <= TOL64


def test_wide_many_rhs(bss):
    import torch
    rng = np.random.default_rng(9)
    A, B, d = O.gen_shifted_family(rng, 40, 128, 40)
    _, x = _run(bss, A, B, d, torch.float64)
    assert O.rel_error(x, O.cpu_solve(A, B, d)) <= TOL64


def test_wide_not_spd_is_reported(bss):
    import torch
    rng = np.random.default_rng(10)
    A, B, d = O.gen_shifted_family(rng, 50, 96, 1)
    A[21] = -np.eye(96)
    data = bss.initialize_batched(50, 96, torch.float64)
    upload(data, A, B, d)
    bss.factorize_(data)
    with pytest.raises(bss.NotSPDError):
        bss.synchronize(data)


def test_batch_with_wide_systems(bss):
    """The uneven-batch family with every block-size class, n in
    {16, 32, 48, 64, 96, 128}, mixed precision to 1e-12."""
    import torch
    rng = np.random.default_rng(11)
    systems = [(int(rng.integers(16, 200)), n, int(rng.integers(1, 9))) for n in (16, 32, 48, 64, 96, 128)
               for _ in range(2)]
    probs = []
    for (N, n, k) in systems:
        probs.append(O.gen_shifted_family(rng, N, n, k, diag_shift=2.0 * n, b_scale=0.5))
    b = bss.initialize_multi([s[0] for s in systems], [s[1] for s in systems], [s[2] for s in systems],
                             torch.float64, precision="mixed")
    for sysv, (A, B, d) in zip(b.systems, probs):
        upload(sysv, A, B, d)
    b.factorize()
    b.solve()
    b.synchronize()
    for s, ((A, B, d), sysv) in enumerate(zip(probs, b.systems)):
        x = download_x(sysv, sysv.N)
        assert O.rel_residual(A, B, x, d) <= 1e-12
        assert b.info(s)["rel_residual"] <= 1e-12


def test_mixed_rejects_n_above_128(bss):
    import torch
    with pytest.raises(bss.BSSError):
        bss.initialize_batched(10, 160, torch.float64, precision="mixed")
