"""GPU parity of the many-system batch (bss_batch_*: independent systems of
uneven N, n and k factored and solved together) against the oracle.

Tolerances: relative error vs the CPU block Cholesky oracle (cpu.jl
restated) <= 1e-10 in FP64 and <= 1e-4 in FP32; mixed precision reaches a
relative residual <= 1e-12 for every system.
"""
import numpy as np
import pytest

from oracle import oracle as O
from tests.gpu_util import download_x, upload

pytestmark = pytest.mark.gpu

TOL64 = 1e-10
TOL32 = 1e-4

# (N, n, k): ragged sizes, every block-size class, single-block systems
SYSTEMS = [(1, 8, 1), (2, 16, 2), (3, 5, 1), (17, 32, 3), (64, 48, 1), (200, 64, 2), (300, 24, 4),
           (513, 16, 1), (40, 1, 1), (9, 64, 8), (130, 33, 2), (257, 64, 1)]


@pytest.fixture(scope="module")
def bss():
    import torch
    import blockstructuredsolvers_gb300 as bss
    from blockstructuredsolvers_gb300 import _lib
    assert torch.cuda.is_available()
    _lib.load()
    return bss


def _gen(seed, systems, family="c0"):
    rng = np.random.default_rng(seed)
    out = []
    for (N, n, k) in systems:
        if family == "c0":
            A, B, d = O.gen_shifted_family(rng, N, n, k, diag_shift=max(n, 12))
        else:  # the uneven-batch family: A = G G^T + 2n I, B = 0.5 N(0,1)
            A, B, d = O.gen_shifted_family(rng, N, n, k, diag_shift=2.0 * max(n, 6), b_scale=0.5)
        out.append((A, B, d))
    return out


def _run(bss, systems, probs, T, **kw):
    import torch
    b = bss.initialize_multi([s[0] for s in systems], [s[1] for s in systems], [s[2] for s in systems], T, **kw)
    for sysv, (A, B, d) in zip(b.systems, probs):
        upload(sysv, A, B, d)
    b.factorize()
    b.solve()
    b.synchronize()
    torch.cuda.synchronize()
    return b, [download_x(sysv, sysv.N) for sysv in b.systems]


def test_batch_plain_fp64_matches_oracle(bss):
    import torch
    probs = _gen(11, SYSTEMS)
    _, xs = _run(bss, SYSTEMS, probs, torch.float64)
    for (A, B, d), x in zip(probs, xs):
        x_ref = O.cpu_solve(A, B, d)
        assert O.rel_error(x, x_ref) <= TOL64
        if A.shape[0] * A.shape[1] <= 2000:
            assert O.rel_error(x, O.dense_solve(A, B, d)) <= TOL64


def test_batch_plain_fp32_matches_oracle(bss):
    import torch
    probs = _gen(12, SYSTEMS, family="c3")
    _, xs = _run(bss, SYSTEMS, probs, torch.float32)
    for (A, B, d), x in zip(probs, xs):
        assert O.rel_error(x, O.cpu_solve(A, B, d)) <= TOL32


def test_batch_mixed_reaches_1e12(bss):
    import torch
    probs = _gen(13, SYSTEMS, family="c3")
    b, xs = _run(bss, SYSTEMS, probs, torch.float64, precision="mixed", tol=1e-12)
    for s, ((A, B, d), x) in enumerate(zip(probs, xs)):
        inf = b.info(s)
        assert O.rel_residual(A, B, x, d) <= 1e-12
        assert inf["rel_residual"] <= 1e-12
        assert 0 <= inf["refine_steps"] <= 10
        assert O.rel_error(x, O.cpu_solve(A, B, d)) <= TOL64


@pytest.mark.parametrize("precision", ["plain", "mixed"])
def test_batch_graph_replay_bitwise(bss, precision):
    """First call eager, second captures a CUDA graph, third replays it: the
    three results are bitwise identical."""
    import torch
    probs = _gen(14, SYSTEMS, family="c3")
    b = bss.initialize_multi([s[0] for s in SYSTEMS], [s[1] for s in SYSTEMS], [s[2] for s in SYSTEMS],
                             torch.float64, precision=precision)
    runs = []
    for _ in range(3):
        for sysv, (A, B, d) in zip(b.systems, probs):
            upload(sysv, A, B, d)
        b.factorize()
        b.solve()
        b.synchronize()
        runs.append([download_x(sysv, sysv.N) for sysv in b.systems])
    for r in runs[1:]:
        for x0, x1 in zip(runs[0], r):
            assert np.array_equal(x0, x1)


@pytest.mark.parametrize("precision", ["plain", "mixed"])
def test_batch_result_same_alone_and_in_mix(bss, precision):
    """A system's plan depends only on itself, so its solution is bitwise the
    same solved alone and inside a batch of other systems."""
    import torch
    probs = _gen(15, SYSTEMS, family="c3")
    _, mix = _run(bss, SYSTEMS, probs, torch.float64, precision=precision)
    for i in (0, 5, 7, 11):
        _, alone = _run(bss, [SYSTEMS[i]], [probs[i]], torch.float64, precision=precision)
        assert np.array_equal(alone[0], mix[i])


def test_batch_repeat_solve_on_resident_factors(bss):
    """One factorize, several solves with new right-hand sides."""
    import torch
    probs = _gen(16, SYSTEMS, family="c3")
    b, _ = _run(bss, SYSTEMS, probs, torch.float64, precision="mixed")
    rng = np.random.default_rng(99)
    for _ in range(2):
        ds = []
        for sysv, (A, B, _) in zip(b.systems, probs):
            d = rng.standard_normal((sysv.N, sysv.n, sysv.k))
            ds.append(d)
            sysv.d_tensor.copy_(torch.from_numpy(d).to(sysv.d_tensor.device).permute(1, 2, 0))
        b.solve()
        b.synchronize()
        for sysv, (A, B, _), d in zip(b.systems, probs, ds):
            assert O.rel_residual(A, B, download_x(sysv, sysv.N), d) <= 1e-12


def test_batch_not_spd_reports_system(bss):
    import torch
    systems = SYSTEMS[:6]
    probs = _gen(17, systems, family="c3")
    A, B, d = probs[4]
    A = A.copy()
    A[10] = -np.eye(A.shape[1])
    probs[4] = (A, B, d)
    b = bss.initialize_multi([s[0] for s in systems], [s[1] for s in systems], [s[2] for s in systems],
                             torch.float64)
    for sysv, (A_, B_, d_) in zip(b.systems, probs):
        upload(sysv, A_, B_, d_)
    b.factorize()
    with pytest.raises(bss.NotSPDError):
        b.synchronize()
    assert b.info(4)["failed_block"] >= 0
    for s in (0, 1, 2, 3, 5):
        assert b.info(s)["failed_block"] == -1


def test_batch_rejects_unsupported_block_size(bss):
    import torch
    with pytest.raises(bss.BSSError):
        bss.initialize_multi([10, 10], [16, 2000], [1, 1], torch.float64)


def test_batch_cfg3_family_sample(bss):
    """A sample of the uneven-batch workload (N ~ U{16..1024}, n in the
    supported classes, k ~ U{1..8}), mixed precision to 1e-12."""
    import torch
    rng = np.random.default_rng(2048)
    systems = [(int(rng.integers(16, 1025)), int(rng.choice([16, 32, 48, 64])), int(rng.integers(1, 9)))
               for _ in range(48)]
    probs = _gen(18, systems, family="c3")
    b, xs = _run(bss, systems, probs, torch.float64, precision="mixed")
    for s, ((A, B, d), x) in enumerate(zip(probs, xs)):
        assert O.rel_residual(A, B, x, d) <= 1e-12
        assert b.info(s)["rel_residual"] <= 1e-12
