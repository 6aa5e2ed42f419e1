"""GPU parity: the sm_103a path (through the C ABI, via the Python mirror of
initialize_batched / factorize! / solve!) against the oracle.

Tolerances (tighter than the reference's own
10*sqrt(eps) of test/test_cuda.jl:119): relative error vs the CPU oracle
(backbone_cpu.jl restated) and vs a dense FP64 Cholesky <= 1e-10 in FP64,
<= 1e-4 in FP32; mixed precision reaches relative residual <= 1e-12.
"""
import ctypes
import glob
import os

import numpy as np
import pytest

from oracle import oracle as O
from tests.gpu_util import download_blocks, download_x, upload

pytestmark = pytest.mark.gpu

GOLD = os.path.join(os.path.dirname(__file__), "golden")
FIXTURES = sorted(glob.glob(os.path.join(GOLD, "*.npz")))
FIX_IDS = [os.path.basename(p)[:-4] for p in FIXTURES]

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


def _fixture(path):
    z = np.load(path)
    N, n, k, seed = int(z["N"]), int(z["n"]), int(z["k"]), int(z["seed"])
    A, B, x, _ = O.gen_golden_system(seed, N, n, k)
    return z, A, B, z["d"], N, n, k


def _run(bss, A, B, d, T, **kw):
    import torch
    N, n, _ = A.shape
    k = d.shape[2]
    data = bss.initialize_batched(N, n, T, k=k, **kw)
    upload(data, A, B, d)
    bss.factorize_(data)
    bss.solve_(data)
    bss.synchronize(data)
    torch.cuda.synchronize()
    return data, download_x(data, N)


@pytest.mark.parametrize("plan", ["auto", "reference"])
@pytest.mark.parametrize("path", FIXTURES, ids=FIX_IDS)
def test_golden_fp64(bss, path, plan):
    import torch
    z, A, B, d, N, n, k = _fixture(path)
    data, x = _run(bss, A, B, d, torch.float64, plan=plan)
    assert O.rel_error(x, z["x_cpu_f64"]) <= TOL64
    assert O.rel_error(x, z["x_dense"]) <= TOL64
    assert O.rel_error(x, z["x_true"]) <= 10 * np.sqrt(np.finfo(np.float64).eps)
    assert O.rel_residual(A, B, x, d) <= 1e-14
    # padding blocks (gpu_batched.jl:177-179) solve to zero
    if data.N > N:
        assert np.abs(download_x(data)[N:]).max() == 0.0


@pytest.mark.parametrize("path", FIXTURES, ids=FIX_IDS)
def test_golden_fp32(bss, path):
    import torch
    z, A, B, d, N, n, k = _fixture(path)
    _, x = _run(bss, A, B, d, torch.float32)
    assert O.rel_error(x, z["x_cpu_f64"]) <= TOL32
    assert O.rel_error(x, z["x_cpu_f32"]) <= TOL32
    assert O.rel_error(x, z["x_true"]) <= 10 * np.sqrt(np.finfo(np.float32).eps)


@pytest.mark.parametrize("path", FIXTURES, ids=FIX_IDS)
def test_golden_mixed(bss, path):
    import torch
    z, A, B, d, N, n, k = _fixture(path)
    data, x = _run(bss, A, B, d, torch.float64, precision="mixed")
    info = bss.get_info(data)
    assert info["rel_residual"] <= 1e-12
    assert O.rel_residual(A, B, x, d) <= 1e-12
    assert O.rel_error(x, z["x_dense"]) <= TOL64
    # A and B are left untouched by the mixed path
    assert np.array_equal(download_blocks(data.A_tensor, N), A)


def test_separator_system_matches_reference_restatement(bss):
    """With the reference plan, the assembled level-1 separator system equals
    the reference's NextData.A_tensor / B_tensor after factorize!
    (gpu_batched.jl:223-224), restated in numpy."""
    import torch
    from blockstructuredsolvers_gb300 import _lib
    L = _lib.load()
    for path in FIXTURES:
        z = np.load(path)
        if "lhs_A" not in z.files:
            continue
        _, A, B, d, N, n, k = _fixture(path)
        data = bss.initialize_batched(N, n, torch.float64, k=k, plan="reference")
        upload(data, A, B, d)
        _lib.check(L.bss_factorize_levels(data.handle, 1))
        torch.cuda.synchronize()
        Nl = ctypes.c_int64()
        Q = ctypes.c_int64()
        Ap = ctypes.c_void_p()
        Bp = ctypes.c_void_p()
        dp = ctypes.c_void_p()
        dt = ctypes.c_int32()
        _lib.check(L.bss_get_level(data.handle, 1, ctypes.byref(Nl), ctypes.byref(Q), ctypes.byref(Ap),
                                   ctypes.byref(Bp), ctypes.byref(dp), ctypes.byref(dt)))
        P = Nl.value
        assert P == z["lhs_A"].shape[0]
        nn = n * n
        a = torch.empty(P * nn, dtype=torch.float64, device="cuda")
        b = torch.empty(max(P - 1, 1) * nn, dtype=torch.float64, device="cuda")
        torch.cuda.synchronize()
        from blockstructuredsolvers_gb300 import _DevView
        av = torch.as_tensor(_DevView(Ap.value, (P * nn,), (8,), "<f8", data), device="cuda")
        bv = torch.as_tensor(_DevView(Bp.value, ((P - 1) * nn,), (8,), "<f8", data), device="cuda")
        a.copy_(av)
        b[: (P - 1) * nn].copy_(bv)
        lhsA = a.view(P, n, n).transpose(1, 2).cpu().numpy()
        lhsB = b[: (P - 1) * nn].view(P - 1, n, n).transpose(1, 2).cpu().numpy()
        scale = np.abs(z["lhs_A"]).max()
        assert np.abs(lhsA - z["lhs_A"]).max() <= 1e-12 * scale, path
        assert np.abs(lhsB - z["lhs_B"]).max() <= 1e-12 * scale, path


def test_seq_api(bss):
    import torch
    z, A, B, d, N, n, k = _fixture(os.path.join(GOLD, "reftest_N50_n32_k1.npz"))
    data = bss.initialize_seq(N, n, torch.float64, k=k)
    assert data.N == N
    upload(data, A, B, d)
    bss.factorize_(data)
    bss.solve_(data)
    bss.synchronize(data)
    x = download_x(data)
    assert O.rel_error(x, z["x_cpu_f64"]) <= TOL64


def test_repeat_solve_after_one_factorize(bss):
    import torch
    rng = np.random.default_rng(5)
    A, B, d = O.gen_shifted_family(rng, 200, 24, 3)
    data = bss.initialize_batched(200, 24, torch.float64, k=3)
    upload(data, A, B, d)
    bss.factorize_(data)
    bss.solve_(data)
    x1 = download_x(data, 200)
    d2 = rng.random((200, 24, 3))
    data.d_tensor[:, :, :200] = torch.from_numpy(d2).cuda().permute(1, 2, 0)
    bss.solve_(data)
    x2 = download_x(data, 200)
    xr = O.cpu_solve(A, B, d)
    xr2 = O.cpu_solve(A, B, d2)
    assert O.rel_error(x1, xr) <= TOL64 and O.rel_error(x2, xr2) <= TOL64
    data.d_tensor[:, :, :200] = torch.from_numpy(d).cuda().permute(1, 2, 0)
    bss.solve_(data)
    assert np.array_equal(download_x(data, 200), x1)  # deterministic


@pytest.mark.parametrize("n", [1, 2, 7, 16, 17, 31, 33, 63, 64])
def test_ragged_block_sizes(bss, n):
    import torch
    rng = np.random.default_rng(n)
    N = 61
    # G G^T + n I with B ~ N(0,1) is SPD only when n > 4 sqrt(n) roughly;
    # small n needs a larger shift to stay SPD
    A, B, d = O.gen_shifted_family(rng, N, n, 2, diag_shift=max(n, 12.0))
    _, x = _run(bss, A, B, d, torch.float64)
    assert O.rel_error(x, O.cpu_solve(A, B, d)) <= TOL64


@pytest.mark.parametrize("k", [1, 5, 33, 70])
def test_many_rhs(bss, k):
    import torch
    rng = np.random.default_rng(k)
    A, B, d = O.gen_shifted_family(rng, 120, 16, k)
    _, x = _run(bss, A, B, d, torch.float64)
    assert O.rel_error(x, O.cpu_solve(A, B, d)) <= TOL64


@pytest.mark.parametrize("parts", [1, 2, 3, 7, 40])
def test_partition_counts(bss, parts):
    import torch
    rng = np.random.default_rng(parts)
    A, B, d = O.gen_shifted_family(rng, 333, 8, 1)
    _, x = _run(bss, A, B, d, torch.float64, target_partitions=parts, seq_cutoff=3)
    assert O.rel_error(x, O.cpu_solve(A, B, d)) <= TOL64


def test_not_spd_is_reported(bss):
    import torch
    rng = np.random.default_rng(9)
    A, B, d = O.gen_shifted_family(rng, 100, 8, 1)
    A[37] = -A[37]
    data = bss.initialize_batched(100, 8, torch.float64)
    upload(data, A, B, d)
    bss.factorize_(data)
    with pytest.raises(bss.NotSPDError):
        bss.synchronize(data)
    info = bss.get_info(data)
    assert info["failed_block"] >= 0


def test_config2_family_mixed(bss):
    """log-spaced-spectrum generator (lambda in [1, 1e4]) at a reduced size: FP32 factor
    + FP64 refinement reaches 1e-12."""
    import torch
    rng = np.random.default_rng(2)
    A, B, d = O.gen_logspectrum(rng, 400, 32, 4)
    data, x = _run(bss, A, B, d, torch.float64, precision="mixed")
    assert bss.get_info(data)["rel_residual"] <= 1e-12
    assert O.rel_residual(A, B, x, d) <= 1e-12
    assert O.rel_error(x, O.cpu_solve(A, B, d)) <= 1e-9


def test_kalman_family(bss):
    import torch
    rng = np.random.default_rng(4)
    A, B, d = O.gen_kalman(rng, 500, 16, 1)
    _, x = _run(bss, A, B, d, torch.float64)
    assert O.rel_error(x, O.cpu_solve(A, B, d)) <= TOL64


def test_residual_entry_point(bss):
    import torch
    rng = np.random.default_rng(1)
    A, B, d = O.gen_shifted_family(rng, 64, 16, 2)
    # a perturbed solution, so the residual is well above roundoff
    x = O.cpu_solve(A, B, d) + 1e-6 * rng.standard_normal(d.shape)
    to = lambda a: torch.from_numpy(np.ascontiguousarray(a)).cuda().permute(1, 2, 0)
    At = bss.colmajor_empty((16, 16, 64), torch.float64)
    At.copy_(to(A))
    Bt = bss.colmajor_empty((16, 16, 63), torch.float64)
    Bt.copy_(to(B))
    xt = bss.colmajor_empty((16, 2, 64), torch.float64)
    xt.copy_(to(x))
    dt = bss.colmajor_empty((16, 2, 64), torch.float64)
    dt.copy_(to(d))
    r = bss.residual(At, Bt, xt, dt)
    want = O.rel_residual(A, B, x, d)
    # numerator in FP64; ||T||_inf accumulated in FP32 (relative accuracy ~1e-6)
    assert want > 1e-9 and abs(r - want) <= 1e-5 * want


@pytest.fixture(scope="module")
def config1_system():
    """N=16384 blocks of n=64, k=1 (A_i = G G^T + n I, B_i ~ N(0,1),
    d ~ U[0,1)) generated once with numpy's seeded Generator, and its
    solution by the C oracle (the restatement of backbone_cpu.jl) in FP64."""
    from oracle import cref
    rng = np.random.default_rng(20261204)
    A, B, d = O.gen_shifted_family(rng, 16384, 64, 1)
    cref.set_blas_threads(os.cpu_count() or 1)
    x_ref = cref.solve_math(A, B, d, np.float64)
    return A, B, d, x_ref


@pytest.mark.parametrize("T", ["f64", "f32", "mixed"])
def test_config1_full_size_vs_oracle(bss, config1_system, T):
    """N=16384, n=64 at full size: the solution against the C oracle's FP64
    solve of the same inputs (relative error <= 1e-10 in FP64 and mixed,
    <= 1e-4 in FP32), and the relative residual recomputed here in FP64 on the
    GPU (<= 1e-14 FP64, <= 1e-6 FP32, <= 1e-12 mixed)."""
    import torch
    A_np, B_np, d_np, x_ref = config1_system
    N, n = 16384, 64
    A = torch.from_numpy(A_np).cuda()
    B = torch.from_numpy(B_np).cuda()
    d = torch.from_numpy(d_np).cuda()
    dt = torch.float32 if T == "f32" else torch.float64
    kw = {"precision": "mixed"} if T == "mixed" else {}
    data = bss.initialize_batched(N, n, dt, **kw)
    data.A_tensor[:, :, :N] = A.to(dt).permute(1, 2, 0)
    data.B_tensor[:, :, :N - 1] = B.to(dt).permute(1, 2, 0)
    data.d_tensor[:, :, :N] = d.to(dt).permute(1, 2, 0)
    bss.factorize_(data)
    bss.solve_(data)
    bss.synchronize(data)
    x = data.d_tensor[:, :, :N].permute(2, 0, 1).double()
    err = O.rel_error(x.cpu().numpy(), x_ref)
    assert err <= {"f64": TOL64, "f32": TOL32, "mixed": TOL64}[T], err
    r = d - A @ x
    r[:-1] -= B @ x[1:]
    r[1:] -= B.transpose(1, 2) @ x[:-1]
    rs = A.abs().sum(2)
    rs[:-1] += B.abs().sum(2)
    rs[1:] += B.abs().sum(1)
    rel = (r.abs().max() / (rs.max() * x.abs().max() + d.abs().max())).item()
    bound = {"f64": 1e-14, "f32": 1e-6, "mixed": 1e-12}[T]
    assert rel <= bound, rel
    if T == "mixed":
        info = bss.get_info(data)
        assert info["rel_residual"] <= 1e-12 and info["refine_steps"] >= 1


@pytest.mark.parametrize("precision", ["plain", "mixed"])
def test_graph_replay_matches_eager(bss, precision):
    """Calls after the first replay CUDA graphs (the mixed refinement loop on
    the device); results must equal the eager first call bit for bit and the
    refinement outcome must be reported after synchronize."""
    import torch
    rng = np.random.default_rng(11)
    A, B, d = O.gen_shifted_family(rng, 700, 32, 2)
    outs = []
    for use_graphs in (True, False):
        data = bss.initialize_batched(700, 32, torch.float64, k=2, precision=precision, use_graphs=use_graphs)
        for rep in range(3):
            upload(data, A, B, d)
            bss.factorize_(data)
            bss.solve_(data)
            bss.synchronize(data)
            outs.append(download_x(data, 700))
            if precision == "mixed":
                info = bss.get_info(data)
                assert info["rel_residual"] <= 1e-12 and info["refine_steps"] >= 1
    for x in outs[1:]:
        assert np.array_equal(x, outs[0])
    assert O.rel_error(outs[0], O.cpu_solve(A, B, d)) <= TOL64
