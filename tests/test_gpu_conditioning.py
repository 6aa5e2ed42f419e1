"""Mixed precision on ill-conditioned systems: block-Laplacian operators
T = tridiag(-I, (2 + eps) I + 1e-3 R R^T / n, -I), whose condition number grows
like (N / pi)^2 up to about 1e8 at N = 16384 with eps = 0.  The FP32
factorization of every level (the coarsest Schur complement included) must
still precondition the FP64 refinement to rel-resid <= 1e-12 within three
steps; the residual is re-checked here in FP64 with torch.  Each case runs
with the FP32 coarsest level (the default) and with the FP64 one, and on the
log-spectrum family at full size (N = 65536, n = 128, k = 4) the two must
agree."""
import pytest

pytestmark = pytest.mark.gpu


def _block_laplacian(N, n, eps, seed):
    import torch
    dev = torch.device("cuda")
    g = torch.Generator(device=dev).manual_seed(seed)
    R = torch.randn(N, n, n, device=dev, dtype=torch.float64, generator=g)
    A = (2.0 + eps) * torch.eye(n, device=dev, dtype=torch.float64) + 1e-3 * (R @ R.transpose(1, 2)) / n
    B = -torch.eye(n, device=dev, dtype=torch.float64).expand(N - 1, n, n).clone()
    d = torch.rand(N, n, 1, device=dev, dtype=torch.float64, generator=g)
    return A, B, d


def _rel_residual(A, B, x, d):
    import torch
    r = d - A @ x
    r[:-1] -= B @ x[1:]
    r[1:] -= B.transpose(1, 2) @ x[:-1]
    tn = A.abs().sum(2).amax()  # ||T||_inf: the B rows add 2 (|-I|) away from the ends
    tn = tn + 2.0
    return (r.abs().max() / (tn * x.abs().max() + d.abs().max())).item()


@pytest.mark.parametrize("coarsest_fp64", [False, True], ids=["coarsest32", "coarsest64"])
@pytest.mark.parametrize("N,n,eps", [(4096, 16, 1e-6), (16384, 32, 0.0), (65536, 8, 0.0)])
def test_mixed_converges_on_block_laplacian(N, n, eps, coarsest_fp64):
    import torch
    import blockstructuredsolvers_gb300 as bss
    A, B, d = _block_laplacian(N, n, eps, seed=3)
    data = bss.initialize_batched(N, n, torch.float64, precision="mixed", max_refine=10,
                                  coarsest_fp64=coarsest_fp64)
    data.A_tensor[:, :, :N] = A.permute(1, 2, 0)
    data.B_tensor[:, :, :N - 1] = B.permute(1, 2, 0)
    data.d_tensor[:, :, :N] = d.permute(1, 2, 0)
    bss.factorize_(data)
    bss.solve_(data)
    bss.synchronize(data)
    info = bss.get_info(data)
    x = data.d_tensor[:, :, :N].permute(2, 0, 1).contiguous()
    assert info["refine_steps"] <= 3
    assert info["rel_residual"] <= 1e-12
    assert _rel_residual(A, B, x, d) <= 1e-12


def _logspectrum(N, n, k, seed):
    """A_i = Q diag(logspace(0, 4, n)) Q^T, B_i = 0.45 lambda_min U V^T with
    Q, U, V random orthogonal, d ~ N(0,1): SPD by construction (the B's
    operator norm is below half the smallest eigenvalue of any A_i)."""
    import torch
    dev = torch.device("cuda")
    g = torch.Generator(device=dev).manual_seed(seed)
    lam = torch.logspace(0, 4, n, device=dev, dtype=torch.float64)
    A = torch.empty(N, n, n, device=dev, dtype=torch.float64)
    B = torch.empty(N - 1, n, n, device=dev, dtype=torch.float64)
    step = 8192
    for s0 in range(0, N, step):
        c = min(step, N - s0)
        Q, _ = torch.linalg.qr(torch.randn(c, n, n, device=dev, dtype=torch.float64, generator=g))
        A[s0:s0 + c] = (Q * lam) @ Q.transpose(1, 2)
        cb = min(c, N - 1 - s0)
        if cb > 0:
            U, _ = torch.linalg.qr(torch.randn(cb, n, n, device=dev, dtype=torch.float64, generator=g))
            V, _ = torch.linalg.qr(torch.randn(cb, n, n, device=dev, dtype=torch.float64, generator=g))
            B[s0:s0 + cb] = 0.45 * (U @ V.transpose(1, 2))
    d = torch.randn(N, n, k, device=dev, dtype=torch.float64, generator=g)
    return A, B, d


def test_coarsest_fp64_agrees_with_fp32_on_logspectrum_full_size():
    """N = 65536 blocks of n = 128, k = 4, eigenvalues log-spaced over
    [1, 1e4]: the FP32-coarsest default and the FP64-coarsest option both
    reach rel-resid <= 1e-12 (recomputed in FP64 here) and their solutions
    agree to 1e-9 relative (each is within cond * 1e-12 of the exact x)."""
    import torch
    import blockstructuredsolvers_gb300 as bss
    N, n, k = 65536, 128, 4
    A, B, d = _logspectrum(N, n, k, seed=7)
    rs = A.abs().sum(2)
    rs[:-1] += B.abs().sum(2)
    rs[1:] += B.abs().sum(1)
    tn = rs.max().item()  # ||T||_inf
    del rs
    xs = []
    for c64 in (False, True):
        data = bss.initialize_batched(N, n, torch.float64, k=k, precision="mixed", coarsest_fp64=c64)
        data.A_tensor[:, :, :N] = A.permute(1, 2, 0)
        data.B_tensor[:, :, :N - 1] = B.permute(1, 2, 0)
        data.d_tensor[:, :, :N] = d.permute(1, 2, 0)
        bss.factorize_(data)
        bss.solve_(data)
        bss.synchronize(data)
        info = bss.get_info(data)
        x = data.d_tensor[:, :, :N].permute(2, 0, 1).contiguous()
        r = d - A @ x
        r[:-1] -= B @ x[1:]
        r[1:] -= B.transpose(1, 2) @ x[:-1]
        rel = (r.abs().max() / (tn * x.abs().max() + d.abs().max())).item()
        assert info["rel_residual"] <= 1e-12 and info["refine_steps"] <= 4, (c64, info)
        assert rel <= 1e-12, (c64, rel)
        xs.append(x)
        del data
        torch.cuda.empty_cache()
    diff = ((xs[0] - xs[1]).abs().max() / xs[1].abs().max()).item()
    assert diff <= 1e-9, diff
