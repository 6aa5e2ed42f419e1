"""Mixed precision on ill-conditioned systems: block-Laplacian operators
T = tridiag(-I, (2 + eps) I + 1e-3 R R^T / n, -I), whose condition number grows
like (N / pi)^2 up to about 1e8 at N = 16384 with eps = 0.  The FP32
factorization of every level (the coarsest Schur complement included) must
still precondition the FP64 refinement to rel-resid <= 1e-12 within three
steps; the residual is re-checked here in FP64 with torch."""
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


@pytest.mark.parametrize("N,n,eps", [(4096, 16, 1e-6), (16384, 32, 0.0), (65536, 8, 0.0)])
def test_mixed_converges_on_block_laplacian(N, n, eps):
    import torch
    import blockstructuredsolvers_gb300 as bss
    A, B, d = _block_laplacian(N, n, eps, seed=3)
    data = bss.initialize_batched(N, n, torch.float64, precision="mixed", max_refine=10)
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
