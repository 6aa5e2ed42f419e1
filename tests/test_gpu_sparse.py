"""GPU parity of the sparse harness: the device assembly of
construct_block_tridiagonal (benchmark/utils.jl:59-103; bss_csr_assemble)
against the oracle's restatement, bit for bit, and the sparse-Cholesky
comparison (benchmark/benchmark_gpu.jl:75-117; bss_spchol_*) against the
oracle's block Cholesky.  Tolerances: relative error <= 1e-10 (FP64),
<= 1e-4 (FP32)."""
import numpy as np
import pytest

from oracle import oracle as O
from tests.gpu_util import download_x, upload

pytestmark = pytest.mark.gpu


def _bits(a):
    a = np.ascontiguousarray(a)
    return a.view(np.uint64 if a.dtype == np.float64 else np.uint32)


@pytest.mark.parametrize("N,n,T", [(1, 4, "f64"), (2, 3, "f64"), (7, 5, "f64"), (40, 64, "f64"), (9, 33, "f32"),
                                   (5, 128, "f64"), (100, 32, "f64"), (3, 48, "f32")])
def test_assembly_bit_exact(N, n, T):
    import torch
    import blockstructuredsolvers_gb300 as bss
    npdt = np.float64 if T == "f64" else np.float32
    tdt = torch.float64 if T == "f64" else torch.float32
    rng = np.random.default_rng(7 * N + n)
    A = rng.standard_normal((N, n, n)).astype(npdt)
    B = rng.standard_normal((max(N - 1, 0), n, n)).astype(npdt)
    d = rng.standard_normal((N, n, 2)).astype(npdt)
    At = torch.from_numpy(A).cuda().permute(1, 2, 0)   # (n, n, N), not column-major in memory
    Bt = torch.from_numpy(B).cuda().permute(1, 2, 0)
    dt = torch.from_numpy(d).cuda().permute(1, 2, 0)
    M, dv = bss.construct_block_tridiagonal(At, Bt, dt)
    torch.cuda.synchronize()
    rp, ci, v, dref = O.construct_block_tridiagonal(A, B, d)
    assert M.dtype == tdt and tuple(M.shape) == (N * n, N * n)
    assert np.array_equal(M.crow_indices().cpu().numpy(), rp)
    assert np.array_equal(M.col_indices().cpu().numpy(), ci)
    assert np.array_equal(_bits(M.values().cpu().numpy()), _bits(v))
    assert np.array_equal(dv.cpu().numpy(), dref)


@pytest.mark.parametrize("N,n,k,T", [(50, 32, 1, "f64"), (100, 32, 1, "f64"), (64, 64, 3, "f64"),
                                     (30, 16, 2, "f32"), (1, 8, 1, "f64"), (2, 5, 1, "f64"), (17, 40, 2, "f64")])
def test_sparse_cholesky_matches_oracle(N, n, k, T):
    import torch
    import blockstructuredsolvers_gb300 as bss
    tdt = torch.float64 if T == "f64" else torch.float32
    rng = np.random.default_rng(N + 3 * n)
    A, B, d = O.gen_shifted_family(rng, N, n, k, diag_shift=max(n, 12))
    data = bss.initialize_sparse_cholesky(N, n, tdt, k=k)
    upload(data, A, B, d)
    bss.analyze_(data)
    bss.factorize_(data)
    bss.solve_(data)
    torch.cuda.synchronize()
    x = download_x(data, N)
    tol = 1e-10 if T == "f64" else 1e-4
    assert O.rel_error(x, O.cpu_solve(A, B, d)) <= tol
    # the handle's own CSR matrix is the oracle's assembly of its inputs
    npdt = np.float64 if T == "f64" else np.float32
    rp, ci, v, _ = O.construct_block_tridiagonal(A.astype(npdt), B.astype(npdt))
    M = data.csr()
    assert np.array_equal(M.crow_indices().cpu().numpy(), rp)
    assert np.array_equal(M.col_indices().cpu().numpy(), ci)
    assert np.array_equal(_bits(M.values().cpu().numpy()), _bits(v))


def test_sparse_cholesky_refactor_new_values():
    """A second factorize re-assembles the values only (the pattern and the
    analysis are kept) and solves the new system."""
    import torch
    import blockstructuredsolvers_gb300 as bss
    N, n, k = 60, 16, 1
    data = bss.initialize_sparse_cholesky(N, n, torch.float64, k=k)
    for seed in (1, 2):
        rng = np.random.default_rng(seed)
        A, B, d = O.gen_shifted_family(rng, N, n, k, diag_shift=16)
        upload(data, A, B, d)
        bss.factorize_(data)
        bss.solve_(data)
        torch.cuda.synchronize()
        assert O.rel_error(download_x(data, N), O.cpu_solve(A, B, d)) <= 1e-10


@pytest.mark.parametrize("blk,row,val", [(0, 0, -1.0), (3, 5, -100.0), (9, 7, -1000.0), (2, 3, 0.0)])
def test_sparse_cholesky_not_spd_names_the_block(blk, row, val):
    """A non-positive pivot raises NotSPDError naming the 0-based row and
    block (B = 0, so the pivot is the planted diagonal entry itself)."""
    import torch
    import blockstructuredsolvers_gb300 as bss
    N, n = 10, 8
    rng = np.random.default_rng(0)
    A, B, d = O.gen_shifted_family(rng, N, n, 1, diag_shift=12)
    B[:] = 0.0
    A[blk] = np.eye(n)
    A[blk][row, row] = val
    data = bss.initialize_sparse_cholesky(N, n, torch.float64)
    upload(data, A, B, d)
    with pytest.raises(bss.NotSPDError, match=rf"row {blk * n + row} \(block {blk}\)"):
        bss.factorize_(data)


def test_sparse_cholesky_call_order():
    """analyze twice keeps the analysis; solve before a successful
    factorize is BSS_ERR_STATE; after it, the solve is correct."""
    import torch
    import blockstructuredsolvers_gb300 as bss
    from blockstructuredsolvers_gb300 import _lib
    N, n, k = 20, 8, 1
    rng = np.random.default_rng(11)
    A, B, d = O.gen_shifted_family(rng, N, n, k, diag_shift=12)
    data = bss.initialize_sparse_cholesky(N, n, torch.float64, k=k)
    upload(data, A, B, d)
    bss.analyze_(data)
    bss.analyze_(data)
    with pytest.raises(bss.BSSError) as exc:
        bss.solve_(data)
    assert exc.value.code == _lib.BSS_ERR_STATE
    bss.factorize_(data)
    bss.solve_(data)
    torch.cuda.synchronize()
    assert O.rel_error(download_x(data, N), O.cpu_solve(A, B, d)) <= 1e-10
