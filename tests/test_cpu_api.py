"""The CPU API drop-in (bss_cpu_*: initialize_cpu / factorize! / solve! of
src/cpu.jl) against the oracle.  Runs without a GPU.

Tolerances: relative error vs the oracle's OpenBLAS restatement <= 1e-12
(FP64; the same operation sequence with different summation order) and
<= 1e-4 (FP32); the reference's own test bound 10 sqrt(eps) ||x|| on the
recovered solution (test/test_cpu.jl:71) and ||A x - d|| (test_cpu.jl:92).
"""
import numpy as np
import pytest

from oracle import oracle as O


@pytest.fixture(scope="module")
def bss():
    import blockstructuredsolvers_gb300 as bss
    return bss


def _load(data, A, B, d):
    N = A.shape[0]
    for i in range(N):
        data.A_list[i][:] = A[i]
        data.d_list[i][:] = d[i]
    for i in range(N - 1):
        data.B_list[i][:] = B[i]


@pytest.mark.parametrize("T", [np.float64, np.float32])
@pytest.mark.parametrize("N,n,k", [(50, 32, 1), (1, 8, 1), (2, 5, 3), (100, 16, 2)])
def test_cpu_api_matches_oracle(bss, T, N, n, k):
    rng = np.random.default_rng(N * 31 + n)
    A, B, d = O.gen_shifted_family(rng, N, n, k, diag_shift=max(n, 12))
    data = bss.initialize_cpu(N, n, T, k=k)
    assert data.N == N and len(data.A_list) == N and len(data.B_list) == N - 1
    _load(data, A, B, d)
    bss.factorize_(data)
    bss.solve_(data)
    x = np.stack([np.asarray(data.d_list[i], dtype=np.float64) for i in range(N)])
    ref = O.cpu_solve(A, B, d, dtype=T)
    tol = 1e-12 if T == np.float64 else 1e-4
    assert O.rel_error(x, ref) <= tol


def test_cpu_api_reference_known_answer(bss):
    """test/test_cpu.jl:15-92 form: x known, d = A x, recover x."""
    N, n = 50, 32
    rng = np.random.default_rng(42)
    A, B, x, d = O.gen_golden_system(7, N, n, 1)
    data = bss.initialize_cpu(N, n)
    _load(data, A, B, d)
    bss.factorize_(data)
    bss.solve_(data)
    xs = np.stack([np.array(data.d_list[i]) for i in range(N)])
    eps = np.finfo(np.float64).eps
    assert np.linalg.norm(xs - x) <= 10 * np.sqrt(eps) * np.linalg.norm(x)
    assert np.linalg.norm(O.block_matvec(A, B, xs) - d) <= 10 * np.sqrt(eps) * np.linalg.norm(d)


def test_cpu_api_factor_contents_match_reference_semantics(bss):
    """After factorize!, A_i's upper triangle is U_i (U_i^T U_i = A_i -
    B_{i-1}^T U_{i-1}^{-1} ... ) and B_i = U_i^{-T} B_i, as the reference
    leaves them; compared with the oracle's restatement of
    backbone_cpu.jl's factorize."""
    rng = np.random.default_rng(3)
    N, n = 12, 9
    A, B, d = O.gen_shifted_family(rng, N, n, 1)
    data = bss.initialize_cpu(N, n)
    _load(data, A, B, d)
    bss.factorize_(data)
    Ar = np.array(A, order="C")
    Br = np.array(B, order="C")
    O.cholesky_factorize(Ar, Br)
    for i in range(N):
        assert np.allclose(np.triu(data.A_list[i]), np.triu(Ar[i]), rtol=1e-12, atol=1e-12)
    for i in range(N - 1):
        assert np.allclose(data.B_list[i], Br[i], rtol=1e-12, atol=1e-12)


def test_cpu_api_not_spd(bss):
    rng = np.random.default_rng(4)
    A, B, d = O.gen_shifted_family(rng, 10, 6, 1)
    A[4] = -np.eye(6)
    data = bss.initialize_cpu(10, 6)
    _load(data, A, B, d)
    with pytest.raises(bss.NotSPDError):
        bss.factorize_(data)
