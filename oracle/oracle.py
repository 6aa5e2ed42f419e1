"""CPU oracle for the batched block-tridiagonal SPD solver.

TEST INFRASTRUCTURE ONLY.  Nothing in the product path imports this module:
only ``tests/``, ``__graft_entry__.smoke()`` and the ``cpu_baseline`` /
``--impl reference`` legs of ``bench.py`` may use it, and only to check results
or as the timed CPU baseline.

What it restates (reference = BlockStructuredSolvers.jl, Julia):

* ``build_sequence`` / ``find_sequence_upper``  -- the level planner of
  ``src/gpu_batched.jl:112-162`` (integer, bit-exact).
* ``cholesky_factorize`` / ``cholesky_solve``    -- the sequential block
  Cholesky of ``src/backbone_cpu.jl:5-33`` wrapped by ``src/cpu.jl:30-50``
  (LAPACK potrf 'U', BLAS trsm L/U/T/N, gemm T/N; backward trsm L/U/N/N, gemm
  N/N), called here through scipy's LAPACK/BLAS.
* ``batched_factorize`` / ``batched_solve``      -- the recursive
  Schur-complement algorithm of ``src/gpu_batched.jl:184-258`` with the batched
  kernels of ``src/backbone_cuda.jl:70-184`` (potrfBatched / trsmBatched /
  gemmBatched over strided partitions, G/F fill, M_2n Schur blocks, Schur RHS,
  boundary update), restated with numpy loops over the partitions.
* ``dense_solve``                                 -- an independent FP64 dense
  Cholesky of the assembled matrix (convention of ``test/utils.jl:32-74``:
  block (i,i+1) = B_i, block (i+1,i) = B_i^T).

Parity pinning: the reference publishes no golden vectors and cannot run here
(Julia is not installed).  The oracle is pinned against the reference's own
known-answer tests (``test/test_cpu.jl:9-92``, ``test/test_cuda.jl:3-119``:
x known, d = A x, recover x within 10*sqrt(eps(T))*||x||) restated with a
platform-independent generator, against the independent dense Cholesky, and
the planner against the level tables derived from ``gpu_batched.jl``.

Array conventions used throughout the Python side:

* "math" blocks: ``A[i]`` is the n x n matrix A_i itself (numpy C order).
* "storage" (Julia column-major, what the C ABI and device buffers hold):
  ``A_tensor`` n x n x N column-major == numpy C-order array of shape
  (N, n, n) holding ``A[i].T``; ``d_tensor`` n x k x N == shape (N, k, n)
  holding ``d[i].T`` (d[i] is n x k).
"""
from __future__ import annotations

import hashlib
import math

import numpy as np

try:  # scipy is present on both the build host and the GPU host
    import scipy.linalg as sla
    from scipy.linalg import blas as _blas
    from scipy.linalg import lapack as _lapack
except Exception:  # pragma: no cover - scipy missing: only the planner works
    sla = None
    _blas = None
    _lapack = None


# ----------------------------------------------------------------------------
# planner: gpu_batched.jl:112-162
# ----------------------------------------------------------------------------
def build_sequence(start: int):
    """Restates ``_build_sequence`` (gpu_batched.jl:112-143).

    Walks from ``start`` toward coarser levels: for the current level size
    Ncur, pick the smallest m in 3..(Ncur-3)//2 with (Ncur+m) % (m+1) == 0 and
    Pprev = (Ncur+m)/(m+1) >= 3, preferring m < Pprev (gpu_batched.jl:124-126)
    and otherwise the first valid m (:127-129, :133-135).  Returns
    (P_list, N_list, m_list) ordered coarsest -> finest.
    """
    P_list, N_list, m_list = [], [], []
    ncur = int(start)
    while True:
        best = None
        backup = None
        # Julia's ``(Ncur - 3) ÷ 2`` truncates toward zero; for Ncur < 9 the
        # range 3:max_m is empty under either rounding, so // is equivalent.
        max_m = int((ncur - 3) / 2) if ncur < 3 else (ncur - 3) // 2
        for m in range(3, max_m + 1):
            num = ncur + m
            den = m + 1
            if num % den == 0:
                pprev = num // den
                if pprev >= 3:
                    if m < pprev:
                        best = (m, pprev)
                        break
                    elif backup is None:
                        backup = (m, pprev)
        if best is None and backup is not None:
            best = backup
        if best is None:
            break
        P_list.insert(0, best[1])
        N_list.insert(0, ncur)
        m_list.insert(0, best[0])
        ncur = best[1]
    return P_list, N_list, m_list


def find_sequence_upper(N: int):
    """Restates ``find_sequence_upper`` (gpu_batched.jl:155-162): the first
    N_use >= N for which ``build_sequence`` is non-empty.  Returns
    (P_list, N_list, m_list); N_use == N_list[-1]."""
    n_use = int(N)
    while True:
        P, Nl, ml = build_sequence(n_use)
        if P:
            return P, Nl, ml
        n_use += 1


def reference_plan(N: int):
    """Finest-first level list [(N_l, m_l, P_l), ...] plus the coarsest
    sequential size, as ``initialize_batched`` builds it (gpu_batched.jl:165-182)."""
    P, Nl, ml = find_sequence_upper(N)
    levels = list(zip(Nl, ml, P))[::-1]
    return levels, P[0]


# ----------------------------------------------------------------------------
# layout helpers
# ----------------------------------------------------------------------------
def to_storage(blocks: np.ndarray) -> np.ndarray:
    """math blocks (N, r, c) -> Julia column-major storage (N, c, r); always a
    fresh C-contiguous copy (a k = 1 swap is already contiguous, and callers
    solve in place on the result)."""
    return np.array(np.swapaxes(blocks, 1, 2), order="C", copy=True)


def from_storage(stor: np.ndarray) -> np.ndarray:
    """Julia column-major storage (N, c, r) -> math blocks (N, r, c) (a copy)."""
    return np.array(np.swapaxes(stor, 1, 2), order="C", copy=True)


# ----------------------------------------------------------------------------
# generators
# ----------------------------------------------------------------------------
_M64 = np.uint64(0xFFFFFFFFFFFFFFFF)


def _mix64(x: np.ndarray) -> np.ndarray:
    """splitmix64 finaliser on a uint64 array (wrapping arithmetic)."""
    with np.errstate(over="ignore"):
        x = x.astype(np.uint64, copy=True)
        x ^= x >> np.uint64(30)
        x *= np.uint64(0xBF58476D1CE4E5B9)
        x ^= x >> np.uint64(27)
        x *= np.uint64(0x94D049BB133111EB)
        x ^= x >> np.uint64(31)
    return x


def _bits(seed: int, stream: int, count: int, nbits: int) -> np.ndarray:
    with np.errstate(over="ignore"):
        key = _mix64(np.array([(seed * 0x9E3779B97F4A7C15 + stream * 0xD1B54A32D192ED03)
                               & 0xFFFFFFFFFFFFFFFF], dtype=np.uint64))[0]
        idx = np.arange(count, dtype=np.uint64) * np.uint64(0x9E3779B97F4A7C15) + key
    return (_mix64(idx) >> np.uint64(64 - nbits)).astype(np.int64)


def dyadic_normal(seed: int, stream: int, shape) -> np.ndarray:
    """Approximately N(0,1) values that are exact dyadic rationals (Irwin-Hall
    sum of 12 16-bit uniforms, scaled by 2^-16).  Pure integer arithmetic, so
    the values are bit-identical on every platform and numpy version, and
    products/sums of a few hundred of them are exact in FP64."""
    count = int(np.prod(shape))
    u = _bits(seed, stream, count * 12, 16).reshape(count, 12).sum(axis=1)
    return ((u - 12 * 32768).astype(np.float64) / 65536.0).reshape(shape)


def dyadic_uniform(seed: int, stream: int, shape) -> np.ndarray:
    """U[0,1) values k/2^24 (exact, platform independent)."""
    count = int(np.prod(shape))
    return (_bits(seed, stream, count, 24).astype(np.float64) / 16777216.0).reshape(shape)


def gen_golden_system(seed: int, N: int, n: int, k: int = 1):
    """The reference test family (test/test_cpu.jl:15-36, test/test_cuda.jl:20-46):
    A_i = G_i G_i^T + n I, B_i ~ N(0,1), x_i ~ U[0,1), d = A x.  Drawn from the
    platform-independent dyadic generator so A and B are bit-reproducible from
    ``seed`` (G G^T is exact in FP64 for n <= 128).  Returns math blocks
    (A (N,n,n), B (N-1,n,n), x (N,n,k), d (N,n,k))."""
    G = dyadic_normal(seed, 1, (N, n, n))
    A = np.einsum("irk,ick->irc", G, G) + n * np.eye(n)[None]
    B = dyadic_normal(seed, 2, (max(N - 1, 0), n, n))
    x = dyadic_uniform(seed, 3, (N, n, k))
    d = block_matvec(A, B, x)
    return A, B, x, d


def gen_shifted_family(rng: np.random.Generator, N: int, n: int, k: int = 1,
                       diag_shift: float | None = None, b_scale: float = 1.0,
                       rhs: str = "uniform"):
    """The G G^T + shift family (the reference tests' generator) with numpy's Generator:
    A_i = G G^T + shift*I (shift = n by default), B_i = b_scale*N(0,1),
    d ~ U[0,1) n x k (rhs='uniform') or d ~ N(0,1) (rhs='normal')."""
    shift = float(n if diag_shift is None else diag_shift)
    G = rng.standard_normal((N, n, n))
    A = G @ np.swapaxes(G, 1, 2) + shift * np.eye(n)[None]
    B = b_scale * rng.standard_normal((max(N - 1, 0), n, n))
    if rhs == "uniform":
        d = rng.random((N, n, k))
    else:
        d = rng.standard_normal((N, n, k))
    return A, B, d


def _rand_orth(rng, count, n):
    Q, R = np.linalg.qr(rng.standard_normal((count, n, n)))
    s = np.sign(np.diagonal(R, axis1=1, axis2=2))
    s[s == 0] = 1.0
    return Q * s[:, None, :]


def gen_logspectrum(rng: np.random.Generator, N: int, n: int, k: int = 4,
                lam_min: float = 1.0, lam_max: float = 1e4):
    """Wide-block workload: A_i = Q_i diag(lambda) Q_i^T, lambda log-spaced over
    [lam_min, lam_max]; B_i = 0.45*lam_min*U_i V_i^T (U, V random orthogonal);
    d ~ N(0,1) n x k.  ||B_i|| = 0.45 lam_min so A is SPD by diagonal dominance
    of the spectrum (lambda_min(A) >= lam_min - 2*0.45*lam_min)."""
    lam = np.logspace(math.log10(lam_min), math.log10(lam_max), n)
    Q = _rand_orth(rng, N, n)
    A = (Q * lam[None, None, :]) @ np.swapaxes(Q, 1, 2)
    A = 0.5 * (A + np.swapaxes(A, 1, 2))
    U = _rand_orth(rng, max(N - 1, 0), n)
    V = _rand_orth(rng, max(N - 1, 0), n)
    B = 0.45 * lam_min * (U @ np.swapaxes(V, 1, 2))
    d = rng.standard_normal((N, n, k))
    return A, B, d


def gen_kalman_model(rng: np.random.Generator, N: int, n: int, k: int = 1):
    """Kalman-smoother workload model (normal equations):
    F ~ N(0,1) rescaled to spectral radius 0.95, H ~ N(0,1) (n/2 x n),
    Q = 0.1 I, R = 0.5 I, k observation sequences Y (N, m, k) simulated from
    the model (benchmark/benchmark_kf.jl:79-102 form).  Returns
    (F, H, Qinv, Rinv, Y)."""
    m = max(n // 2, 1)
    F = rng.standard_normal((n, n))
    F *= 0.95 / max(np.max(np.abs(np.linalg.eigvals(F))), 1e-30)
    H = rng.standard_normal((m, n))
    Y = np.empty((N, m, k))
    for j in range(k):
        xs = np.zeros(n)
        for i in range(N):
            xs = F @ xs + math.sqrt(0.1) * rng.standard_normal(n)
            Y[i, :, j] = H @ xs + math.sqrt(0.5) * rng.standard_normal(m)
    return F, H, np.eye(n) / 0.1, np.eye(m) / 0.5, Y


def gen_kalman(rng: np.random.Generator, N: int, n: int, k: int = 1):
    """Kalman-smoother workload blocks, uniform: A_i = Q^-1 + F^T Q^-1 F + H^T R^-1 H,
    B_i = -F^T Q^-1, d_i = H^T R^-1 y_i (benchmark/benchmark_kf.jl:79-102,
    147-150 form) from gen_kalman_model."""
    F, H, Qinv, Rinv, Y = gen_kalman_model(rng, N, n, k)
    return kf_blocks(F, H, Qinv, Rinv, Y)


def kf_blocks(F, H, Qinv, Rinv, Y, P0inv=None, x0=None):
    """Normal equations of the Kalman smoother, restating build_kf_blocks
    (benchmark/benchmark_kf.jl:105-154) with the inverses given:
    F (n,n), H (m,n), Qinv (n,n), Rinv (m,m), Y (N,m,k) -> A (N,n,n),
    B (N-1,n,n), d (N,n,k).  With P0inv: A_1 += P0inv (no Q^-1), A_N has no
    F^T Q^-1 F (the reference's boundary blocks); without it every A_i is
    H^T R^-1 H + Q^-1 + F^T Q^-1 F.  A_i is taken from its upper triangle
    (Symmetric(Akk))."""
    N = Y.shape[0]
    n = F.shape[0]
    QF = Qinv @ F
    FQF = F.T @ QF
    HRH = H.T @ (Rinv @ H)
    Bup = -QF.T

    def sym_upper(M):
        U = np.triu(M)
        return U + np.triu(M, 1).T

    Aint = sym_upper(HRH + Qinv + FQF)
    if P0inv is not None:
        Afirst = sym_upper(HRH + P0inv + FQF)
        Alast = sym_upper(HRH + Qinv)
    else:
        Afirst = Alast = Aint
    A = np.broadcast_to(Aint, (N, n, n)).copy()
    A[0] = Afirst
    if N > 1:
        A[N - 1] = Alast
    B = np.broadcast_to(Bup, (max(N - 1, 0), n, n)).copy()
    RH = Rinv @ H
    d = np.einsum("mn,imk->ink", RH, Y)
    if P0inv is not None and x0 is not None:
        d[0] += (P0inv @ x0)[:, None]
    return A, B, d


def input_digest(A: np.ndarray, B: np.ndarray) -> str:
    h = hashlib.sha256()
    h.update(np.ascontiguousarray(A, dtype=np.float64).tobytes())
    h.update(np.ascontiguousarray(B, dtype=np.float64).tobytes())
    return h.hexdigest()


# ----------------------------------------------------------------------------
# operator, residual, norms
# ----------------------------------------------------------------------------
def block_matvec(A: np.ndarray, B: np.ndarray, x: np.ndarray) -> np.ndarray:
    """y = T x for the block-tridiagonal T (diag A_i, super B_i, sub B_i^T);
    x is (N, n, k) math blocks."""
    y = A @ x
    if B.shape[0]:
        y[:-1] += B @ x[1:]
        y[1:] += np.swapaxes(B, 1, 2) @ x[:-1]
    return y


def operator_inf_norm(A: np.ndarray, B: np.ndarray) -> float:
    """||T||_inf = max row sum of |T| over the block-tridiagonal operator."""
    rs = np.abs(A).sum(axis=2)
    if B.shape[0]:
        rs[:-1] += np.abs(B).sum(axis=2)
        rs[1:] += np.abs(B).sum(axis=1)
    return float(rs.max())


def rel_residual(A, B, x, d) -> float:
    """||d - T x||_inf / (||T||_inf ||x||_inf + ||d||_inf), all in FP64."""
    A = np.asarray(A, np.float64)
    B = np.asarray(B, np.float64)
    x = np.asarray(x, np.float64)
    d = np.asarray(d, np.float64)
    r = d - block_matvec(A, B, x)
    den = operator_inf_norm(A, B) * np.abs(x).max() + np.abs(d).max()
    return float(np.abs(r).max() / den) if den > 0 else 0.0


def rel_error(x, x_ref) -> float:
    """Frobenius norm over blocks, as ``_bss_norm`` (test/test_cpu.jl:1-7)."""
    x = np.asarray(x, np.float64)
    x_ref = np.asarray(x_ref, np.float64)
    den = np.linalg.norm(x_ref.ravel())
    return float(np.linalg.norm((x - x_ref).ravel()) / (den if den > 0 else 1.0))


# ----------------------------------------------------------------------------
# sequential block Cholesky: backbone_cpu.jl:5-33 (cpu.jl:30-50)
# ----------------------------------------------------------------------------
def _pfx(dtype):
    return "d" if np.dtype(dtype) == np.float64 else "s"


def _potrf_upper(a):
    f = getattr(_lapack, _pfx(a.dtype) + "potrf")
    c, info = f(a, lower=0, clean=0, overwrite_a=0)
    if info != 0:
        raise np.linalg.LinAlgError(f"potrf info={info}")
    return c


def _trsm(a, b, trans):
    # trsm!('L','U',trans,'N', 1, a, b): solve op(U) X = b
    f = getattr(_blas, _pfx(a.dtype) + "trsm")
    return f(1.0, a, b, side=0, lower=0, trans_a=trans, diag=0)


def _gemm(alpha, a, b, beta, c, trans_a, trans_b):
    f = getattr(_blas, _pfx(a.dtype) + "gemm")
    return f(alpha, a, b, beta, c, trans_a=trans_a, trans_b=trans_b)


def cholesky_factorize(A: np.ndarray, B: np.ndarray) -> None:
    """In place, math blocks.  backbone_cpu.jl:5-15:
    potrf!('U', A_1); for i = 2..N: trsm!('L','U','T','N', 1, A_{i-1}, B_{i-1});
    gemm!('T','N', -1, B_{i-1}, B_{i-1}, 1, A_i); potrf!('U', A_i)."""
    N = A.shape[0]
    A[0] = _potrf_upper(A[0])
    for i in range(1, N):
        B[i - 1] = _trsm(A[i - 1], B[i - 1], 1)
        A[i] = _gemm(-1.0, B[i - 1], B[i - 1], 1.0, A[i], 1, 0)
        A[i] = _potrf_upper(A[i])


def cholesky_solve(A: np.ndarray, B: np.ndarray, d: np.ndarray) -> None:
    """In place on d (N, n, k).  backbone_cpu.jl:17-33."""
    N = A.shape[0]
    d[0] = _trsm(A[0], d[0], 1)
    for i in range(1, N):
        d[i] = _gemm(-1.0, B[i - 1], d[i - 1], 1.0, d[i], 1, 0)
        d[i] = _trsm(A[i], d[i], 1)
    d[N - 1] = _trsm(A[N - 1], d[N - 1], 0)
    for i in range(N - 2, -1, -1):
        d[i] = _gemm(-1.0, B[i], d[i + 1], 1.0, d[i], 0, 0)
        d[i] = _trsm(A[i], d[i], 0)


def cpu_solve(A, B, d, dtype=np.float64):
    """initialize_cpu + factorize! + solve! (cpu.jl) on copies; returns x."""
    A = np.array(A, dtype=dtype, order="C")
    B = np.array(B, dtype=dtype, order="C")
    x = np.array(d, dtype=dtype, order="C")
    # scipy BLAS wants Fortran-ordered operands for zero-copy; per-block copies
    # are small, correctness does not depend on it.
    cholesky_factorize(A, B)
    cholesky_solve(A, B, x)
    return x


# ----------------------------------------------------------------------------
# dense FP64 Cholesky of the assembled matrix (test/utils.jl:32-74 convention)
# ----------------------------------------------------------------------------
def assemble_dense(A: np.ndarray, B: np.ndarray) -> np.ndarray:
    N, n, _ = A.shape
    M = np.zeros((N * n, N * n))
    for i in range(N):
        M[i * n:(i + 1) * n, i * n:(i + 1) * n] = A[i]
        if i + 1 < N:
            M[i * n:(i + 1) * n, (i + 1) * n:(i + 2) * n] = B[i]
            M[(i + 1) * n:(i + 2) * n, i * n:(i + 1) * n] = B[i].T
    return M


def construct_block_tridiagonal(A: np.ndarray, B: np.ndarray, d: np.ndarray | None = None):
    """benchmark/utils.jl:59-103: the (N n) x (N n) matrix as coordinate
    triples (I, J, V), pushed for every entry of every stored block in the
    reference's loop order (block row i, block column j in {i-1, i, i+1}
    with A_i, B_i or B_{j}^T, then row, then column), turned into compressed
    rows: returns ``(row_ptr, col_idx, vals, d_vec)`` with 0-based int32
    indices, columns ascending within a row, explicit zeros kept (as
    Julia's ``sparse(I, J, V)`` keeps them), d_vec = vcat(d_list...) of shape
    (N n, k) or None.  Bit-exact: the values are copies of the block entries.
    """
    A = np.asarray(A)
    N, n, _ = A.shape
    I_parts, J_parts, V_parts = [], [], []
    rr, cc = np.meshgrid(np.arange(n), np.arange(n), indexing="ij")
    for i in range(N):                       # utils.jl:72
        for j in (i - 1, i, i + 1):          # utils.jl:74-86 (other blocks skipped)
            if j < 0 or j >= N:
                continue
            if j == i:
                blk = A[i]
            elif j == i + 1:
                blk = B[i]
            else:
                blk = B[j].T
            I_parts.append((i * n + rr).ravel())   # utils.jl:89-94: row-major pushes
            J_parts.append((j * n + cc).ravel())
            V_parts.append(np.asarray(blk).ravel())
    I = np.concatenate(I_parts)
    J = np.concatenate(J_parts)
    V = np.concatenate(V_parts)
    order = np.lexsort((J, I))               # compressed rows, columns ascending
    I, J, V = I[order], J[order], V[order]
    if I.size > 1:
        dup = (I[1:] == I[:-1]) & (J[1:] == J[:-1])
        assert not dup.any(), "block pattern has no duplicate coordinates"
    row_ptr = np.zeros(N * n + 1, dtype=np.int64)
    np.add.at(row_ptr, I + 1, 1)
    row_ptr = np.cumsum(row_ptr).astype(np.int32)
    d_vec = None
    if d is not None:
        d = np.asarray(d)
        d_vec = d.reshape(N * n, d.shape[2])  # utils.jl:100: vcat(d_list...)
    return row_ptr, J.astype(np.int32), V, d_vec


def dense_solve(A, B, d) -> np.ndarray:
    N, n, _ = A.shape
    k = d.shape[2]
    M = assemble_dense(np.asarray(A, np.float64), np.asarray(B, np.float64))
    rhs = np.asarray(d, np.float64).reshape(N * n, k)
    c = sla.cho_factor(M, lower=False)
    return sla.cho_solve(c, rhs).reshape(N, n, k)


# ----------------------------------------------------------------------------
# reference batched algorithm: gpu_batched.jl:184-258 + backbone_cuda.jl:70-184
# ----------------------------------------------------------------------------
def _chain_factor_ref(A, B, idx, m):
    """cholesky_factorize_batched! (backbone_cuda.jl:70-101) for one partition:
    interior blocks idx..idx+m-1 (0-based); the first block is potrf'd with no
    left coupling; B between interior blocks becomes U^-T B."""
    A[idx] = _potrf_upper(A[idx])
    for i in range(idx + 1, idx + m):
        B[i - 1] = _trsm(A[i - 1], B[i - 1], 1)
        A[i] = _gemm(-1.0, B[i - 1], B[i - 1], 1.0, A[i], 1, 0)
        A[i] = _potrf_upper(A[i])


def _chain_solve_ref(A, B, X, idx, m):
    """cholesky_solve_batched! (backbone_cuda.jl:103-141) for one partition,
    X[idx..idx+m-1] (each n x nd) in place."""
    X[idx] = _trsm(A[idx], X[idx], 1)
    for i in range(idx + 1, idx + m):
        X[i] = _gemm(-1.0, B[i - 1], X[i - 1], 1.0, X[i], 1, 0)
        X[i] = _trsm(A[i], X[i], 1)
    for i in range(idx + m - 1, idx, -1):
        X[i] = _trsm(A[i], X[i], 0)
        X[i - 1] = _gemm(-1.0, B[i - 1], X[i], 1.0, X[i - 1], 0, 0)
    X[idx] = _trsm(A[idx], X[idx], 0)


class RefBatchedLevel:
    """One level of ``BlockTriDiagData_batched`` (gpu_batched.jl:1-71) holding
    the quantities the reference computes, for intermediate-value parity."""

    def __init__(self, N, m, P, n, dtype):
        self.N, self.m, self.P, self.n = N, m, P, n
        self.dtype = dtype
        self.M1 = self.M2 = self.F = self.LHS_A = self.LHS_B = None


def batched_factorize(A, B, plan_levels, dtype=np.float64):
    """Restates factorize!(BlockTriDiagData_batched) (gpu_batched.jl:184-227)
    level by level.  ``A`` (N_use,n,n), ``B`` (N_use-1,n,n) math blocks are
    factored in place.  Returns the per-level state list (finest first) plus
    the coarsest (A, B) pair which is factored sequentially
    (gpu_seq.jl:61-71 -> backbone_cuda.jl:14-37)."""
    levels = []
    curA, curB = A, B
    n = A.shape[1]
    for (N, m, P) in plan_levels:
        L = RefBatchedLevel(N, m, P, n, dtype)
        seps = list(range(0, N, m + 1))           # 1:(m+1):N (1-based)
        assert len(seps) == P and seps[-1] == N - 1
        L.M1 = np.array([curB[s] for s in seps[:-1]])            # B[:,:,1:(m+1):N-1]
        L.M2 = np.array([curB[s + m] for s in seps[:-1]])        # B[:,:,(m+1):(m+1):N-1]
        L.LHS_A = np.array([curA[s] for s in seps])
        L.LHS_B = np.zeros((P - 1, n, n), dtype=dtype)
        # G/F: n x 2n per block, nonzero at first/last interior blocks
        L.F = np.zeros((N, n, 2 * n), dtype=dtype)
        for p, s in enumerate(seps[:-1]):
            L.F[s + 1][:, :n] = L.M1[p].T
            L.F[s + m][:, n:] += L.M2[p]
        G = L.F.copy()
        for s in seps[:-1]:
            _chain_factor_ref(curA, curB, s + 1, m)
        for s in seps[:-1]:
            _chain_solve_ref(curA, curB, L.F, s + 1, m)
        for p, s in enumerate(seps[:-1]):                      # compute_schur_complement!
            M2n = np.zeros((2 * n, 2 * n), dtype=dtype)
            for j in range(1, m + 1):
                M2n = _gemm(1.0, G[s + j], L.F[s + j], 1.0, M2n, 1, 0)
            L.LHS_A[p] -= M2n[:n, :n]
            L.LHS_A[p + 1] -= M2n[n:, n:]
            L.LHS_B[p] -= M2n[:n, n:]
        L.A, L.B = curA, curB
        levels.append(L)
        curA = L.LHS_A.copy()
        curB = L.LHS_B.copy()
    cholesky_factorize(curA, curB)                              # coarsest seq level
    return levels, (curA, curB)


def batched_solve(d, levels, coarsest):
    """Restates solve!(BlockTriDiagData_batched) (gpu_batched.jl:229-258) on
    the factored state from ``batched_factorize``; d (N_use,n,1) in place."""
    if not levels:
        cholesky_solve(coarsest[0], coarsest[1], d)
        return
    L = levels[0]
    A, B = L.A, L.B
    rest = levels[1:]
    N, m, P, n = L.N, L.m, L.P, L.n
    seps = list(range(0, N, m + 1))
    b = np.zeros((P - 1, 2 * n, d.shape[2]), dtype=d.dtype)
    for p, s in enumerate(seps[:-1]):                          # compute_schur_RHS!
        for j in range(1, m + 1):
            b[p] = _gemm(-1.0, L.F[s + j], d[s + j], 1.0, b[p], 1, 0)
    for p, s in enumerate(seps[:-1]):
        d[s] += b[p][:n]
        d[s + m + 1] += b[p][n:]
    dn = np.array([d[s] for s in seps])
    batched_solve(dn, rest, coarsest)
    for q, s in enumerate(seps):
        d[s] = dn[q]
    for p, s in enumerate(seps[:-1]):                          # update_boundary!
        d[s + 1] = _gemm(-1.0, L.M1[p], d[s], 1.0, d[s + 1], 1, 0)
        d[s + m] = _gemm(-1.0, L.M2[p], d[s + m + 1], 1.0, d[s + m], 0, 0)
    for s in seps[:-1]:
        _chain_solve_ref(A, B, d, s + 1, m)


def batched_reference_solve(A, B, d, N_user=None, dtype=np.float64):
    """initialize_batched + copyto! + factorize! + solve! on copies, following
    the reference's padding (identity A, zero B/d for blocks N_user..N_use,
    gpu_batched.jl:177-179).  Returns (x (N_user,n,k), levels, plan)."""
    N = A.shape[0] if N_user is None else N_user
    n = A.shape[1]
    plan_levels, pc = reference_plan(N)
    n_use = plan_levels[0][0] if plan_levels else pc
    k = d.shape[2]
    Au = np.zeros((n_use, n, n), dtype=dtype)
    Au[:] = np.eye(n, dtype=dtype)
    Bu = np.zeros((n_use - 1, n, n), dtype=dtype)
    du = np.zeros((n_use, n, k), dtype=dtype)
    Au[:N] = A
    Bu[:N - 1] = B
    du[:N] = d
    levels, coarsest = batched_factorize(Au, Bu, plan_levels, dtype)
    # the reference batched path is k = 1 only (gpu_batched.jl:78,91,257);
    # the restatement loops the columns.
    for j in range(k):
        col = np.ascontiguousarray(du[:, :, j:j + 1])
        batched_solve(col, levels, coarsest)
        du[:, :, j:j + 1] = col
    return du[:N], levels, (plan_levels, pc)
