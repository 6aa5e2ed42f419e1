"""CPU tests of the oracle: pins it to the reference before it is trusted.

* planner restatement vs the level tables derived from gpu_batched.jl:112-162
  and its invariants;
* the C restatement of backbone_cpu.jl (OpenBLAS) vs the committed golden
  fixtures, vs the reference's own known-answer criterion
  (test/test_cpu.jl:53-92: ||x^ - x|| <= 10 sqrt(eps) ||x||, residual
  <= 10 sqrt(eps) ||d||) and vs an independent dense Cholesky;
* the numpy restatement of the batched algorithm (gpu_batched.jl) vs the
  sequential one and the fixtures' separator systems.
"""
import glob
import json
import os

import numpy as np
import pytest

from oracle import cref
from oracle import oracle as O

GOLD = os.path.join(os.path.dirname(__file__), "golden")
FIXTURES = sorted(glob.glob(os.path.join(GOLD, "*.npz")))


def _fix(path):
    z = np.load(path)
    N, n, k, seed = int(z["N"]), int(z["n"]), int(z["k"]), int(z["seed"])
    A, B, x, d = O.gen_golden_system(seed, N, n, k)
    return z, A, B, x, d


# the level tables of gpu_batched.jl:112-162 for the sizes the reference's
# tests and benchmarks use (N_l, m_l, P_l finest first; coarsest size)
PLAN_TABLE = {
    50: ([(50, 6, 8)], 8),
    100: ([(100, 8, 12)], 12),
    16384: ([(16384, 42, 382), (382, 126, 4)], 4),
    65536: ([(65536, 4, 13108), (13108, 16, 772), (772, 256, 4)], 4),
    2: ([(9, 3, 3)], 3),
    8: ([(9, 3, 3)], 3),
    9: ([(9, 3, 3)], 3),
}


@pytest.mark.parametrize("N", sorted(PLAN_TABLE))
def test_planner_table(N):
    assert O.reference_plan(N) == PLAN_TABLE[N]


def test_planner_5000_pads_one_block():
    levels, coarse = O.reference_plan(5000)
    assert levels[0][0] == 5001 and len(levels) == 5 and coarse == 3
    assert all(m in (3, 4) for (_, m, _) in levels)


def _brute_m(ncur):
    """Direct reading of gpu_batched.jl:118-135 for one level."""
    cands = [(m, (ncur + m) // (m + 1)) for m in range(3, (ncur - 3) // 2 + 1)
             if (ncur + m) % (m + 1) == 0 and (ncur + m) // (m + 1) >= 3]
    pref = [c for c in cands if c[0] < c[1]]
    return pref[0] if pref else (cands[0] if cands else None)


def test_planner_invariants_sweep():
    for N in range(1, 1500):
        levels, coarse = O.reference_plan(N)
        assert levels[0][0] >= N
        for i, (Nl, m, P) in enumerate(levels):
            assert Nl == (P - 1) * (m + 1) + 1 and m >= 3 and P >= 3
            assert _brute_m(Nl) == (m, P)
            nxt = levels[i + 1][0] if i + 1 < len(levels) else coarse
            assert nxt == P
        assert _brute_m(coarse) is None
        # smallest padded size: every N' in [N, N_use) has no plan
        for Np in range(N, levels[0][0]):
            assert _brute_m(Np) is None


def test_fixtures_present():
    assert len(FIXTURES) >= 8


@pytest.mark.parametrize("path", FIXTURES, ids=lambda p: os.path.basename(p)[:-4])
def test_golden_inputs_regenerate(path):
    z, A, B, x, d = _fix(path)
    assert O.input_digest(A, B) == str(z["digest"])
    np.testing.assert_array_equal(x, z["x_true"])
    # d is stored (A x is not exact in FP64); it must be A x to rounding
    assert O.rel_error(O.block_matvec(A, B, x), z["d"]) < 1e-15


@pytest.mark.parametrize("path", FIXTURES, ids=lambda p: os.path.basename(p)[:-4])
def test_c_oracle_matches_golden(path):
    z, A, B, x, d = _fix(path)
    d = z["d"]
    xc = cref.solve_math(A, B, d, np.float64)
    eps64 = np.finfo(np.float64).eps
    assert O.rel_error(xc, z["x_cpu_f64"]) < 1e-12
    assert O.rel_error(xc, z["x_dense"]) < 1e-12
    # the reference's known-answer criterion, test/test_cpu.jl:53,71,92
    assert O.rel_error(xc, x) <= 10 * np.sqrt(eps64)
    r = O.block_matvec(A, B, xc) - d
    assert np.linalg.norm(r.ravel()) <= 10 * np.sqrt(eps64) * np.linalg.norm(d.ravel())
    x32 = cref.solve_math(A, B, d, np.float32)
    eps32 = np.finfo(np.float32).eps
    assert O.rel_error(x32, x) <= 10 * np.sqrt(eps32)
    assert O.rel_error(x32, z["x_cpu_f32"]) < 1e-5


@pytest.mark.parametrize("path", FIXTURES, ids=lambda p: os.path.basename(p)[:-4])
def test_numpy_and_port_oracles_agree(path):
    z, A, B, x, d = _fix(path)
    d = z["d"]
    xn = O.cpu_solve(A, B, d)
    xp = cref.solve_math(A, B, d, np.float64, use_blas=False)
    assert O.rel_error(xn, z["x_cpu_f64"]) < 1e-12
    assert O.rel_error(xp, z["x_cpu_f64"]) < 1e-12


@pytest.mark.parametrize("path", FIXTURES, ids=lambda p: os.path.basename(p)[:-4])
def test_batched_restatement_matches_golden(path):
    z, A, B, x, d = _fix(path)
    d = z["d"]
    xb, levels, (plan_levels, pc) = O.batched_reference_solve(A, B, d)
    assert [tuple(p) for p in z["plan"].tolist()] == [tuple(p) for p in plan_levels]
    assert O.rel_error(xb, z["x_dense"]) < 1e-12
    if levels:
        scale = np.abs(z["lhs_A"]).max()
        assert np.abs(levels[0].LHS_A - z["lhs_A"]).max() <= 1e-12 * scale
        assert np.abs(levels[0].LHS_B - z["lhs_B"]).max() <= 1e-12 * scale


@pytest.mark.parametrize("T", [np.float64, np.float32])
def test_reference_known_answer_numpy_rng(T):
    """test/test_cpu.jl:9-92 with numpy's RNG (Julia's stream cannot be
    reproduced): N=50, n=32, both precisions."""
    rng = np.random.default_rng(42)
    N, n = 50, 32
    G = rng.standard_normal((N, n, n))
    A = G @ np.swapaxes(G, 1, 2) + n * np.eye(n)
    B = rng.standard_normal((N - 1, n, n))
    x = rng.random((N, n, 1))
    d = O.block_matvec(A, B, x)
    xs = cref.solve_math(A.astype(T), B.astype(T), d.astype(T), T)
    eps = np.sqrt(np.finfo(T).eps)
    assert O.rel_error(xs, x) <= 10 * eps
    r = O.block_matvec(A.astype(T), B.astype(T), xs.astype(T)) - d.astype(T)
    assert np.linalg.norm(r.ravel()) <= 10 * eps * np.linalg.norm(d.ravel())


def test_batched_restatement_intermediate_system_is_schur_complement():
    """The separator system after one level equals the exact Schur complement
    of the interior blocks (dense check of gpu_batched.jl:184-227)."""
    A, B, x, d = O.gen_golden_system(3, 23, 4, 1)
    plan, pc = O.reference_plan(23)
    levels, _ = O.batched_factorize(A.copy(), B.copy(), plan)
    Nl, m, P = plan[0]
    M = O.assemble_dense(A, B)
    n = 4
    seps = list(range(0, Nl, m + 1))
    sidx = np.concatenate([np.arange(s * n, (s + 1) * n) for s in seps])
    iidx = np.setdiff1d(np.arange(Nl * n), sidx)
    S = M[np.ix_(sidx, sidx)] - M[np.ix_(sidx, iidx)] @ np.linalg.solve(M[np.ix_(iidx, iidx)],
                                                                        M[np.ix_(iidx, sidx)])
    Sa = O.assemble_dense(levels[0].LHS_A, levels[0].LHS_B)
    assert np.abs(S - Sa).max() < 1e-10 * np.abs(S).max()


def test_summary_json_consistent():
    with open(os.path.join(GOLD, "golden_summary.json")) as f:
        js = json.load(f)
    for N, ent in js["planner"].items():
        levels, coarse = O.reference_plan(int(N))
        assert [list(l) for l in levels] == ent["levels"] and coarse == ent["coarsest"]


@pytest.mark.parametrize("N,n,k", [(1, 4, 1), (2, 3, 2), (7, 5, 1), (12, 8, 3), (5, 33, 1)])
def test_sparse_assembly_restatement(N, n, k):
    """construct_block_tridiagonal (benchmark/utils.jl:59-103) restated:
    the CSR matrix equals the dense assembly entry for entry, every block
    entry is stored (nnz = n^2 (3N - 2), explicit zeros kept), rows are
    sorted, d_vec = vcat(d_list...), and scipy's own COO -> CSR conversion
    of the same triples gives the same arrays."""
    rng = np.random.default_rng(N * 100 + n)
    A = rng.standard_normal((N, n, n))
    B = rng.standard_normal((max(N - 1, 0), n, n))
    if N > 1:
        B[0, 0, :] = 0.0  # explicit zeros stay stored
    d = rng.standard_normal((N, n, k))
    rp, ci, v, dv = O.construct_block_tridiagonal(A, B, d)
    assert rp.dtype == np.int32 and ci.dtype == np.int32
    assert rp[-1] == n * n * (3 * N - 2) == ci.size == v.size
    M = O.assemble_dense(A, B)
    dense = np.zeros_like(M)
    for R in range(N * n):
        cols = ci[rp[R]:rp[R + 1]]
        assert np.all(np.diff(cols) > 0)
        dense[R, cols] = v[rp[R]:rp[R + 1]]
    assert np.array_equal(dense, M)
    assert np.array_equal(dv, np.concatenate([d[i] for i in range(N)], axis=0))
    sp = pytest.importorskip("scipy.sparse")
    rows = np.repeat(np.arange(N * n), np.diff(rp))
    C = sp.coo_matrix((v, (rows, ci)), shape=M.shape).tocsr()
    C.sort_indices()
    assert np.array_equal(C.indptr, rp) and np.array_equal(C.indices, ci) and np.array_equal(C.data, v)


def _split_df_restated(a):
    """The double-float split of the refinement residual kernel restated on
    the bit patterns: a_hi = a truncated to 24 significant bits (exponent
    rebiased, top 23 mantissa bits), a_lo = the next 23 bits scaled by
    a_hi's signed power of two; |a| < 2^-126 -> (0, 0)."""
    b = np.ascontiguousarray(a, np.float64).view(np.uint64)
    hi = (b >> np.uint64(32)).astype(np.uint64)
    lo = (b & np.uint64(0xFFFFFFFF)).astype(np.uint64)
    mag = hi & np.uint64(0x7FFFFFFF)
    t = (mag - np.uint64(0x38000000)) & np.uint64(0xFFFFFFFF)
    hb0 = (((t << np.uint64(3)) | (lo >> np.uint64(29))) & np.uint64(0xFFFFFFFF)) | (hi & np.uint64(0x80000000))
    hb = np.where(mag < np.uint64(0x38100000), np.uint64(0), hb0).astype(np.uint32)
    magic = (((lo >> np.uint64(6)) & np.uint64(0x7FFFFF)) | np.uint64(0x4B000000)).astype(np.uint32)
    q = (magic.view(np.float32).astype(np.float64) * 2.0 ** -46 - 2.0 ** -23).astype(np.float32)
    assert np.all(q.astype(np.float64) == magic.view(np.float32).astype(np.float64) * 2.0 ** -46 - 2.0 ** -23)
    hbe = (hb & np.uint32(0xFF800000)).view(np.float32)
    return hb.view(np.float32), (q * hbe).astype(np.float32)


def test_double_float_split_bits():
    rng = np.random.default_rng(5)
    a = rng.standard_normal(20000) * 2.0 ** rng.integers(-90, 91, size=20000)
    a = np.concatenate([a, [0.0, -0.0, 1.0, -1.0, 2.0 ** -126, 3.0 * 2.0 ** -120, np.nextafter(1.0, 2.0)]])
    h, l = _split_df_restated(a)
    err = np.abs(a - h.astype(np.float64) - l.astype(np.float64))
    big = np.abs(a) >= 2.0 ** -100
    assert np.all(err[big] < 2.0 ** -46 * np.abs(a[big]))
    assert np.all(np.abs(h.astype(np.float64)) <= np.abs(a))      # truncation toward zero
    assert np.all(np.sign(h[a != 0]) == np.sign(a[a != 0]))
    assert h[-7] == 0.0 and l[-7] == 0.0 and h[-6] == 0.0
