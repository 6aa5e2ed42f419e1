"""Generate the golden fixtures under tests/golden/.

Each fixture is one block-tridiagonal SPD system of the reference test family
(test/test_cpu.jl:15-36: A_i = G G^T + n I, B_i ~ N(0,1), x ~ U[0,1),
d = A x), drawn from the platform-independent dyadic generator of
``oracle.oracle.gen_golden_system`` so that A and B are regenerated
bit-exactly from the seed anywhere (their SHA-256 is stored to prove it).
Stored: d, the true x, and the solutions of
  * the C restatement of backbone_cpu.jl on OpenBLAS, FP64 and FP32
    (``x_cpu_f64``, ``x_cpu_f32``),
  * the numpy restatement of the reference batched algorithm
    (gpu_batched.jl + backbone_cuda.jl, reference planner) (``x_batched``),
  * an FP64 dense Cholesky (``x_dense``),
and, for the batched restatement, the separator system of its first level
(``lhs_A``, ``lhs_B``: the reference's NextData.A_tensor / B_tensor after
factorize!), which pins the Schur-complement assembly.

Run from the repository root:  python tests/golden/make_golden.py
"""
from __future__ import annotations

import json
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

from oracle import cref  # noqa: E402
from oracle import oracle as O  # noqa: E402

HERE = os.path.dirname(os.path.abspath(__file__))

CASES = [
    # name, seed, N, n, k
    ("reftest_N50_n32_k1", 42, 50, 32, 1),
    ("cfg0_N100_n32_k1", 100, 100, 32, 1),
    ("ragged_N23_n5_k3", 7, 23, 5, 3),
    ("single_N1_n4_k1", 11, 1, 4, 1),
    ("pair_N2_n3_k2", 12, 2, 3, 2),
    ("pad_N37_n48_k2", 13, 37, 48, 2),
    ("n64_N40_k1", 14, 40, 64, 1),
    ("n16_N150_k2", 15, 150, 16, 2),
]


def make(name, seed, N, n, k):
    A, B, x, d = O.gen_golden_system(seed, N, n, k)
    x_c64 = cref.solve_math(A, B, d, np.float64)
    x_c32 = cref.solve_math(A, B, d, np.float32)
    x_dense = O.dense_solve(A, B, d)
    xb, levels, (plan_levels, pc) = O.batched_reference_solve(A, B, d)
    out = dict(
        seed=np.int64(seed), N=np.int64(N), n=np.int64(n), k=np.int64(k),
        digest=np.array(O.input_digest(A, B)),
        d=d, x_true=x, x_cpu_f64=x_c64, x_cpu_f32=x_c32.astype(np.float32),
        x_dense=x_dense, x_batched=xb,
        plan=np.array(plan_levels, dtype=np.int64).reshape(-1, 3), plan_coarsest=np.int64(pc),
    )
    if levels:
        out["lhs_A"] = levels[0].LHS_A
        out["lhs_B"] = levels[0].LHS_B
    np.savez_compressed(os.path.join(HERE, name + ".npz"), **out)
    return {
        "name": name, "N": N, "n": n, "k": k, "seed": seed,
        "err_cpu_f64_vs_true": O.rel_error(x_c64, x),
        "err_cpu_f64_vs_dense": O.rel_error(x_c64, x_dense),
        "err_batched_vs_dense": O.rel_error(xb, x_dense),
        "err_cpu_f32_vs_true": O.rel_error(x_c32, x),
        "relres_cpu_f64": O.rel_residual(A, B, x_c64, d),
        "plan": [list(map(int, p)) for p in plan_levels], "plan_coarsest": int(pc),
    }


def main():
    summary = [make(*c) for c in CASES]
    # planner table (gpu_batched.jl:112-162) for the sizes the tests and
    # benchmarks use, plus a dense sweep checked by the tests
    table = {str(N): {"levels": [list(map(int, lv)) for lv in O.reference_plan(N)[0]],
                      "coarsest": int(O.reference_plan(N)[1])}
             for N in list(range(1, 130)) + [5000, 16384, 65536]}
    with open(os.path.join(HERE, "golden_summary.json"), "w") as f:
        json.dump({"cases": summary, "planner": table}, f, indent=1)
    for s in summary:
        print(s["name"], "err vs true %.2e, vs dense %.2e, batched vs dense %.2e" % (
            s["err_cpu_f64_vs_true"], s["err_cpu_f64_vs_dense"], s["err_batched_vs_dense"]))


if __name__ == "__main__":
    main()
