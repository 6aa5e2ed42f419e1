"""Benchmark: factorize! + solve! of one block-tridiagonal SPD system,
N = 16384 blocks of n = 64, k = 1 right-hand side (
A_i = G G^T + n I, B_i ~ N(0,1), d ~ U[0,1), generated once on the host by
numpy's seeded Generator; both arms solve these same bytes).

A "step" is one complete solve request: put d into the handle, factorize!,
solve!, to a relative residual ||d - A x||_inf / (||A|| ||x|| + ||d||)
<= 1e-12.  The headline path is the mixed-precision one (FP32 chain
factorization on the sm_103a kernels + FP64 iterative refinement); the same
JSON line carries the plain FP64 and plain FP32 GPU paths for comparison.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl reference]

--impl reference times the reference's CPU path (cpu.jl / backbone_cpu.jl
restated in C on OpenBLAS, ``oracle/``) on the host cores instead.
Multi-GPU: the solver does not shard a single system across GPUs here, so
each rank runs an independent replica ("scaling": "weak").
"""
from __future__ import annotations

import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

N_BLK, N_SZ, K_RHS = 16384, 64, 1
METRIC = "solves/s (factorize!+solve!, rel-resid <= 1e-12)"
WORKLOAD = "block-tridiagonal SPD, N=16384 blocks of n=64, k=1 (A_i=G G^T+nI, B_i~N(0,1), d~U[0,1))"


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=200)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--quick", action="store_true", help="skip the secondary legs")
    ap.add_argument("--no-extra", action="store_true", help="skip the large-system (N=65536, n=128), uneven-batch and served legs")
    ap.add_argument("--case", default=None,
                    help="run one small named case for a profiler and exit: "
                         "chain_n64 (N=4096, n=64, mixed), wide_n128 (N=2048, n=128, mixed), "
                         "headline_eager (N=16384, n=64, mixed, no CUDA graphs: every kernel a launch), "
                         "csr_n64 (CSR assembly of N=4096, n=64), chain_n64_k16 (N=4096, n=64, k=16, mixed), "
                         "batch_small (64 uneven systems, mixed), batch_2048 (the 2048-system batch, mixed), "
                         "wide_n128_k4 (N=4096, n=128, k=4, mixed, no CUDA graphs), "
                         "wide_n128_k4_16k (N=16384, n=128, k=4, mixed, no CUDA graphs)")
    return ap.parse_args()


def dist_env():
    from blockstructuredsolvers_gb300 import replicas
    return replicas.rank_env()


# --------------------------------------------------------------------------
# CPU reference arm / baseline (oracle: test infrastructure, timed only here)
# --------------------------------------------------------------------------
def gen_host(seed=1):
    import numpy as np
    rng = np.random.default_rng(seed)
    G = rng.standard_normal((N_BLK, N_SZ, N_SZ))
    A = G @ np.swapaxes(G, 1, 2) + N_SZ * np.eye(N_SZ)
    B = rng.standard_normal((N_BLK - 1, N_SZ, N_SZ))
    d = rng.random((N_BLK, N_SZ, K_RHS))
    # Julia column-major storage: (N, c, r) C-order
    return (np.ascontiguousarray(np.swapaxes(A, 1, 2)), np.ascontiguousarray(np.swapaxes(B, 1, 2)),
            np.ascontiguousarray(np.swapaxes(d, 1, 2)))


def cpu_solve_time(As, Bs, ds, reps=1, threads=None):
    """Seconds per factorize!+solve! of the reference CPU path (C restatement
    of backbone_cpu.jl on OpenBLAS) on copies of the inputs."""
    from oracle import cref
    cref.lib(True)
    if threads is not None:
        cref.set_blas_threads(threads)
    ts = []
    for _ in range(reps):
        A, B, d = As.copy(), Bs.copy(), ds.copy()
        t0 = time.perf_counter()
        info = cref.solve(A, B, d)
        ts.append(time.perf_counter() - t0)
        assert info == 0
    return min(ts), d


def run_reference(args):
    rank, world, _ = dist_env()
    if rank != 0:
        return
    As, Bs, ds = gen_host()
    cores = os.cpu_count() or 1
    # the reference CPU path is a sequential block chain; BLAS threads are the
    # only host parallelism it has.  Use whichever thread count is faster.
    best = None
    for th in sorted({1, cores}):
        t, _ = cpu_solve_time(As, Bs, ds, reps=1, threads=th)
        if best is None or t < best[0]:
            best = (t, th)
    th = best[1]
    from oracle import cref
    cref.set_blas_threads(th)
    for _ in range(max(args.warmup, 0)):
        cpu_solve_time(As, Bs, ds, reps=1)
    ts = []
    for _ in range(args.steps):
        t, _ = cpu_solve_time(As, Bs, ds, reps=1)
        ts.append(t)
    total = sum(ts)
    val = args.steps / total
    line = {
        "impl": "reference", "metric": METRIC, "value": val, "unit": "solves/s",
        "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": 1e3 * total / args.steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded numpy: A_i = G G^T + n I, B_i ~ N(0,1), d ~ U[0,1))",
        "config": {"workload": WORKLOAD, "N": N_BLK, "n": N_SZ, "k": K_RHS},
        "cpu_baseline": {"value": val, "unit": "solves/s", "cores": th, "kind": "port",
                         "sample": f"{args.steps} full factorize!+solve! of the workload, OpenBLAS "
                                   f"({th} thread(s)) via the C restatement of backbone_cpu.jl"},
        "e2e": {"value": val, "unit": "solves/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


# --------------------------------------------------------------------------
# GPU arm
# --------------------------------------------------------------------------
class ClockSampler:
    """nvidia-smi clocks + throttle reasons sampled every 100 ms."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index):
        self.idx = gpu_index
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.idx}", f"--query-gpu={self.Q}",
                                          "--format=csv,noheader,nounits", "-lms", "100"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.th = threading.Thread(target=self._read, daemon=True)
            self.th.start()
        except Exception:
            self.proc = None

    def _read(self):
        for ln in self.proc.stdout:
            self.lines.append(ln.strip())

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        sm, mx, reasons = [], [], set()
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx.append(float(f[2]))
            except ValueError:
                continue
            for name, val in zip(("hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"),
                                 f[5:9]):
                if val.lower().startswith("active"):
                    reasons.add(name)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def gen_device(dev, seed=1):
    import torch
    g = torch.Generator(device=dev).manual_seed(seed)
    G = torch.randn(N_BLK, N_SZ, N_SZ, device=dev, dtype=torch.float64, generator=g)
    A = G @ G.transpose(1, 2) + N_SZ * torch.eye(N_SZ, device=dev, dtype=torch.float64)
    del G
    B = torch.randn(N_BLK - 1, N_SZ, N_SZ, device=dev, dtype=torch.float64, generator=g)
    d = torch.rand(N_BLK, N_SZ, K_RHS, device=dev, dtype=torch.float64, generator=g)
    # column-major (n, n, N) views, as the handle tensors are laid out
    return A.permute(1, 2, 0), B.permute(1, 2, 0), d.permute(1, 2, 0)


def rel_residual_dev(A, B, x, d):
    """FP64 relative residual with torch on the device (checker only)."""
    import torch
    Am, Bm, xm, dm = (t.permute(2, 0, 1) for t in (A, B, x, d))
    r = dm - Am @ xm
    r[:-1] -= Bm @ xm[1:]
    r[1:] -= Bm.transpose(1, 2) @ xm[:-1]
    rs = Am.abs().sum(2)
    rs[:-1] += Bm.abs().sum(2)
    rs[1:] += Bm.abs().sum(1)
    return (r.abs().max() / (rs.max() * xm.abs().max() + dm.abs().max())).item()


def time_leg(bss, A, B, d, T, precision, steps, warmup, restore_AB, ev_stream=None):
    """K timed steps; returns (seconds total, factor ms list, solve ms list, data)."""
    import torch
    N = N_BLK
    data = bss.initialize_batched(N, N_SZ, T, k=K_RHS, precision=precision)
    At, Bt, dt = data.A_tensor[:, :, :N], data.B_tensor[:, :, :N - 1], data.d_tensor[:, :, :N]
    Ac, Bc, dc = A.to(T), B.to(T), d.to(T)
    At.copy_(Ac)
    Bt.copy_(Bc)

    def step(record=None):
        if restore_AB:
            At.copy_(Ac)
            Bt.copy_(Bc)
        dt.copy_(dc)
        if record:
            record[0].record()
        bss.factorize_(data)
        if record:
            record[1].record()
        bss.solve_(data)
        if record:
            record[2].record()

    for _ in range(warmup):
        step()
    bss.synchronize(data)
    torch.cuda.synchronize()
    evs = [[torch.cuda.Event(enable_timing=True) for _ in range(3)] for _ in range(steps)]
    t0 = torch.cuda.Event(enable_timing=True)
    t1 = torch.cuda.Event(enable_timing=True)
    t0.record()
    for s in range(steps):
        step(evs[s])
    t1.record()
    bss.synchronize(data)
    torch.cuda.synchronize()
    total_ms = t0.elapsed_time(t1)
    fac = [e[0].elapsed_time(e[1]) for e in evs]
    sol = [e[1].elapsed_time(e[2]) for e in evs]
    return total_ms / 1e3, fac, sol, data


def run_k16(bss, A, B, dev, peaks, hbm, check, reps=3):
    """Config 1 with k = 16 right-hand sides ~ U[0,1) (numpy, seed 16):
    factorize!+solve! in mixed precision (to rel-resid 1e-12), plain FP64 and
    plain FP32; each result against the C oracle's FP64 x when `check`."""
    import numpy as np
    import torch
    n, _, N = A.shape
    rng = np.random.default_rng(16)
    ds16 = np.ascontiguousarray(rng.random((N, 16, n)))  # storage order (N, k, n)
    d16 = torch.from_numpy(ds16).to(dev).permute(2, 1, 0)
    x_ref = None
    if check:
        As = A.permute(2, 1, 0).contiguous().cpu().numpy()
        Bs = B.permute(2, 1, 0).contiguous().cpu().numpy()
        x_ref = oracle_x(As, Bs, ds16)
        del As, Bs
    out = {"workload": "N=16384, n=64, k=16, d~U[0,1)"}
    for name, T, prec in (("mixed", torch.float64, "mixed"), ("plain_fp64", torch.float64, "plain"),
                          ("plain_fp32", torch.float32, "plain")):
        data = bss.initialize_batched(N, n, T, k=16, precision=prec)
        At, Bt, dt = data.A_tensor[:, :, :N], data.B_tensor[:, :, :N - 1], data.d_tensor[:, :, :N]
        Ac, Bc, dc = A.to(T), B.to(T), d16.to(T)
        fac, sol = [], []
        for r in range(reps + 1):
            At.copy_(Ac)
            Bt.copy_(Bc)
            dt.copy_(dc)
            e0, e1, e2 = (torch.cuda.Event(enable_timing=True) for _ in range(3))
            e0.record()
            bss.factorize_(data)
            e1.record()
            bss.solve_(data)
            e2.record()
            bss.synchronize(data)
            torch.cuda.synchronize()
            if r > 0:
                fac.append(e0.elapsed_time(e1))
                sol.append(e1.elapsed_time(e2))
        f, s_ = statistics.median(fac), statistics.median(sol)
        rr = rel_residual_dev(Ac.double(), Bc.double(), dt.double(), dc.double())
        res = {"solves_per_s": 1e3 / (f + s_), "factor_ms": f, "solve_ms": s_, "rel_residual": rr,
               "refine_steps": bss.get_info(data)["refine_steps"] if prec == "mixed" else 0}
        if x_ref is not None:
            res["rel_error_vs_oracle"] = rel_err_stor(dt.permute(2, 1, 0).double().cpu().numpy(), x_ref)
        pk = ("f32", "FP32") if (prec == "mixed" or T == torch.float32) else ("f64", "FP64")
        res["roofline"] = leg_roofline([(N, n, 16)], 4 if T == torch.float32 else 8, f, s_, peaks[pk[0]], pk[1], hbm)
        out[name] = res
        del data, At, Bt, dt
        torch.cuda.empty_cache()
    return out


def run_autotuned(bss, A, B, d, steps=10):
    """The headline system with the autotuner's kernel and plan for (n=64,
    FP64 tensors, mixed precision) against the defaults: the tuner times both
    chain kernels of 64-wide FP32 factors and the partition/cutoff plans on a
    probe system, then both configurations solve the workload here."""
    import torch
    out = {}
    bss.autotune_clear()
    secs, fac, sol, data = time_leg(bss, A, B, d, torch.float64, "mixed", steps, 2, False)
    out["default"] = {"solves_per_s": steps / secs, "factor_ms": statistics.median(fac),
                      "solve_ms": statistics.median(sol)}
    del data
    t0 = time.perf_counter()
    e = bss.autotune(N_SZ, torch.float64, "mixed", N_probe=N_BLK)
    out["tuning_s"] = time.perf_counter() - t0
    out["entry"] = e
    secs, fac, sol, data = time_leg(bss, A, B, d, torch.float64, "mixed", steps, 2, False)
    out["tuned"] = {"solves_per_s": steps / secs, "factor_ms": statistics.median(fac),
                    "solve_ms": statistics.median(sol),
                    "rel_residual": rel_residual_dev(A, B, data.d_tensor[:, :, :N_BLK], d)}
    del data
    bss.autotune_clear()
    out["tuned_over_default"] = out["tuned"]["solves_per_s"] / out["default"]["solves_per_s"]
    return out


def time_reference_algorithm(bss, A, B, d, reps=3):
    """The reference's own batched GPU algorithm (gpu_batched.jl over batched
    cuSOLVER/cuBLAS, restated in C++: bss_refalgo_*) in FP64 on the same
    system: factorize!+solve! with CUDA events, inputs copied in before each
    rep (outside the timed region); median ms."""
    import torch
    n, _, N = A.shape
    data = bss.initialize_reference_algorithm(N, n, torch.float64, k=d.shape[1])
    At, Bt, dt = data.A_tensor[:, :, :N], data.B_tensor[:, :, :N - 1], data.d_tensor[:, :, :N]
    fac, sol = [], []
    for r in range(reps + 1):
        At.copy_(A)
        Bt.copy_(B)
        dt.copy_(d)
        e0, e1, e2 = (torch.cuda.Event(enable_timing=True) for _ in range(3))
        e0.record()
        bss.factorize_(data)
        e1.record()
        bss.solve_(data)
        e2.record()
        torch.cuda.synchronize()
        if r > 0:
            fac.append(e0.elapsed_time(e1))
            sol.append(e1.elapsed_time(e2))
    rr = rel_residual_dev(A, B, dt, d)
    f, s_ = statistics.median(fac), statistics.median(sol)
    del data, At, Bt, dt
    return {"solves_per_s": 1e3 / (f + s_), "factor_ms": f, "solve_ms": s_, "rel_residual": rr,
            "what": "reference gpu_batched.jl algorithm over batched cuSOLVER/cuBLAS (FP64), restated in C++"}


def hbm_peak():
    """(GB/s, "measured" | "fallback"): the measured HBM copy bandwidth of
    MEASURED_PEAKS.json, else the fallback 6.8 TB/s."""
    peaks = {}
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            peaks = json.load(f)
    except Exception:
        pass
    hbm = peaks.get("hbm_gbs")
    return (hbm, "measured") if hbm else (6800.0, "fallback")


def fma_peaks():
    """{"f64": TFLOP/s, "f32": TFLOP/s} of the FMA pipes of this GPU, measured
    by the library's microbenchmark (bss_diag_fma_peak)."""
    import ctypes
    from blockstructuredsolvers_gb300 import _lib
    L = _lib.load()
    out = {}
    for name, code in (("f64", _lib.BSS_F64), ("f32", _lib.BSS_F32)):
        v = ctypes.c_double()
        _lib.check(L.bss_diag_fma_peak(code, ctypes.byref(v)))
        out[name] = v.value
    return out


def work(N, n, k):
    """Algorithmic work of one factorize!+solve! from (N, n, k) alone:
    F_factor = N n^3/3 + 2 (N-1) n^3 (potrf, trsm, syrk per block),
    F_solve = k (2N + 4(N-1)) n^2, and the elements of A, B and d."""
    F_fac = N * n ** 3 / 3.0 + 2.0 * (N - 1) * n ** 3
    F_sol = k * (2.0 * N + 4.0 * (N - 1)) * n ** 2
    elems_ab = (2 * N - 1) * n * n
    return F_fac, F_sol, elems_ab, N * n * k


def leg_roofline(systems, itemsize, factor_ms, solve_ms, peak_tflops, peak_name, hbm_gbs):
    """GFLOP/s and the fraction of the roofline for a leg that solves the
    (N, n, k) `systems` once in factor_ms + solve_ms: roofline time =
    max(F / compute peak, bytes of A, B, d / HBM bandwidth), fraction =
    roofline time / measured time.  Also the same for factorize! alone
    (F_factor, bytes of A and B)."""
    F_fac = F_sol = ab = dd = 0.0
    for (N, n, k) in systems:
        a, b, c, e = work(N, n, k)
        F_fac, F_sol, ab, dd = F_fac + a, F_sol + b, ab + c, dd + e
    t = (factor_ms + solve_ms) * 1e-3
    t_flop = (F_fac + F_sol) / (peak_tflops * 1e12)
    t_mem = itemsize * (ab + dd) / (hbm_gbs * 1e9)
    roof = max(t_flop, t_mem)
    f_flop = F_fac / (peak_tflops * 1e12)
    f_mem = itemsize * ab / (hbm_gbs * 1e9)
    return {"gflops": (F_fac + F_sol) / t / 1e9, "factor_gflops": F_fac / (factor_ms * 1e-3) / 1e9,
            "roofline_ms": roof * 1e3, "roofline_frac": roof / t,
            "factor_roofline_frac": max(f_flop, f_mem) / (factor_ms * 1e-3),
            "bound": "compute" if t_flop >= t_mem else "hbm",
            "peaks": f"{peak_name} FMA {peak_tflops:.2f} TFLOP/s (bss_diag_fma_peak, measured here); "
                     f"HBM {hbm_gbs:.0f} GB/s",
            "work": {"F_factor": F_fac, "F_solve": F_sol, "bytes": itemsize * (ab + dd)}}


def oracle_x(As, Bs, ds, threads=None):
    """x of the C oracle (backbone_cpu.jl restated, FP64) for storage-order
    inputs; returns storage-order x (N, k, n).  Checker only."""
    from oracle import cref
    cref.lib(True)
    cref.set_blas_threads(threads or os.cpu_count() or 1)
    A, B, d = As.copy(), Bs.copy(), ds.copy()
    assert cref.solve(A, B, d) == 0
    return d


def rel_err_stor(x, x_ref):
    """max |x - x_ref| / max |x_ref| over storage-order arrays."""
    import numpy as np
    x = np.asarray(x, np.float64)
    return float(np.abs(x - x_ref).max() / np.abs(x_ref).max())


def time_sparse_cholesky(bss, A, B, d, hbm_gbs):
    """The reference's sparse comparison (benchmark/benchmark_gpu.jl:75-117:
    analysis, factorization and solve of the assembled CSR matrix with a
    sparse direct solver) in FP64 on the same system.  cuDSS is not in this
    toolkit: cuSOLVER's GPU sparse Cholesky (csrchol*) stands in.  Each phase
    runs once (seconds at this size), timed on the host around a
    synchronize.  The CSR assembly kernel alone (bss_csr_assemble,
    construct_block_tridiagonal of benchmark/utils.jl:59-103) is timed with
    CUDA events over 5 launches (inputs and outputs larger than L2) against
    the HBM copy peak."""
    import ctypes
    import torch
    from blockstructuredsolvers_gb300 import _lib
    n, _, N = A.shape
    k = d.shape[1]
    L = _lib.load()
    nnz = int(L.bss_csr_nnz(N, n))
    dev = A.device
    crow = torch.empty(N * n + 1, dtype=torch.int32, device=dev)
    col = torch.empty(nnz, dtype=torch.int32, device=dev)
    val = torch.empty(nnz, dtype=torch.float64, device=dev)
    Ac = A.permute(2, 1, 0).contiguous()   # (N, c, r): column-major blocks
    Bc = B.permute(2, 1, 0).contiguous()
    stream = torch.cuda.current_stream()
    sp = ctypes.c_void_p(int(stream.cuda_stream))
    ms = []
    for r in range(6):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        _lib.check(L.bss_csr_assemble(N, n, _lib.BSS_F64, ctypes.c_void_p(Ac.data_ptr()),
                                      ctypes.c_void_p(Bc.data_ptr()), ctypes.c_void_p(crow.data_ptr()),
                                      ctypes.c_void_p(col.data_ptr()), ctypes.c_void_p(val.data_ptr()), sp))
        e1.record(stream)
        torch.cuda.synchronize()
        if r > 0:
            ms.append(e0.elapsed_time(e1))
    asm_ms = statistics.median(ms)
    asm_bytes = 8 * n * n * (2 * N - 1) + 12 * nnz + 4 * (N * n + 1)
    del crow, col, val, Ac, Bc
    data = bss.initialize_sparse_cholesky(N, n, torch.float64, k=k)
    data.A_tensor.copy_(A)
    data.B_tensor.copy_(B)
    data.d_tensor.copy_(d)
    torch.cuda.synchronize()
    t = {}
    for ph, fn in (("analysis", bss.analyze_), ("factorization", bss.factorize_), ("solve", bss.solve_)):
        t0 = time.perf_counter()
        fn(data)
        torch.cuda.synchronize()
        t[ph] = (time.perf_counter() - t0) * 1e3
    rr = rel_residual_dev(A, B, data.d_tensor, d)
    del data
    torch.cuda.empty_cache()
    return {"solves_per_s": 1e3 / (t["factorization"] + t["solve"]), "analysis_ms": t["analysis"],
            "factor_ms": t["factorization"], "solve_ms": t["solve"], "rel_residual": rr, "nnz": nnz,
            "what": "assembled CSR matrix (construct_block_tridiagonal) on cuSOLVER's GPU sparse Cholesky "
                    "(FP64), standing in for the reference's cuDSS comparison; cuDSS is not in this toolkit",
            "csr_assembly": {"ms": asm_ms, "bytes": asm_bytes, "gbs": asm_bytes / asm_ms / 1e6,
                             "frac_of_measured_hbm": asm_bytes / asm_ms / 1e6 / hbm_gbs}}


def run_ours(args):
    import numpy as np
    import torch
    rank, world, local = dist_env()
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    import blockstructuredsolvers_gb300 as bss
    from blockstructuredsolvers_gb300 import _lib
    L = _lib.load()

    # the same seeded host inputs as the reference arm, in Julia storage order
    As, Bs, ds = gen_host()
    # column-major (n, n, N) device views, the handle tensors' layout
    A = torch.from_numpy(As).to(dev).permute(2, 1, 0)
    B = torch.from_numpy(Bs).to(dev).permute(2, 1, 0)
    d = torch.from_numpy(ds).to(dev).permute(2, 1, 0)
    hbm, peak_kind = hbm_peak()
    peaks = fma_peaks()
    # ---- e2e through the public API with host buffers ----------------------
    # (first of the legs: measured in a process that has not yet run the others)
    # A stream of requests, each: pinned host A, B, d -> device (bss.upload),
    # factorize!, solve!, x -> pinned host (bss.download).  Three handles on
    # three CUDA streams take requests in turn (the buffering a serving caller
    # uses), so one request's copies overlap another's compute; every request
    # still pays its own H2D and D2H inside the timed region.  (Two handles
    # reach the same rate once warm, three absorb the jitter of the copies.)  The
    # host link bounds it: the copy engines' rate from pinned host memory is
    # measured beside it (one whole-buffer copy), with the solves/s that rate
    # allows for these bytes; the one-handle serial figure is reported too.
    e2e = None
    if not args.quick:
        # host copies in the handle's storage order: (N, c, r) C-order == column-major blocks
        Ah = torch.from_numpy(As).pin_memory()
        Bh = torch.from_numpy(Bs).pin_memory()
        dh = torch.from_numpy(ds).pin_memory()
        streams = [torch.cuda.Stream() for _ in range(3)]
        slots = []
        for st in streams:
            with torch.cuda.stream(st):
                data = bss.initialize_batched(N_BLK, N_SZ, torch.float64, k=K_RHS, precision="mixed", stream=st)
            slots.append((st, data, torch.empty_like(dh).pin_memory()))
        ne = max(20, args.steps // 4)
        moved = [0]

        def e2e_step(slot):
            st, data, xh = slot
            moved[0] = bss.upload(data, Ah, Bh, dh)
            bss.factorize_(data)
            bss.solve_(data)
            bss.download(data, xh)

        def e2e_run(count, use):
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            for i in range(count):
                e2e_step(use[i % len(use)])
            torch.cuda.synchronize()
            return time.perf_counter() - t0

        for slot in slots:  # first calls run eagerly and capture the graphs
            for _ in range(2):
                e2e_step(slot)
        # host-to-device copies reach the link's full rate only after ~0.3 s of
        # sustained transfers (the first 50 requests after an idle pause ran at
        # 140 - 180 solves/s, the next 50 at 192.5): warm the pipeline first
        e2e_run(max(60, ne), slots)
        te = e2e_run(ne, slots)
        bi = moved[0]
        n1 = max(5, ne // 2)
        te1 = e2e_run(n1, slots[:1]) / n1
        x_e2e = slots[0][2].permute(2, 1, 0)  # (n, k, N) view of the last x
        rr_e2e = rel_residual_dev(A, B, x_e2e.to(dev), d)
        bo = slots[0][2].numel() * 8
        # the host link's rate: one whole-buffer pinned copy of B, timed on the device
        lk_dst = slots[0][1].B_tensor[:, :, :N_BLK - 1].permute(2, 1, 0)
        lk0, lk1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        lk_dst.copy_(Bh, non_blocking=True)
        lk0.record()
        for _ in range(3):
            lk_dst.copy_(Bh, non_blocking=True)
        lk1.record()
        torch.cuda.synchronize()
        link_gbs = 3 * Bh.numel() * 8 / (lk0.elapsed_time(lk1) * 1e-3) / 1e9
        e2e = {"value": world * ne / te, "unit": "solves/s", "h2d_bytes_per_step": bi, "d2h_bytes_per_step": bo,
               "requests_timed": ne,
               "mode": "three handles on three streams, requests in turn, copies inside the timed region; "
                       "bss.upload / bss.download",
               "serial_one_handle": world / te1, "rel_residual_last_x": rr_e2e,
               "rel_error_vs_oracle_last_x": None,
               "link": {"h2d_gbs": link_gbs, "bound_solves_per_s": world * link_gbs * 1e9 / bi,
                        "note": "one pinned copy engine transfer of B, timed on the device"}}
        x_e2e_host = slots[0][2].numpy().copy()
        del slots

    # ---- headline: mixed precision, inputs resident in HBM -------------------
    sampler = ClockSampler(local)
    if world > 1:
        dist.barrier()
    torch.cuda.synchronize()
    launches0 = L.bss_kernel_launches()
    sampler.start()
    secs, fac, sol, data = time_leg(bss, A, B, d, torch.float64, "mixed", args.steps, args.warmup, False)
    clocks = sampler.stop()
    launches = L.bss_kernel_launches() - launches0
    info = bss.get_info(data)
    x = data.d_tensor[:, :, :N_BLK]
    relres = rel_residual_dev(A, B, x, d)
    x_head = x.permute(2, 1, 0).contiguous().cpu().numpy()  # (N, k, n): the oracle's storage order
    del data, x
    # the warmup steps launched too: count per step from the total
    launches_per_step = launches / max(args.steps + args.warmup, 1)
    from blockstructuredsolvers_gb300 import replicas
    secs = replicas.reduce_max(secs)  # the slowest replica's time
    value = world * args.steps / secs
    x_ref = oracle_x(As, Bs, ds) if rank == 0 else None
    if e2e is not None and rank == 0:
        e2e["rel_error_vs_oracle_last_x"] = rel_err_stor(x_e2e_host, x_ref)
    err_head = rel_err_stor(x_head, x_ref) if rank == 0 else None
    cfg1 = [(N_BLK, N_SZ, K_RHS)]
    head_roof = leg_roofline(cfg1, 8, statistics.median(fac), statistics.median(sol), peaks["f32"], "FP32", hbm)

    extra = {"peaks_measured": {"fp64_fma_tflops": peaks["f64"], "fp32_fma_tflops": peaks["f32"],
                                "hbm_gbs": hbm, "hbm_source": f"MEASURED_PEAKS.json ({peak_kind})"}}
    if not args.quick:
        # ---- plain FP64 and plain FP32 GPU paths (same request) ---------------
        n64 = max(3, args.steps // 4)
        s64, f64, so64, d64 = time_leg(bss, A, B, d, torch.float64, "plain", n64, 1, True)
        rr64 = rel_residual_dev(A, B, d64.d_tensor[:, :, :N_BLK], d)
        x64 = d64.d_tensor[:, :, :N_BLK].permute(2, 1, 0).contiguous().cpu().numpy()
        del d64
        s32, f32, so32, d32 = time_leg(bss, A, B, d, torch.float32, "plain", n64, 1, True)
        rr32 = rel_residual_dev(A.float().double(), B.float().double(), d32.d_tensor[:, :, :N_BLK].double(),
                                d.float().double())
        x32 = d32.d_tensor[:, :, :N_BLK].permute(2, 1, 0).double().contiguous().cpu().numpy()
        del d32
        extra["autotuned"] = run_autotuned(bss, A, B, d)
        extra["reference_algorithm_gpu"] = time_reference_algorithm(bss, A, B, d)
        extra["sparse_cholesky_gpu"] = time_sparse_cholesky(bss, A, B, d, hbm)
        extra["k16"] = run_k16(bss, A, B, dev, peaks, hbm, rank == 0)
        fm64, sm64 = statistics.median(f64), statistics.median(so64)
        extra["plain_fp64"] = {"solves_per_s": n64 / s64, "factor_ms": fm64, "solve_ms": sm64,
                               "rel_residual": rr64,
                               "rel_error_vs_oracle": rel_err_stor(x64, x_ref) if rank == 0 else None,
                               "refine_steps": 0,
                               "roofline": leg_roofline(cfg1, 8, fm64, sm64, peaks["f64"], "FP64", hbm),
                               "note": "solves/s includes the device copy of A, B, d into the handle per step"}
        fm32, sm32 = statistics.median(f32), statistics.median(so32)
        extra["plain_fp32"] = {"solves_per_s": n64 / s32, "factor_ms": fm32, "solve_ms": sm32,
                               "rel_residual_fp32_system": rr32,
                               "rel_error_vs_oracle": rel_err_stor(x32, x_ref) if rank == 0 else None,
                               "refine_steps": 0,
                               "roofline": leg_roofline(cfg1, 4, fm32, sm32, peaks["f32"], "FP32", hbm),
                               "note": "FP32 accuracy only; not a rel-resid <= 1e-12 result"}

    # ---- roofline of the dominant kernel ----------------------------------
    roof = roofline_chain_factor(bss, A, B, d, hbm, peak_kind)

    cpu_base = None
    if rank == 0 and not args.no_cpu_baseline and world == 1:
        try:
            cores = os.cpu_count() or 1
            t1, _ = cpu_solve_time(As, Bs, ds, reps=1, threads=1)
            tN, xcpu = cpu_solve_time(As, Bs, ds, reps=1, threads=cores)
            best = min((t1, 1), (tN, cores))
            cpu_base = {"value": 1.0 / best[0], "unit": "solves/s", "cores": best[1], "kind": "port",
                        "sample": "one full factorize!+solve! of the workload (C restatement of "
                                  "backbone_cpu.jl on OpenBLAS); best of 1 thread and "
                                  f"{cores} BLAS threads"}
        except Exception as e:  # pragma: no cover
            cpu_base = {"value": None, "unit": "solves/s", "cores": None, "kind": "port", "sample": f"failed: {e}"}

    others = {}
    if not args.quick and not args.no_extra:
        del A, B, d
        torch.cuda.empty_cache()
        others["large_system_n128"] = run_large_system(bss, dev, peaks, hbm, rank == 0)
        others["uneven_batch"] = run_uneven_batch(bss, dev, peaks, hbm, rank == 0)
        others["served_kalman"] = run_served_legs(bss, rank == 0)

    if rank == 0:
        line = {
            "metric": METRIC, "value": value, "unit": "solves/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": 1e3 * secs / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32 factor + f64 refinement",
            "data": "synthetic (seeded numpy on the host, the reference arm's bytes: "
                    "A_i = G G^T + n I, B_i ~ N(0,1), d ~ U[0,1))",
            "config": {"workload": WORKLOAD, "N": N_BLK, "n": N_SZ, "k": K_RHS, "precision": "mixed",
                       "levels": info["levels"], "coarsest_blocks": info["coarsest_blocks"],
                       "l2": "inputs (1.07 GB FP64 A,B) larger than L2; no flush",
                       "parallelism": "replicas" if world > 1 else "single GPU"},
            "factor_ms_median": statistics.median(fac), "solve_ms_median": statistics.median(sol),
            "refine_steps": info["refine_steps"], "rel_residual": relres, "rel_error_vs_oracle": err_head,
            "gflops": head_roof["gflops"], "roofline_8d": head_roof,
            "gpu_launches": int(round(launches_per_step * args.steps)),
            "gpu_launches_per_step": launches_per_step,
            "clocks": clocks, "roofline": roof, "cpu_baseline": cpu_base, "e2e": e2e,
        }
        line.update(extra)
        line.update(others)
        print(json.dumps(line), flush=True)
    if world > 1:
        dist.barrier()
        dist.destroy_process_group()


# --------------------------------------------------------------------------
# served Kalman-smoother request stream
# --------------------------------------------------------------------------
KF_SIZES = (8, 16, 32, 64)


def gen_kf_stream(n_requests, rate, repeat_frac=0.3, seed=4, recent=32):
    """Seeded request stream: Poisson arrivals at `rate` req/s; a request is
    a new Kalman model (n from {8,16,32,64}, horizon N ~ U{50..5000}, F ~
    N(0,1) rescaled to spectral radius 0.95, H ~ N(0,1) (n/2 x n), Q = 0.1 I,
    R = 0.5 I, observations simulated from the model) or, with probability
    `repeat_frac`, new observations for one of the `recent` last models
    (a repeat right-hand side on its resident factor).  Host buffers are
    page-locked torch tensors in column-major storage order."""
    import numpy as np
    import torch
    pin = (lambda t: t.pin_memory()) if torch.cuda.is_available() else (lambda t: t)
    rng = np.random.default_rng(seed)
    gaps = rng.exponential(1.0 / rate, n_requests) if rate else np.zeros(n_requests)
    t_arr = np.cumsum(gaps) - gaps[0]
    kinds = []
    models = []
    for i in range(n_requests):
        if models and rng.random() < repeat_frac:
            kinds.append(("rhs", int(rng.integers(max(0, len(models) - recent), len(models)))))
        else:
            n = int(rng.choice(KF_SIZES))
            N = int(rng.integers(50, 5001))
            models.append({"n": n, "N": N})
            kinds.append(("new", len(models) - 1))
    # models, batched per state size
    for n in KF_SIZES:
        idx = [j for j, mdl in enumerate(models) if mdl["n"] == n]
        if not idx:
            continue
        m = n // 2
        F = rng.standard_normal((len(idx), n, n))
        rho = np.abs(np.linalg.eigvals(F)).max(axis=1)
        F *= (0.95 / rho)[:, None, None]
        H = rng.standard_normal((len(idx), m, n))
        for j, a in enumerate(idx):
            models[a]["F"], models[a]["H"] = F[j], H[j]
    # observation sequences, one per request (new models and repeats),
    # simulated for all requests of one state size at once
    Ys = [None] * n_requests
    for n in KF_SIZES:
        idx = [i for i, (kind, a) in enumerate(kinds) if models[a]["n"] == n]
        if not idx:
            continue
        m = n // 2
        Fb = np.stack([models[kinds[i][1]]["F"] for i in idx])
        Hb = np.stack([models[kinds[i][1]]["H"] for i in idx])
        Ns = np.array([models[kinds[i][1]]["N"] for i in idx])
        T = int(Ns.max())
        W = rng.standard_normal((T, len(idx), n)) * np.sqrt(0.1)
        V = rng.standard_normal((len(idx), T, m)) * np.sqrt(0.5)
        dev = "cuda" if torch.cuda.is_available() else "cpu"  # input synthesis only
        Ft, Wt = torch.from_numpy(Fb).to(dev), torch.from_numpy(W).to(dev)
        Xt = torch.empty((T, len(idx), n), dtype=torch.float64, device=dev)
        x = torch.zeros((len(idx), n, 1), dtype=torch.float64, device=dev)
        for t in range(T):
            x = torch.bmm(Ft, x) + Wt[t][:, :, None]
            Xt[t] = x[:, :, 0]
        X = Xt.permute(1, 0, 2).cpu().numpy()
        Y = np.matmul(X, np.swapaxes(Hb, 1, 2)) + V
        for j, i in enumerate(idx):
            Ys[i] = pin(torch.from_numpy(np.ascontiguousarray(Y[j, :Ns[j]])).reshape(int(Ns[j]), 1, m))
    reqs = []
    for i, ((kind, a), t) in enumerate(zip(kinds, t_arr)):
        mdl = models[a]
        reqs.append({"kind": kind, "model": a, "t": float(t), "y": Ys[i],
                     "x": pin(torch.zeros((mdl["N"], 1, mdl["n"]), dtype=torch.float64))})
    for mdl in models:
        n, m = mdl["n"], mdl["n"] // 2
        colmaj = lambda M: pin(torch.from_numpy(np.ascontiguousarray(M.T)))
        mdl["Fh"], mdl["Hh"] = colmaj(mdl["F"]), colmaj(mdl["H"])
        mdl["Qi"] = pin(torch.eye(n, dtype=torch.float64).mul_(10.0))
        mdl["Ri"] = pin(torch.eye(m, dtype=torch.float64).mul_(2.0))
    return models, reqs


def served_sample_check(models, reqs, ids, every=40):
    """Every `every`-th completed request of a served stream against the C
    oracle: its blocks rebuilt on the host by the oracle's restatement of
    build_kf_blocks, solved in FP64 on the host cores; returns the worst
    relative error of x and the worst FP64 relative residual over the
    sample, and the sample size."""
    import numpy as np
    import oracle.oracle as O
    from oracle import cref
    cref.lib(True)
    cref.set_blas_threads(1)
    worst_err = worst_res = 0.0
    cnt = 0
    for i in range(0, len(reqs), every):
        if ids[i] is None:
            continue
        r = reqs[i]
        mdl = models[r["model"]]
        n, m = mdl["n"], mdl["n"] // 2
        Y = np.swapaxes(r["y"].numpy(), 1, 2)  # (N, m, k) math
        A, B, d = O.kf_blocks(mdl["F"], mdl["H"], 10.0 * np.eye(n), 2.0 * np.eye(m), Y)
        x_ref = cref.solve_math(A, B, d, np.float64)
        x = np.swapaxes(r["x"].numpy(), 1, 2)
        worst_err = max(worst_err, O.rel_error(x, x_ref))
        worst_res = max(worst_res, O.rel_residual(A, B, x, d))
        cnt += 1
    return worst_err, worst_res, cnt


def run_served(bss, precision, models, reqs, budget=100 * 10**9, streams=8, check=False):
    """Replay the stream against a server: a submitter thread releases each
    request at its arrival time; returns solves/s, latency percentiles and
    the worst relative residual the solver reported (mixed precision), and
    with `check` a sample of the results against the C oracle."""
    import threading
    srv = bss.Server(hbm_budget_bytes=budget, streams=streams, max_inflight=64, precision=precision)
    fids = {}
    ids = [None] * len(reqs)
    errors = []

    def submitter():
        t0 = time.perf_counter()
        for i, r in enumerate(reqs):
            wait = r["t"] - (time.perf_counter() - t0)
            if wait > 0:
                time.sleep(wait)
            mdl = models[r["model"]]
            try:
                if r["kind"] == "new":
                    rid, fid = srv.submit_kalman(mdl["Fh"], mdl["Hh"], mdl["Qi"], mdl["Ri"], r["y"], r["x"],
                                                 keep=True)
                    fids[r["model"]] = fid
                else:
                    rid = srv.submit_rhs(fids[r["model"]], r["y"], r["x"])
                ids[i] = rid
            except Exception as e:  # an evicted factor: counted, not fatal
                errors.append(str(e))

    th = threading.Thread(target=submitter)
    th.start()
    th.join()
    worst = 0.0
    steps = []
    failed = 0
    for rid in ids:
        if rid is None:
            continue
        info = srv.wait(rid, check=False)
        if info["status"] != 0:
            failed += 1
        worst = max(worst, info["rel_residual"])
        steps.append(info["refine_steps"])
    st = srv.stats()
    srv.close()
    out = {"solves_per_s": st["completed"] / st["busy_s"] if st["busy_s"] > 0 else None,
           "p50_ms": st["p50_ms"], "p99_ms": st["p99_ms"], "mean_ms": st["mean_ms"], "max_ms": st["max_ms"],
           "completed": st["completed"], "failed": failed + len(errors), "evictions": st["evictions"],
           "bytes_peak": st["bytes_peak"], "worst_rel_residual": worst if precision == "mixed" else None,
           "mean_refine_steps": (sum(steps) / len(steps)) if steps else None,
           "max_refine_steps": max(steps) if steps else None}
    if check:
        e, r, c = served_sample_check(models, reqs, ids)
        out.update({"sample_worst_rel_error_vs_oracle": e, "sample_worst_rel_residual": r,
                    "sample": f"{c} requests (every 40th), blocks rebuilt on the host, C oracle FP64"})
    return out


# --------------------------------------------------------------------------
# one large system of wide blocks (N=65536, n=128, k=4) and the uneven batch of 2048 systems
# --------------------------------------------------------------------------
def _orthogonal(G):
    """Q of the QR factorization of G (positive diagonal R) by CholeskyQR2:
    Q1 = G R1^{-1} with R1 = chol(G^T G), then the same once more on Q1."""
    import torch
    Q = G
    for _ in range(2):
        R = torch.linalg.cholesky(Q.transpose(1, 2) @ Q, upper=True)
        Q = torch.linalg.solve_triangular(R, Q, upper=True, left=False)
    return Q


def gen_logspectrum(dev, N=65536, n=128, k=4, seed=2):
    """A_i = Q_i diag(lambda) Q_i^T (lambda log-spaced over [1, 1e4]),
    B_i = 0.45 U_i V_i^T, d ~ N(0,1); Q, U, V orthogonal factors of
    Gaussian matrices.  Column-major (n, n, N) views."""
    import torch
    g = torch.Generator(device=dev).manual_seed(seed)
    lam = torch.logspace(0, 4, n, dtype=torch.float64, device=dev)
    A = torch.empty((N, n, n), dtype=torch.float64, device=dev)
    B = torch.empty((N - 1, n, n), dtype=torch.float64, device=dev)
    ch = 8192
    for s0 in range(0, N, ch):
        e = min(N, s0 + ch)
        Q = _orthogonal(torch.randn((e - s0, n, n), dtype=torch.float64, device=dev, generator=g))
        Ab = (Q * lam[None, None, :]) @ Q.transpose(1, 2)
        A[s0:e] = 0.5 * (Ab + Ab.transpose(1, 2))
    for s0 in range(0, N - 1, ch):
        e = min(N - 1, s0 + ch)
        U = _orthogonal(torch.randn((e - s0, n, n), dtype=torch.float64, device=dev, generator=g))
        V = _orthogonal(torch.randn((e - s0, n, n), dtype=torch.float64, device=dev, generator=g))
        B[s0:e] = 0.45 * (U @ V.transpose(1, 2))
    d = torch.randn((N, n, k), dtype=torch.float64, device=dev, generator=g)
    return A.permute(1, 2, 0), B.permute(1, 2, 0), d.permute(1, 2, 0)


def _timed_handle_leg(bss, A, B, d, precision, reps):
    """factorize!+solve! of one system on the device, inputs copied into the
    handle before each rep (outside the timed region); median ms."""
    import torch
    n, _, N = A.shape
    k = d.shape[1]
    data = bss.initialize_batched(N, n, torch.float64, k=k, precision=precision)
    At, Bt, dt = data.A_tensor[:, :, :N], data.B_tensor[:, :, :N - 1], data.d_tensor[:, :, :N]
    fac, sol = [], []
    for r in range(reps + 1):
        At.copy_(A)
        Bt.copy_(B)
        dt.copy_(d)
        e0, e1, e2 = (torch.cuda.Event(enable_timing=True) for _ in range(3))
        e0.record()
        bss.factorize_(data)
        e1.record()
        bss.solve_(data)
        e2.record()
        bss.synchronize(data)
        torch.cuda.synchronize()
        if r > 0 or reps == 0:
            fac.append(e0.elapsed_time(e1))
            sol.append(e1.elapsed_time(e2))
    info = bss.get_info(data)
    relres = rel_residual_dev(A, B, dt, d)
    x = dt.permute(2, 1, 0).contiguous().cpu().numpy()
    del data
    torch.cuda.empty_cache()
    f, s_ = statistics.median(fac), statistics.median(sol)
    return {"solves_per_s": 1e3 / (f + s_), "factor_ms": f, "solve_ms": s_, "rel_residual": relres,
            "refine_steps": info["refine_steps"], "levels": info["levels"]}, x


def run_large_system(bss, dev, peaks, hbm, check):
    """N=65536 blocks of n=128, k=4 (log-spaced spectra over [1, 1e4]):
    mixed precision and plain FP64 on the device; each x against the C
    oracle's FP64 solve of the same inputs on the host cores."""
    import torch
    A, B, d = gen_logspectrum(dev)
    n, _, N = A.shape
    k = d.shape[1]
    out = {"workload": "N=65536, n=128, k=4, A_i=Q diag(logspace(0,4)) Q^T, B_i=0.45 U V^T, d~N(0,1)"}
    legs = {}
    for name, prec, reps in (("mixed", "mixed", 3), ("plain_fp64", "plain", 1)):
        res, x = _timed_handle_leg(bss, A, B, d, prec, reps)
        pk = ("f32", "FP32") if prec == "mixed" else ("f64", "FP64")
        res["roofline"] = leg_roofline([(N, n, k)], 8, res["factor_ms"], res["solve_ms"], peaks[pk[0]], pk[1], hbm)
        out[name] = res
        legs[name] = x
    out["mixed_over_plain_fp64"] = out["mixed"]["solves_per_s"] / out["plain_fp64"]["solves_per_s"]
    if check:
        As = A.permute(2, 1, 0).contiguous().cpu().numpy()
        Bs = B.permute(2, 1, 0).contiguous().cpu().numpy()
        ds = d.permute(2, 1, 0).contiguous().cpu().numpy()
        t0 = time.perf_counter()
        x_ref = oracle_x(As, Bs, ds)
        out["oracle_s"] = time.perf_counter() - t0
        del As, Bs, ds
        for name, x in legs.items():
            out[name]["rel_error_vs_oracle"] = rel_err_stor(x, x_ref)
    del A, B, d, legs
    torch.cuda.empty_cache()
    return out


def run_uneven_batch(bss, dev, peaks, hbm, check, steps=3, seed=3, sample_every=32):
    """2048 independent systems, N ~ U{16..1024}, n from {16,32,48,64,96,128},
    k ~ U{1..8}, A_i = G G^T + 2n I, B_i ~ 0.5 N(0,1), d ~ U[0,1); mixed
    precision, one batch (graph-replayed after the first call).  Every
    `sample_every`-th system is also solved by the C oracle on the host cores
    (one thread per system, all cores: the CPU baseline of this config) and
    its GPU x compared with the oracle's."""
    import numpy as np
    import torch
    rng = np.random.default_rng(seed)
    S = 2048
    Ns = rng.integers(16, 1025, S)
    ns = rng.choice([16, 32, 48, 64, 96, 128], S)
    ks = rng.integers(1, 9, S)
    res = {"workload": "2048 systems, N~U{16..1024}, n in {16,32,48,64,96,128}, k~U{1..8}, "
                       "A=GG^T+2nI, B~0.5N(0,1)"}
    def fill(b):  # seeded inputs written straight into the batch tensors
        g = torch.Generator(device=dev).manual_seed(seed)
        for sv in b.systems:
            N, n, k = sv.N, sv.n, sv.k
            G = torch.randn((N, n, n), dtype=torch.float64, device=dev, generator=g)
            sv.A_tensor.copy_((G @ G.transpose(1, 2) + 2 * n * torch.eye(n, dtype=torch.float64, device=dev))
                              .permute(1, 2, 0))
            Bm = 0.5 * torch.randn((max(N - 1, 0), n, n), dtype=torch.float64, device=dev, generator=g)
            if N > 1:
                sv.B_tensor.copy_(Bm.permute(1, 2, 0))
            sv.d_tensor.copy_(torch.rand((N, n, k), dtype=torch.float64, device=dev, generator=g).permute(1, 2, 0))

    sample = list(range(0, S, sample_every))
    host = {}

    def leg(prec):  # in its own scope: the batch dies with the function's locals
        b = bss.initialize_multi(Ns.tolist(), ns.tolist(), ks.tolist(), torch.float64, precision=prec)
        fac, sol = [], []
        nsteps = steps if prec == "mixed" else 1
        dsave = None
        for r in range(nsteps + 1):
            if prec == "plain" or dsave is None:  # plain factors in place: fresh inputs every rep
                fill(b)
                if check and not host:  # the sampled systems' inputs, storage order
                    for i in sample:
                        sv = b.systems[i]
                        host[i] = tuple(t.permute(2, 1, 0).contiguous().cpu().numpy()
                                        for t in (sv.A_tensor, sv.B_tensor, sv.d_tensor))
                if prec == "mixed":
                    dsave = [sv.d_tensor.clone() for sv in b.systems]
            else:
                for sv, dm in zip(b.systems, dsave):
                    sv.d_tensor.copy_(dm)
            torch.cuda.synchronize()
            e0, e1, e2 = (torch.cuda.Event(enable_timing=True) for _ in range(3))
            e0.record()
            b.factorize()
            e1.record()
            b.solve()
            e2.record()
            b.synchronize()
            torch.cuda.synchronize()
            if r > 0:
                fac.append(e0.elapsed_time(e1))
                sol.append(e1.elapsed_time(e2))
        f, s_ = statistics.median(fac), statistics.median(sol)
        out = {"systems_per_s": S * 1e3 / (f + s_), "factor_ms": f, "solve_ms": s_}
        if prec == "mixed":
            out["worst_rel_residual"] = max(b.info(i)["rel_residual"] for i in range(S))
            out["max_refine_steps"] = max(b.info(i)["refine_steps"] for i in range(S))
        else:
            out["max_refine_steps"] = 0
        pk = ("f32", "FP32") if prec == "mixed" else ("f64", "FP64")
        out["roofline"] = leg_roofline(list(zip(Ns.tolist(), ns.tolist(), ks.tolist())), 8, f, s_,
                                       peaks[pk[0]], pk[1], hbm)
        xs = {}
        if check:
            import oracle.oracle as O
            xs = {i: b.systems[i].d_tensor.permute(2, 1, 0).contiguous().cpu().numpy() for i in sample}
            out["sample_worst_rel_residual"] = max(
                O.rel_residual(O.from_storage(host[i][0]), O.from_storage(host[i][1]), O.from_storage(xs[i]),
                               O.from_storage(host[i][2])) for i in sample)
        return out, xs

    import gc
    xs_by = {}
    for prec in ("mixed", "plain"):
        name = "mixed" if prec == "mixed" else "plain_fp64"
        res[name], xs_by[name] = leg(prec)
        gc.collect()
        torch.cuda.empty_cache()
    if check:
        # the sampled systems on the host cores: one BLAS thread per system, all cores
        from oracle import cref
        cores = os.cpu_count() or 1
        cref.lib(True)
        cref.set_blas_threads(1)
        systems = [tuple(a.copy() for a in host[i]) for i in sample]
        t0 = time.perf_counter()
        info = cref.solve_many(systems, cores)
        tcpu = time.perf_counter() - t0
        assert not info.any()
        xref = {i: sy[2] for i, sy in zip(sample, systems)}
        res["cpu_baseline"] = {"value": len(sample) / tcpu, "unit": "systems/s", "cores": cores, "kind": "port",
                               "sample": f"{len(sample)} of the {S} systems (every {sample_every}th), "
                                         "C restatement of backbone_cpu.jl, one BLAS thread per system, "
                                         f"{cores} systems at a time"}
        for name, xs in xs_by.items():
            res[name]["sample_worst_rel_error_vs_oracle"] = max(rel_err_stor(xs[i], xref[i]) for i in sample)
    res["mixed_over_plain_fp64"] = res["mixed"]["systems_per_s"] / res["plain_fp64"]["systems_per_s"]
    return res


def run_served_legs(bss, check, n_requests=1200, rate=2000.0):
    models, reqs = gen_kf_stream(n_requests, rate)
    out = {"workload": f"{n_requests} Kalman-smoother requests, n in {{8,16,32,64}}, N~U{{50..5000}}, "
                       f"Poisson {rate:g} req/s, 30% repeat RHS on resident factors, 100 GB budget"}
    out["mixed"] = run_served(bss, "mixed", models, reqs, check=check)
    out["plain_fp64"] = run_served(bss, "plain", models, reqs, check=check)
    sat = [dict(r, t=0.0) for r in reqs]
    out["saturated_mixed"] = run_served(bss, "mixed", models, sat, check=check)
    out["saturated_plain_fp64"] = run_served(bss, "plain", models, sat, check=check)
    out["saturated_mixed_over_plain_fp64"] = (out["saturated_mixed"]["solves_per_s"] /
                                              out["saturated_plain_fp64"]["solves_per_s"])
    return out


def roofline_chain_factor(bss, A, B, d, hbm_gbs, peak_kind):
    """Roofline of the dominant kernel of the mixed path: the level-0 chain
    factor kernel (FP64 A_i, B_i in; FP32 V_i, W_i, Y_i out).  Algorithmic
    bytes per launch = sum over interior blocks of 2 n^2 * 8 (A_i, B_i read)
    + 3 n^2 * 4 (V, W, Y written); duration from CUDA events around a
    factorize_levels(1) call (the level-0 chain kernel + its assembly)."""
    import torch
    from blockstructuredsolvers_gb300 import _lib
    L = _lib.load()
    data = bss.initialize_batched(N_BLK, N_SZ, torch.float64, k=K_RHS, precision="mixed")
    data.A_tensor[:, :, :N_BLK].copy_(A)
    data.B_tensor[:, :, :N_BLK - 1].copy_(B)
    info = bss.get_info(data)
    torch.cuda.synchronize()
    ts = []
    for r in range(6):
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record()
        _lib.check(L.bss_factorize_levels(data.handle, 1))
        e1.record()
        torch.cuda.synchronize()
        if r:
            ts.append(e0.elapsed_time(e1))
    import ctypes
    Nl = ctypes.c_int64()
    Q = ctypes.c_int64()
    _lib.check(L.bss_get_level(data.handle, 0, ctypes.byref(Nl), ctypes.byref(Q), None, None, None, None))
    interior = Nl.value - (Q.value + 1)
    nn = N_SZ * N_SZ
    alg_bytes = interior * (2 * nn * 8 + 3 * nn * 4) + (Q.value + 1) * nn * 8
    ms = statistics.median(ts)
    ach = alg_bytes / (ms * 1e-3) / 1e9
    # DRAM bytes (read + write) per interior block of this kernel from one ncu
    # capture of a smaller launch (the traffic of a chain grows in proportion
    # to its blocks), used only while the kernel source still matches the
    # capture's
    per_blk, src = captured_traffic()
    traffic = per_blk * interior if per_blk else None
    return {"kernel": "chain_factor level 0 (FP64 A, B in; FP32 V, W, Y out) + assemble_schur", "bound": "hbm",
            "achieved": ach, "peak": hbm_gbs, "unit": "GB/s", "frac": ach / hbm_gbs,
            "peak_source": f"hbm_gbs of MEASURED_PEAKS.json ({peak_kind})", "duration_ms": ms,
            "algorithmic_bytes": alg_bytes, "partitions": Q.value, "traffic": traffic,
            "traffic_source": src,
            "note": "latency-bound chain: the HBM fraction is low by construction"}


TRAFFIC_PROFILE = os.path.join(ROOT, "profiles", "chain64_tc_mixed_N4096_n64.md")
KERNEL_SOURCES = [os.path.join(ROOT, "blockstructuredsolvers_gb300", "csrc", f)
                  for f in ("bss_kernels.cuh", "bss_tc.cuh", "bss_chain64_tc.cuh")]


def kernel_source_sha16():
    """sha256 (first 16 hex digits) of the device sources of the chain kernels."""
    import hashlib
    h = hashlib.sha256()
    for f in KERNEL_SOURCES:
        if os.path.exists(f):
            with open(f, "rb") as fh:
                h.update(fh.read())
    return h.hexdigest()[:16]


def captured_traffic():
    """(bytes per interior block, source note) from the ncu summary of the
    level-0 chain factor kernel, or (None, why) when its recorded kernel
    source hash differs from the current sources."""
    import re
    try:
        with open(TRAFFIC_PROFILE) as f:
            txt = f.read()
    except OSError:
        return None, "no ncu summary"
    m1 = re.search(r"traffic_per_interior_block_bytes\s*=\s*([0-9.eE+]+)", txt)
    m2 = re.search(r"kernel_source_sha16\s*=\s*([0-9a-f]{16})", txt)
    if not (m1 and m2):
        return None, "the ncu summary records no per-block traffic"
    if m2.group(1) != kernel_source_sha16():
        return None, "the ncu summary was taken on other kernel sources (hash differs): traffic not reported"
    return float(m1.group(1)), ("ncu dram__bytes_read.sum + dram__bytes_write.sum per interior block of the "
                                "capture in " + os.path.basename(TRAFFIC_PROFILE) + ", times interior blocks")


def run_case(name, reps=3):
    """A small workload for profiler captures: `reps` factorize!+solve! calls."""
    import numpy as np
    import torch
    import blockstructuredsolvers_gb300 as bss
    dev = torch.device("cuda", 0)
    g = torch.Generator(device=dev).manual_seed(5)
    if name in ("chain_n64", "chain_n64_k16", "wide_n128", "headline_eager", "wide_n128_k4", "wide_n128_k4_16k"):
        N, n = {"chain_n64": (4096, 64), "chain_n64_k16": (4096, 64), "wide_n128": (2048, 128),
                "headline_eager": (N_BLK, N_SZ), "wide_n128_k4": (4096, 128), "wide_n128_k4_16k": (16384, 128)}[name]
        k = {"chain_n64_k16": 16, "wide_n128_k4": 4, "wide_n128_k4_16k": 4}.get(name, 1)
        eager = name in ("headline_eager", "wide_n128_k4", "wide_n128_k4_16k")
        G = torch.randn((N, n, n), dtype=torch.float64, device=dev, generator=g)
        A = (G @ G.transpose(1, 2) + n * torch.eye(n, dtype=torch.float64, device=dev)).permute(1, 2, 0)
        B = torch.randn((N - 1, n, n), dtype=torch.float64, device=dev, generator=g).permute(1, 2, 0)
        d = torch.rand((N, n, k), dtype=torch.float64, device=dev, generator=g).permute(1, 2, 0)
        data = bss.initialize_batched(N, n, torch.float64, k=k, precision="mixed", use_graphs=not eager)
        data.A_tensor[:, :, :N].copy_(A)
        data.B_tensor[:, :, :N - 1].copy_(B)
        for _ in range(reps):
            data.d_tensor[:, :, :N].copy_(d)
            bss.factorize_(data)
            bss.solve_(data)
        bss.synchronize(data)
    elif name == "csr_n64":
        # the sparse harness's CSR assembly (construct_block_tridiagonal) of N=4096 blocks of n=64
        N, n = 4096, 64
        G = torch.randn((N, n, n), dtype=torch.float64, device=dev, generator=g)
        A = (G @ G.transpose(1, 2) + n * torch.eye(n, dtype=torch.float64, device=dev)).permute(1, 2, 0)
        B = torch.randn((N - 1, n, n), dtype=torch.float64, device=dev, generator=g).permute(1, 2, 0)
        for _ in range(reps):
            M, _ = bss.construct_block_tridiagonal(A, B)
            del M
    elif name in ("batch_small", "batch_2048"):
        rng = np.random.default_rng(1 if name == "batch_small" else 3)
        S = 64 if name == "batch_small" else 2048
        Ns, ns, ks = rng.integers(16, 1025, S), rng.choice([16, 32, 48, 64, 96, 128], S), rng.integers(1, 9, S)
        b = bss.initialize_multi(Ns.tolist(), ns.tolist(), ks.tolist(), torch.float64, precision="mixed")
        for sv in b.systems:
            N, n, k = sv.N, sv.n, sv.k
            G = torch.randn((N, n, n), dtype=torch.float64, device=dev, generator=g)
            sv.A_tensor.copy_((G @ G.transpose(1, 2) + 2 * n * torch.eye(n, dtype=torch.float64, device=dev))
                              .permute(1, 2, 0))
            if N > 1:
                sv.B_tensor.copy_(0.5 * torch.randn((N - 1, n, n), dtype=torch.float64, device=dev,
                                                    generator=g).permute(1, 2, 0))
            sv.d_tensor.copy_(torch.rand((N, n, k), dtype=torch.float64, device=dev, generator=g).permute(1, 2, 0))
        for _ in range(reps):
            b.factorize()
            b.solve()
        b.synchronize()
    else:
        raise SystemExit(f"unknown case {name}")
    torch.cuda.synchronize()
    print(json.dumps({"case": name, "reps": reps, "ok": True}))


def main():
    args = parse()
    if args.case:
        run_case(args.case)
        return
    if args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
