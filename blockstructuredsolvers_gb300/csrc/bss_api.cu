// C-ABI host side of the GB300 batched block-tridiagonal SPD solver.
//
// Mirrors BlockStructuredSolvers.jl's batched GPU solver
//   initialize_batched  (src/gpu_batched.jl:165-182)  -> bss_create_batched
//   factorize!          (src/gpu_batched.jl:184-227)  -> bss_factorize
//   solve!              (src/gpu_batched.jl:229-258)  -> bss_solve
//   initialize_seq/...  (src/gpu_seq.jl:45-84)        -> bss_create_seq
// with library-owned device tensors in the reference's column-major layouts.
//
// Every level of the recursion lives in one device arena allocated at
// create time; factorize/solve only launch kernels (no allocation, no host
// round trip except one scalar per refinement step in mixed precision).
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "bss_internal.h"

using namespace bss;

namespace {
thread_local std::string g_last_error;
}  // namespace

int bss::fail(int code, const std::string &msg)
{
    g_last_error = msg;
    return code;
}

void bss::set_last_error(const std::string &msg) { g_last_error = msg; }

int bss::cuda_fail(cudaError_t e, const char *what)
{
    return fail(e == cudaErrorMemoryAllocation ? BSS_ERR_OOM : BSS_ERR_CUDA,
                std::string(what) + ": " + cudaGetErrorString(e));
}



extern "C" void bss_default_options(bss_options *o)
{
    if (!o) return;
    std::memset(o, 0, sizeof(*o));
    o->precision = BSS_PRECISION_PLAIN;
    o->plan = BSS_PLAN_AUTO;
    o->max_refine = 10;
    o->target_partitions = 0;
    o->seq_cutoff = 0;
    o->use_graphs = 1;
    o->tol = 1e-12;
    o->chain_blocks = 0;
    o->coarsest_fp64 = 0;
}

extern "C" const char *bss_last_error_string(void) { return g_last_error.c_str(); }

extern "C" int64_t bss_kernel_launches(void) { return (int64_t)launch_count(); }

extern "C" const char *bss_version(void)
{
    return "bss-gb300 0.1 (sm_103a; fused chain kernels n<=64; FP32/FP64/mixed)";
}

// ---------------------------------------------------------------------------
// planners
// ---------------------------------------------------------------------------
// _build_sequence (reference src/gpu_batched.jl:112-143): finest-first list of
// (N_l, m_l, P_l); empty when no valid level exists.
static void build_sequence(long long start, std::vector<long long> &Nl, std::vector<long long> &ml,
                           std::vector<long long> &Pl)
{
    Nl.clear();
    ml.clear();
    Pl.clear();
    long long ncur = start;
    for (;;) {
        long long best_m = -1, best_P = -1, backup_m = -1, backup_P = -1;
        const long long max_m = (ncur - 3) / 2;  // C++ truncation == Julia ÷
        for (long long m = 3; m <= max_m; ++m) {
            const long long num = ncur + m, den = m + 1;
            if (num % den == 0) {
                const long long pprev = num / den;
                if (pprev >= 3) {
                    if (m < pprev) {
                        best_m = m;
                        best_P = pprev;
                        break;
                    } else if (backup_m < 0) {
                        backup_m = m;
                        backup_P = pprev;
                    }
                }
            }
        }
        if (best_m < 0 && backup_m >= 0) {
            best_m = backup_m;
            best_P = backup_P;
        }
        if (best_m < 0) break;
        Nl.push_back(ncur);
        ml.push_back(best_m);
        Pl.push_back(best_P);
        ncur = best_P;
    }
}

// find_sequence_upper (gpu_batched.jl:155-162)
static void find_sequence_upper(long long N, std::vector<long long> &Nl, std::vector<long long> &ml,
                                std::vector<long long> &Pl)
{
    long long nuse = N;
    for (;;) {
        build_sequence(nuse, Nl, ml, Pl);
        if (!Nl.empty()) return;
        ++nuse;
    }
}

extern "C" int bss_plan_reference(int64_t N, int64_t *levels, int32_t maxlev, int32_t *nlev, int64_t *coarsest)
{
    if (N < 1 || !nlev || !coarsest) return fail(BSS_ERR_ARG, "bss_plan_reference: bad argument");
    std::vector<long long> Nl, ml, Pl;
    find_sequence_upper(N, Nl, ml, Pl);
    const int L = (int)Nl.size();
    *nlev = L;
    *coarsest = Pl.back();
    if (levels)
        for (int l = 0; l < L && l < maxlev; ++l) {
            levels[3 * l] = Nl[l];
            levels[3 * l + 1] = ml[l];
            levels[3 * l + 2] = Pl[l];
        }
    return BSS_OK;
}

// partition plan of this library: one CTA per partition, partitions sized to
// fill the resident CTA slots of the GPU once (a chain is latency-bound, so
// more partitions than slots only lengthens the next level), then halving
// levels down to a short sequential chain.
static void plan_auto(long long N, long long target, long long cutoff, std::vector<long long> &Ns,
                      std::vector<long long> &Qs, long long &coarsest)
{
    Ns.clear();
    Qs.clear();
    long long ncur = N;
    while (ncur > cutoff) {
        const long long qmax = (ncur - 1) / 2;  // every partition keeps >= 1 interior block
        long long q = std::min(target, qmax);
        if (q < 1) break;
        Ns.push_back(ncur);
        Qs.push_back(q);
        ncur = q + 1;
    }
    coarsest = ncur;
}

// ---------------------------------------------------------------------------
// creation
// ---------------------------------------------------------------------------
namespace {

struct ArenaPlan {
    size_t bytes = 0;
    size_t take(size_t b)
    {
        size_t off = bytes;
        bytes += (b + 255) & ~(size_t)255;
        return off;
    }
};

int chain_ctas_per_sm(int tin, int t, int n, int variant)
{
    if (tin == F64 && t == F32) return chain_factor_ctas_per_sm<double, float>(n, variant);
    if (t == F32) return chain_factor_ctas_per_sm<float, float>(n, variant);
    return chain_factor_ctas_per_sm<double, double>(n, variant);
}

}  // namespace

int bss::plan_handle(bss_handle *h)
{
    const long long n = h->n, k = h->k, nn = n * n;
    const bool mixed = h->opt.precision == BSS_PRECISION_MIXED;
    const int D = h->dtype;
    std::vector<long long> Ns, Qs;
    long long coarsest = h->N;
    {
        // kernel variant: the autotuner's choice for (n, dtype, precision), else the default
        bss_tune_entry tv{};
        h->variant = tuned_plan((int)n, D, h->opt.precision, &tv) ? tv.factor_variant : default_factor_variant();
    }
    if (!h->seq_api) {
        if (h->opt.plan == BSS_PLAN_REFERENCE) {
            std::vector<long long> Nl, ml, Pl;
            find_sequence_upper(h->N_user, Nl, ml, Pl);  // finest first
            for (size_t l = 0; l < Nl.size(); ++l) {
                Ns.push_back(Nl[l]);
                Qs.push_back(Pl[l] - 1);
            }
            coarsest = Pl.back();
        } else {
            int sms = 0;
            cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, h->device);
            const int t0 = mixed ? F32 : D;
            const int tin0 = D;
            bss_tune_entry te{};
            const bool tuned = tuned_plan((int)n, D, h->opt.precision, &te);
            const long long wave = (long long)sms * chain_ctas_per_sm(tin0, t0, (int)n, h->variant);
            long long target = h->opt.target_partitions > 0
                                   ? h->opt.target_partitions
                                   : (tuned ? std::max(1LL, wave * te.wave_mult_x4 / 4) : wave);
            // a coarsest chain of 4 blocks balances one more level against a
            // longer sequential chain
            long long cutoff = h->opt.seq_cutoff > 0 ? h->opt.seq_cutoff : (tuned ? te.seq_cutoff : 4);
            plan_auto(h->N, target, cutoff, Ns, Qs, coarsest);
        }
    }
    h->levels.clear();
    for (size_t l = 0; l < Ns.size(); ++l) {
        Level L;
        L.N = Ns[l];
        L.Q = Qs[l];
        L.seq = false;
        L.t = mixed ? F32 : D;
        L.tin = (l == 0) ? D : L.t;
        h->levels.push_back(L);
    }
    {
        // the sequential coarsest level: plain in the tensor dtype; mixed in
        // FP32 like every other level by default (the FP64 refinement corrects
        // the whole factorization, and GB300's FP64 pipe runs at ~1/64 of
        // FP32), or in FP64 on request (the coarsest Schur complement is the
        // worst-conditioned block system of the recursion)
        Level L;
        L.N = coarsest;
        L.Q = 0;
        L.seq = true;
        L.t = mixed ? (h->opt.coarsest_fp64 ? F64 : F32) : D;
        L.tin = h->levels.empty() ? D : L.t;
        h->levels.push_back(L);
    }
    const int nlev = (int)h->levels.size();
    Layout &o = h->layout;
    ArenaPlan ap;
    o.A = ap.take((size_t)h->N * nn * tsize(D));
    o.B = ap.take((size_t)std::max(h->N - 1, 1LL) * nn * tsize(D));
    o.d = ap.take((size_t)h->N * n * k * tsize(D));
    o.lA.assign(nlev, 0);
    o.lB.assign(nlev, 0);
    o.ld.assign(nlev, 0);
    o.lAf.assign(nlev, 0);
    o.lBf.assign(nlev, 0);
    o.lY.assign(nlev, 0);
    o.lC.assign(nlev, 0);
    o.lb.assign(nlev, 0);
    for (int l = 0; l < nlev; ++l) {
        Level &L = h->levels[l];
        const size_t ts = tsize(L.t);
        if (l > 0) {
            o.lA[l] = ap.take((size_t)L.N * nn * ts);
            o.lB[l] = ap.take((size_t)std::max(L.N - 1, 1LL) * nn * ts);
            o.ld[l] = ap.take((size_t)L.N * n * k * ts);
        }
        if (l == 0 && mixed) {
            o.lAf[l] = ap.take((size_t)L.N * nn * ts);
            o.lBf[l] = ap.take((size_t)std::max(L.N - 1, 1LL) * nn * ts);
        }
        if (!L.seq) {
            o.lY[l] = ap.take((size_t)L.N * nn * ts);
            o.lC[l] = ap.take((size_t)L.Q * 3 * nn * ts);
            o.lb[l] = ap.take((size_t)L.Q * 2 * n * std::max(1LL, (long long)h->kc_max) * ts);
        }
    }
    if (mixed) {
        o.c0 = ap.take((size_t)h->N * n * k * tsize(h->levels[0].t));
        o.x = ap.take((size_t)h->N * n * k * 8);
    }
    o.st = ap.take(sizeof(DevStatus));
    h->arena_bytes = ap.bytes;
    h->info.failed_block = -1;
    h->info.failed_level = -1;
    h->info.rel_residual = -1.0;
    h->info.levels = nlev - 1;
    h->info.coarsest_blocks = coarsest;
    return BSS_OK;
}

int bss::bind_handle(bss_handle *h, char *base, bool alloc_host_status)
{
    const bool mixed = h->opt.precision == BSS_PRECISION_MIXED;
    const Layout &o = h->layout;
    const int nlev = (int)h->levels.size();
    BSS_CUDA(cudaMemsetAsync(base, 0, h->arena_bytes, h->stream));
    h->A = base + o.A;
    h->B = base + o.B;
    h->d = base + o.d;
    for (int l = 0; l < nlev; ++l) {
        Level &L = h->levels[l];
        if (l == 0) {
            L.A = h->A;
            L.B = h->B;
        } else {
            L.A = base + o.lA[l];
            L.B = base + o.lB[l];
            L.d = base + o.ld[l];
        }
        if (l == 0 && mixed) {
            L.Af = base + o.lAf[l];
            L.Bf = base + o.lBf[l];
        } else {
            L.Af = L.A;
            L.Bf = L.B;
        }
        if (!L.seq) {
            L.Y = base + o.lY[l];
            L.C = base + o.lC[l];
            L.bvec = base + o.lb[l];
        }
    }
    if (mixed) {
        h->c0 = base + o.c0;
        h->x64 = reinterpret_cast<double *>(base + o.x);
        h->levels[0].d = h->c0;
    } else {
        h->levels[0].d = h->d;
    }
    h->st = reinterpret_cast<DevStatus *>(base + o.st);
    if (alloc_host_status) {
        BSS_CUDA(cudaMallocHost((void **)&h->h_st, sizeof(DevStatus)));
        std::memset(h->h_st, 0, sizeof(DevStatus));
    }
    // identity padding of A (gpu_batched.jl:177-179: blocks N..N_use, 1-based)
    if (!h->seq_api && h->N > h->N_user - 1) {
        const long long first = h->N_user - 1;
        cudaError_t ie = (h->dtype == F64)
                             ? launch_init_identity<double>((double *)h->A, first, h->N, (int)h->n, h->stream)
                             : launch_init_identity<float>((float *)h->A, first, h->N, (int)h->n, h->stream);
        if (ie != cudaSuccess) return cuda_fail(ie, "init_identity");
    }
    return BSS_OK;
}

namespace {

int build_handle(bss_handle *h)
{
    int rc = plan_handle(h);
    if (rc) return rc;
    cudaError_t e = cudaMalloc((void **)&h->arena, h->arena_bytes);
    if (e != cudaSuccess) {
        h->arena = nullptr;
        return cuda_fail(e, "cudaMalloc(arena)");
    }
    return bind_handle(h, h->arena, true);
}

int check_dims(int64_t N, int64_t n, int64_t k, int32_t dtype)
{
    if (N < 1 || n < 1 || k < 1) return fail(BSS_ERR_ARG, "N, n and k must be >= 1");
    if (dtype != BSS_F32 && dtype != BSS_F64) return fail(BSS_ERR_ARG, "dtype must be BSS_F32 or BSS_F64");
    if (tile_for((int)n) == 0)
        return fail(BSS_ERR_UNSUPPORTED, "block size n=" + std::to_string(n) + " exceeds the limit " +
                                             std::to_string(MAX_WIDE_N));
    return BSS_OK;
}

int create_common(bss_handle *h, int64_t N, int64_t n, int64_t k, int32_t dtype, void *stream, bss_handle **out)
{
    h->n = n;
    h->k = k;
    h->dtype = dtype;
    h->stream = (cudaStream_t)stream;
    h->ls = h->stream;
    cudaError_t e = cudaGetDevice(&h->device);
    if (e != cudaSuccess) {
        delete h;
        return cuda_fail(e, "cudaGetDevice");
    }
    h->kc_max = solve_kc_max((int)n, (int)k, (int)tsize(dtype));
    int rc = build_handle(h);
    if (rc != BSS_OK) {
        if (h->arena) cudaFree(h->arena);
        if (h->h_st) cudaFreeHost(h->h_st);
        delete h;
        return rc;
    }
    *out = h;
    return BSS_OK;
}

}  // namespace

extern "C" int bss_create_batched(int64_t N, int64_t n, int64_t k, int32_t dtype, void *stream,
                                  const bss_options *opt, bss_handle **out)
{
    if (!out) return fail(BSS_ERR_ARG, "out is NULL");
    *out = nullptr;
    int rc = check_dims(N, n, k, dtype);
    if (rc) return rc;
    bss_handle *h = new bss_handle();
    if (opt)
        h->opt = *opt;
    else
        bss_default_options(&h->opt);
    if (h->opt.precision == BSS_PRECISION_MIXED && dtype != BSS_F64) {
        delete h;
        return fail(BSS_ERR_ARG, "mixed precision needs FP64 tensors");
    }
    if (h->opt.precision == BSS_PRECISION_MIXED && residual_smem_bytes<double>((int)n, 1) > (size_t)200 * 1024) {
        delete h;
        return fail(BSS_ERR_UNSUPPORTED, "mixed precision supports n <= 128 (the refinement residual keeps one n x n block in shared memory)");
    }
    if (h->opt.max_refine < 0) h->opt.max_refine = 0;
    h->N_user = N;
    std::vector<long long> Nl, ml, Pl;
    find_sequence_upper(N, Nl, ml, Pl);
    h->N = Nl.front();  // N_use (the finest level of the reference plan)
    return create_common(h, N, n, k, dtype, stream, out);
}

extern "C" int bss_create_seq(int64_t N, int64_t n, int64_t k, int32_t dtype, void *stream, bss_handle **out)
{
    if (!out) return fail(BSS_ERR_ARG, "out is NULL");
    *out = nullptr;
    int rc = check_dims(N, n, k, dtype);
    if (rc) return rc;
    bss_handle *h = new bss_handle();
    bss_default_options(&h->opt);
    h->seq_api = true;
    h->N_user = N;
    h->N = N;
    return create_common(h, N, n, k, dtype, stream, out);
}

extern "C" int bss_destroy(bss_handle *h)
{
    if (!h) return BSS_OK;
    if (h->stream) cudaStreamSynchronize(h->stream);
    else cudaDeviceSynchronize();
    if (h->g_factor) cudaGraphExecDestroy(h->g_factor);
    if (h->g_solve) cudaGraphExecDestroy(h->g_solve);
    if (h->cap_stream) cudaStreamDestroy(h->cap_stream);
    if (h->cap_stream2) cudaStreamDestroy(h->cap_stream2);
    if (h->arena && !h->external_arena) cudaFree(h->arena);
    if (h->h_st) cudaFreeHost(h->h_st);
    delete h;
    return BSS_OK;
}

extern "C" int bss_get_tensors(bss_handle *h, void **A, void **B, void **d)
{
    if (!h) return fail(BSS_ERR_ARG, "handle is NULL");
    if (A) *A = h->A;
    if (B) *B = h->B;
    if (d) *d = h->d;
    return BSS_OK;
}

extern "C" int bss_get_dims(bss_handle *h, int64_t *N, int64_t *n, int64_t *k, int32_t *dtype)
{
    if (!h) return fail(BSS_ERR_ARG, "handle is NULL");
    if (N) *N = h->N;
    if (n) *n = h->n;
    if (k) *k = h->k;
    if (dtype) *dtype = h->dtype;
    return BSS_OK;
}

// ---------------------------------------------------------------------------
// factorize
// ---------------------------------------------------------------------------
namespace {

template <class Tin, class T>
cudaError_t factor_level(bss_handle *h, int l)
{
    return launch_chain_factor<Tin, T>(make_factor_args<Tin, T>(h, l), h->ls);
}

}  // namespace

template <class Tin, class T>
ChainFactorArgs<Tin, T> bss::make_factor_args(bss_handle *h, int l)
{
    Level &L = h->levels[l];
    ChainFactorArgs<Tin, T> a;
    a.A_in = (const Tin *)L.A;
    a.B_in = (const Tin *)L.B;
    a.A_f = (T *)L.Af;
    a.B_f = (T *)L.Bf;
    a.Y = (T *)L.Y;
    a.C = (T *)L.C;
    a.N = L.N;
    a.Q = L.Q;
    a.n = (int)h->n;
    a.seq = L.seq ? 1 : 0;
    a.level = l;
    a.st = h->st;
    a.variant = h->variant;
    return a;
}
template ChainFactorArgs<double, double> bss::make_factor_args<double, double>(bss_handle *, int);
template ChainFactorArgs<double, float> bss::make_factor_args<double, float>(bss_handle *, int);
template ChainFactorArgs<float, float> bss::make_factor_args<float, float>(bss_handle *, int);

namespace {

cudaError_t assemble_level(bss_handle *h, int l)
{
    Level &L = h->levels[l];
    Level &X = h->levels[l + 1];
    const int n = (int)h->n;
    if (L.tin == F64 && L.t == F64)
        return launch_assemble_schur<double, double, double>((const double *)L.A, (const double *)L.C,
                                                             (double *)X.A, (double *)X.B, L.N, L.Q, n, h->ls);
    if (L.tin == F32 && L.t == F32 && X.t == F32)
        return launch_assemble_schur<float, float, float>((const float *)L.A, (const float *)L.C, (float *)X.A,
                                                          (float *)X.B, L.N, L.Q, n, h->ls);
    if (L.tin == F32 && L.t == F32 && X.t == F64)
        return launch_assemble_schur<float, float, double>((const float *)L.A, (const float *)L.C, (double *)X.A,
                                                           (double *)X.B, L.N, L.Q, n, h->ls);
    if (L.tin == F64 && L.t == F32 && X.t == F32)
        return launch_assemble_schur<double, float, float>((const double *)L.A, (const float *)L.C, (float *)X.A,
                                                           (float *)X.B, L.N, L.Q, n, h->ls);
    if (L.tin == F64 && L.t == F32 && X.t == F64)
        return launch_assemble_schur<double, float, double>((const double *)L.A, (const float *)L.C,
                                                            (double *)X.A, (double *)X.B, L.N, L.Q, n, h->ls);
    return cudaErrorInvalidValue;
}

cudaError_t factor_any(bss_handle *h, int l)
{
    const Level &L = h->levels[l];
    if (L.tin == F64 && L.t == F64) return factor_level<double, double>(h, l);
    if (L.tin == F64 && L.t == F32) return factor_level<double, float>(h, l);
    if (L.tin == F32 && L.t == F32) return factor_level<float, float>(h, l);
    return cudaErrorInvalidValue;
}

}  // namespace

static int factorize_upto(bss_handle *h, int upto)
{
    BSS_CUDA(cudaMemsetAsync(&h->st->bad_key, 0xFF, sizeof(unsigned long long), h->ls));
    BSS_CUDA(cudaMemsetAsync(&h->st->tc_timeout, 0, sizeof(int), h->ls));
    const bool mixed = h->opt.precision == BSS_PRECISION_MIXED;
    if (mixed) {
        // ||T||_inf is folded into the first residual after this factorization
        BSS_CUDA(cudaMemsetAsync(&h->st->anorm, 0, sizeof(unsigned long long), h->ls));
        BSS_CUDA(cudaMemsetAsync(&h->st->need_anorm, 0, sizeof(int), h->ls));
        BSS_CUDA(cudaMemsetAsync(&h->st->need_anorm, 1, 1, h->ls));
        h->need_anorm = true;
    }
    const int nlev = (int)h->levels.size();
    for (int l = 0; l < nlev && l < upto; ++l) {
        BSS_CUDA(factor_any(h, l));
        if (!h->levels[l].seq) BSS_CUDA(assemble_level(h, l));
    }
    h->factored = upto >= nlev;
    h->sticky = BSS_OK;
    return BSS_OK;
}

// Run `body` (which enqueues on h->ls): eagerly on the first call, afterwards
// as a CUDA graph captured once on a private stream and launched on the
// handle's stream (the caller's stream may be the legacy default stream,
// which cannot be captured).
template <class F>
static int run_graphed(bss_handle *h, cudaGraphExec_t &exec, int &ncalls, long long &nkern, F body)
{
    if (!h->opt.use_graphs || ncalls++ == 0) {
        h->ls = h->stream;
        return body();
    }
    if (!exec) {
        const long long k0 = launch_count();
        if (!h->cap_stream) BSS_CUDA(cudaStreamCreateWithFlags(&h->cap_stream, cudaStreamNonBlocking));
        if (!h->cap_stream2) BSS_CUDA(cudaStreamCreateWithFlags(&h->cap_stream2, cudaStreamNonBlocking));
        h->ls = h->cap_stream;
        BSS_CUDA(cudaStreamBeginCapture(h->cap_stream, cudaStreamCaptureModeRelaxed));
        const int rc = body();
        cudaGraph_t g = nullptr;
        const cudaError_t e = cudaStreamEndCapture(h->cap_stream, &g);
        h->ls = h->stream;
        if (rc != BSS_OK || e != cudaSuccess) {
            if (g) cudaGraphDestroy(g);
            return rc != BSS_OK ? rc : cuda_fail(e, "cudaStreamEndCapture");
        }
        const cudaError_t ei = cudaGraphInstantiate(&exec, g, 0);
        cudaGraphDestroy(g);
        if (ei != cudaSuccess) {
            exec = nullptr;
            return cuda_fail(ei, "cudaGraphInstantiate");
        }
        nkern = launch_count() - k0;
        count_launches(-nkern);  // capture launched nothing; replays are counted below
    }
    BSS_CUDA(cudaGraphLaunch(exec, h->stream));
    if (nkern >= 0) count_launches(nkern);
    return BSS_OK;
}

extern "C" int bss_factorize(bss_handle *h)
{
    if (!h) return fail(BSS_ERR_ARG, "handle is NULL");
    const int nlev = (int)h->levels.size();
    const int rc = run_graphed(h, h->g_factor, h->n_factor, h->k_factor, [&]() { return factorize_upto(h, nlev); });
    h->factored = true;
    return rc;
}

extern "C" int bss_factorize_levels(bss_handle *h, int32_t nlevels)
{
    if (!h) return fail(BSS_ERR_ARG, "handle is NULL");
    h->ls = h->stream;
    if (nlevels < 0 || nlevels >= (int)h->levels.size())
        return fail(BSS_ERR_ARG, "nlevels must be in [0, number of partitioned levels]");
    return factorize_upto(h, nlevels);
}

extern "C" int bss_get_level(bss_handle *h, int32_t level, int64_t *N, int64_t *Q, void **A, void **B, void **d,
                             int32_t *dtype)
{
    if (!h) return fail(BSS_ERR_ARG, "handle is NULL");
    if (level < 0 || level >= (int)h->levels.size()) return fail(BSS_ERR_ARG, "level out of range");
    const Level &L = h->levels[level];
    if (N) *N = L.N;
    if (Q) *Q = L.Q;
    if (A) *A = L.A;
    if (B) *B = L.B;
    if (d) *d = L.d;
    if (dtype) *dtype = L.t == F64 ? BSS_F64 : BSS_F32;
    return BSS_OK;
}

// ---------------------------------------------------------------------------
// solve
// ---------------------------------------------------------------------------
namespace {

}  // namespace

template <class T>
SolveArgs<T> bss::make_solve_args(bss_handle *h, int l, int j0, int kc)
{
    Level &L = h->levels[l];
    SolveArgs<T> a;
    a.Af = (const T *)L.Af;
    a.Bf = (const T *)L.Bf;
    a.Y = (const T *)L.Y;
    a.d = (T *)L.d;
    a.bvec = (T *)L.bvec;
    a.xsep = (l + 1 < (int)h->levels.size()) ? h->levels[l + 1].d : nullptr;
    a.N = L.N;
    a.Q = L.Q;
    a.n = (int)h->n;
    a.k = (int)h->k;
    a.j0 = j0;
    a.kc = kc;
    a.seq = L.seq ? 1 : 0;
    a.st = h->st;
    return a;
}
template SolveArgs<double> bss::make_solve_args<double>(bss_handle *, int, int, int);
template SolveArgs<float> bss::make_solve_args<float>(bss_handle *, int, int, int);

namespace {

template <class T>
SolveArgs<T> solve_args(bss_handle *h, int l, int j0, int kc)
{
    return make_solve_args<T>(h, l, j0, kc);
}

cudaError_t fwd_level(bss_handle *h, int l, int j0, int kc)
{
    const Level &L = h->levels[l];
    if (L.t == F64) return launch_chain_fwd<double>(solve_args<double>(h, l, j0, kc), h->ls);
    return launch_chain_fwd<float>(solve_args<float>(h, l, j0, kc), h->ls);
}

cudaError_t rhs_level(bss_handle *h, int l, int j0, int kc)
{
    const Level &L = h->levels[l];
    const Level &X = h->levels[l + 1];
    const int n = (int)h->n, k = (int)h->k;
    if (L.t == F64 && X.t == F64)
        return launch_assemble_rhs<double, double>((const double *)L.d, (const double *)L.bvec, (double *)X.d, L.N,
                                                   L.Q, n, k, j0, kc, h->ls);
    if (L.t == F32 && X.t == F32)
        return launch_assemble_rhs<float, float>((const float *)L.d, (const float *)L.bvec, (float *)X.d, L.N, L.Q,
                                                 n, k, j0, kc, h->ls);
    if (L.t == F32 && X.t == F64)
        return launch_assemble_rhs<float, double>((const float *)L.d, (const float *)L.bvec, (double *)X.d, L.N,
                                                  L.Q, n, k, j0, kc, h->ls);
    return cudaErrorInvalidValue;
}

cudaError_t bwd_level(bss_handle *h, int l, int j0, int kc)
{
    const Level &L = h->levels[l];
    const Level &X = h->levels[l + 1];
    if (L.t == F64 && X.t == F64) return launch_chain_bwd<double, double>(solve_args<double>(h, l, j0, kc), h->ls);
    if (L.t == F32 && X.t == F32) return launch_chain_bwd<float, float>(solve_args<float>(h, l, j0, kc), h->ls);
    if (L.t == F32 && X.t == F64) return launch_chain_bwd<float, double>(solve_args<float>(h, l, j0, kc), h->ls);
    return cudaErrorInvalidValue;
}

// solve on levels[0].d in place, all k columns
int chain_solve(bss_handle *h)
{
    const int nlev = (int)h->levels.size();
    for (int j0 = 0; j0 < h->k; j0 += h->kc_max) {
        const int kc = (int)std::min<long long>(h->kc_max, h->k - j0);
        for (int l = 0; l + 1 < nlev; ++l) {
            BSS_CUDA(fwd_level(h, l, j0, kc));
            BSS_CUDA(rhs_level(h, l, j0, kc));
        }
        BSS_CUDA(fwd_level(h, nlev - 1, j0, kc));  // sequential coarsest: fwd + bwd
        for (int l = nlev - 2; l >= 0; --l) BSS_CUDA(bwd_level(h, l, j0, kc));
    }
    return BSS_OK;
}

}  // namespace

// Mixed solve in asynchronous pieces: each enqueues its work on h->ls and
// ends with the status (relative residual, convergence) copied to the pinned
// h->h_st, so a driver can wait on an event instead of the stream and
// interleave many systems (the request server does).
//   begin:   c0 = d; x = A32^{-1} c0; r = d - T x; relres
//   correct: c0 = A32^{-1} r; x += c0; r = d - T x; relres
//   finish:  d = x
namespace {

int residual_check(bss_handle *h)
{
    const double *d64 = (const double *)h->d;
    DevStatus *st = h->st;
    BSS_CUDA(cudaMemsetAsync(&st->rnorm, 0, 2 * sizeof(unsigned long long), h->ls));
    const int wn = h->need_anorm ? 1 : 0;
    h->need_anorm = false;
    if (wn) BSS_CUDA(cudaMemsetAsync(&st->need_anorm, 0, sizeof(int), h->ls));
    if (h->levels[0].t == F32)
        BSS_CUDA((launch_residual_df<float>((const double *)h->A, (const double *)h->B, h->x64, d64,
                                            (float *)h->c0, h->N, (int)h->n, (int)h->k, wn, st, h->ls)));
    else
        BSS_CUDA((launch_residual_df<double>((const double *)h->A, (const double *)h->B, h->x64, d64,
                                             (double *)h->c0, h->N, (int)h->n, (int)h->k, wn, st, h->ls)));
    BSS_CUDA(launch_relres(st, h->opt.tol, h->ls));
    BSS_CUDA(cudaMemcpyAsync(h->h_st, st, sizeof(DevStatus), cudaMemcpyDeviceToHost, h->ls));
    return BSS_OK;
}

int chain_solve(bss_handle *h);

}  // namespace

int bss::mixed_begin(bss_handle *h)
{
    const long long cnt = h->N * h->n * h->k;
    const double *d64 = (const double *)h->d;
    BSS_CUDA(cudaMemsetAsync(&h->st->dnorm, 0, sizeof(unsigned long long), h->ls));
    BSS_CUDA(launch_absmax<double>(d64, cnt, &h->st->dnorm, h->ls));
    if (h->levels[0].t == F32)
        BSS_CUDA((launch_convert<double, float>((float *)h->c0, d64, cnt, h->ls)));
    else
        BSS_CUDA((launch_convert<double, double>((double *)h->c0, d64, cnt, h->ls)));
    int rc = chain_solve(h);
    if (rc) return rc;
    if (h->levels[0].t == F32)
        BSS_CUDA(launch_update<float>(h->x64, (const float *)h->c0, cnt, 1, h->ls));
    else
        BSS_CUDA(launch_update<double>(h->x64, (const double *)h->c0, cnt, 1, h->ls));
    return residual_check(h);
}

int bss::mixed_correct(bss_handle *h)
{
    const long long cnt = h->N * h->n * h->k;
    int rc = chain_solve(h);
    if (rc) return rc;
    if (h->levels[0].t == F32)
        BSS_CUDA(launch_update<float>(h->x64, (const float *)h->c0, cnt, 0, h->ls));
    else
        BSS_CUDA(launch_update<double>(h->x64, (const double *)h->c0, cnt, 0, h->ls));
    return residual_check(h);
}

int bss::mixed_finish(bss_handle *h)
{
    const long long cnt = h->N * h->n * h->k;
    BSS_CUDA(cudaMemcpyAsync(h->d, h->x64, cnt * sizeof(double), cudaMemcpyDeviceToDevice, h->ls));
    return BSS_OK;
}

namespace {

// eager mixed solve: the host waits for the status after every step
int solve_mixed(bss_handle *h)
{
    int rc = mixed_begin(h);
    if (rc) return rc;
    BSS_CUDA(cudaStreamSynchronize(h->ls));
    int steps = 0;
    bool converged = false;
    for (;;) {
        h->info.rel_residual = h->h_st->relres;
        if (h->h_st->done) {
            converged = true;
            break;
        }
        if (steps == h->opt.max_refine) break;
        rc = mixed_correct(h);
        if (rc) return rc;
        BSS_CUDA(cudaStreamSynchronize(h->ls));
        ++steps;
    }
    h->info.refine_steps = steps;
    rc = mixed_finish(h);
    if (rc) return rc;
    if (!converged) h->sticky = BSS_ERR_NOT_CONVERGED;
    return BSS_OK;
}

// Mixed solve as one graph with the refinement loop on the device:
//   prologue (x = first FP32-factor solve)
//   WHILE(loop) { residual (FP64); decide on the device (relres_control);
//                 IF(correct) { FP32-factor solve of r; x += c } }
//   copy x -> d
// relres_control sets both conditional values; the host reads the outcome
// (steps, residual, convergence) at bss_synchronize.  Enqueues on h->ls,
// which is the capture stream cap_stream.
int capture_mixed_solve(bss_handle *h)
{
    const long long cnt = h->N * h->n * h->k;
    const double *d64 = (const double *)h->d;
    const bool c_is_f32 = h->levels[0].t == F32;
    DevStatus *st = h->st;
    const long long k0 = launch_count();
    BSS_CUDA(cudaMemsetAsync(&st->dnorm, 0, sizeof(unsigned long long), h->ls));
    BSS_CUDA(cudaMemsetAsync(&st->iters, 0, sizeof(int), h->ls));
    BSS_CUDA(cudaMemsetAsync(&st->done, 0, sizeof(int), h->ls));
    BSS_CUDA(launch_absmax<double>(d64, cnt, &st->dnorm, h->ls));
    if (c_is_f32)
        BSS_CUDA((launch_convert<double, float>((float *)h->c0, d64, cnt, h->ls)));
    else
        BSS_CUDA((launch_convert<double, double>((double *)h->c0, d64, cnt, h->ls)));
    int rc = chain_solve(h);
    if (rc) return rc;
    if (c_is_f32)
        BSS_CUDA(launch_update<float>(h->x64, (const float *)h->c0, cnt, 1, h->ls));
    else
        BSS_CUDA(launch_update<double>(h->x64, (const double *)h->c0, cnt, 1, h->ls));

    const long long k1 = launch_count();
    cudaStreamCaptureStatus cst;
    cudaGraph_t g = nullptr;
    const cudaGraphNode_t *deps = nullptr;
    size_t nd = 0;
    BSS_CUDA(cudaStreamGetCaptureInfo(h->cap_stream, &cst, nullptr, &g, &deps, nullptr, &nd));
    cudaGraphConditionalHandle hloop;
    BSS_CUDA(cudaGraphConditionalHandleCreate(&hloop, g, 1, cudaGraphCondAssignDefault));
    cudaGraphNodeParams wp = {cudaGraphNodeTypeConditional};
    wp.conditional.handle = hloop;
    wp.conditional.type = cudaGraphCondTypeWhile;
    wp.conditional.size = 1;
    cudaGraphNode_t wnode;
    BSS_CUDA(cudaGraphAddNode(&wnode, g, deps, nullptr, nd, &wp));
    cudaGraph_t wbody = wp.conditional.phGraph_out[0];
    BSS_CUDA(cudaStreamUpdateCaptureDependencies(h->cap_stream, &wnode, nullptr, 1, cudaStreamSetCaptureDependencies));
    cudaGraphConditionalHandle hcorr;
    BSS_CUDA(cudaGraphConditionalHandleCreate(&hcorr, wbody, 0, cudaGraphCondAssignDefault));

    // loop body: residual + decision, then the conditional correction
    h->ls = h->cap_stream2;
    BSS_CUDA(cudaStreamBeginCaptureToGraph(h->cap_stream2, wbody, nullptr, nullptr, 0, cudaStreamCaptureModeRelaxed));
    BSS_CUDA(cudaMemsetAsync(&st->rnorm, 0, 2 * sizeof(unsigned long long), h->ls));
    if (c_is_f32)
        BSS_CUDA((launch_residual_df<float>((const double *)h->A, (const double *)h->B, h->x64, d64,
                                            (float *)h->c0, h->N, (int)h->n, (int)h->k, -1, st, h->ls)));
    else
        BSS_CUDA((launch_residual_df<double>((const double *)h->A, (const double *)h->B, h->x64, d64,
                                             (double *)h->c0, h->N, (int)h->n, (int)h->k, -1, st, h->ls)));
    BSS_CUDA(launch_relres_control(st, h->opt.tol, h->opt.max_refine, hloop, hcorr, h->ls));
    const long long k2 = launch_count();
    cudaGraph_t g2 = nullptr;
    BSS_CUDA(cudaStreamGetCaptureInfo(h->cap_stream2, &cst, nullptr, &g2, &deps, nullptr, &nd));
    cudaGraphNodeParams ip = {cudaGraphNodeTypeConditional};
    ip.conditional.handle = hcorr;
    ip.conditional.type = cudaGraphCondTypeIf;
    ip.conditional.size = 1;
    cudaGraphNode_t inode;
    BSS_CUDA(cudaGraphAddNode(&inode, g2, deps, nullptr, nd, &ip));
    cudaGraph_t ibody = ip.conditional.phGraph_out[0];
    BSS_CUDA(cudaStreamUpdateCaptureDependencies(h->cap_stream2, &inode, nullptr, 1, cudaStreamSetCaptureDependencies));
    cudaGraph_t wb_out = nullptr;
    BSS_CUDA(cudaStreamEndCapture(h->cap_stream2, &wb_out));
    BSS_CUDA(cudaStreamBeginCaptureToGraph(h->cap_stream2, ibody, nullptr, nullptr, 0, cudaStreamCaptureModeRelaxed));
    rc = chain_solve(h);
    if (rc == BSS_OK) {
        if (c_is_f32)
            rc = launch_update<float>(h->x64, (const float *)h->c0, cnt, 0, h->ls) == cudaSuccess ? BSS_OK : BSS_ERR_CUDA;
        else
            rc = launch_update<double>(h->x64, (const double *)h->c0, cnt, 0, h->ls) == cudaSuccess ? BSS_OK
                                                                                                  : BSS_ERR_CUDA;
    }
    const long long k3 = launch_count();
    h->k_pro = k1 - k0;
    h->k_body = k2 - k1;
    h->k_corr = k3 - k2;
    count_launches(-(k3 - k0));  // capture launched nothing; replays are counted at synchronize
    cudaGraph_t ib_out = nullptr;
    const cudaError_t e2 = cudaStreamEndCapture(h->cap_stream2, &ib_out);
    h->ls = h->cap_stream;
    if (rc) return rc;
    if (e2 != cudaSuccess) return cuda_fail(e2, "capture of the correction body");
    BSS_CUDA(cudaMemcpyAsync(h->d, h->x64, cnt * sizeof(double), cudaMemcpyDeviceToDevice, h->ls));
    return BSS_OK;
}

}  // namespace

extern "C" int bss_solve(bss_handle *h)
{
    if (!h) return fail(BSS_ERR_ARG, "handle is NULL");
    if (!h->factored) return fail(BSS_ERR_STATE, "solve before factorize");
    if (h->opt.precision == BSS_PRECISION_MIXED) {
        if (!h->opt.use_graphs || h->n_solve == 0) {
            ++h->n_solve;
            h->ls = h->stream;
            h->graph_solve_pending = false;
            return solve_mixed(h);
        }
        long long dummy = -1;  // the loop's kernel count is known only at synchronize
        const int rc = run_graphed(h, h->g_solve, h->n_solve, dummy, [&]() { return capture_mixed_solve(h); });
        if (rc == BSS_OK) {
            h->graph_solve_pending = true;
            ++h->graph_solves_unsynced;
        }
        return rc;
    }
    return run_graphed(h, h->g_solve, h->n_solve, h->k_solve, [&]() { return chain_solve(h); });
}

extern "C" int bss_synchronize(bss_handle *h)
{
    if (!h) return fail(BSS_ERR_ARG, "handle is NULL");
    BSS_CUDA(cudaStreamSynchronize(h->stream));
    BSS_CUDA(cudaMemcpy(h->h_st, h->st, sizeof(DevStatus), cudaMemcpyDeviceToHost));
    if (h->graph_solve_pending) {  // outcome of the device-side refinement loop
        h->graph_solve_pending = false;
        h->info.refine_steps = h->h_st->iters;
        h->info.rel_residual = h->h_st->relres;
        const long long dit = (long long)(h->h_st->iters_total - h->iters_total_seen);
        count_launches(h->graph_solves_unsynced * (h->k_pro + h->k_body) + dit * (h->k_body + h->k_corr));
        h->graph_solves_unsynced = 0;
        h->iters_total_seen = h->h_st->iters_total;
        h->sticky = h->h_st->done ? BSS_OK : BSS_ERR_NOT_CONVERGED;
    }
    if (h->factored && h->h_st->tc_timeout)
        return fail(BSS_ERR_TIMEOUT, "a bounded device wait expired (tensor-core factorization or streamed solve); "
                                     "the result is void");
    const unsigned long long key = h->h_st->bad_key;
    if (h->factored && key != ~0ULL) {
        h->info.failed_level = (int32_t)(key >> 40);
        h->info.failed_block = (int64_t)(key & ((1ULL << 40) - 1));
        return fail(BSS_ERR_NOT_SPD, "pivot failed at level " + std::to_string(h->info.failed_level) + ", block " +
                                         std::to_string(h->info.failed_block));
    }
    h->info.failed_block = -1;
    h->info.failed_level = -1;
    if (h->sticky != BSS_OK) return fail(h->sticky, "refinement did not reach the tolerance");
    return BSS_OK;
}

extern "C" int bss_get_info(bss_handle *h, bss_info *info)
{
    if (!h || !info) return fail(BSS_ERR_ARG, "NULL argument");
    *info = h->info;
    return BSS_OK;
}

// ---------------------------------------------------------------------------
// standalone residual
// ---------------------------------------------------------------------------
extern "C" int bss_residual(int64_t N, int64_t n, int64_t k, int32_t dtype, const void *A, const void *B,
                            const void *x, const void *d, void *stream, double *out)
{
    if (!out || !A || !x || !d || N < 1 || n < 1 || k < 1) return fail(BSS_ERR_ARG, "bss_residual: bad argument");
    cudaStream_t s = (cudaStream_t)stream;
    DevStatus *st = nullptr;
    BSS_CUDA(cudaMallocAsync((void **)&st, sizeof(DevStatus), s));
    BSS_CUDA(cudaMemsetAsync(st, 0, sizeof(DevStatus), s));
    const long long cnt = N * n * k;
    cudaError_t e;
    if (dtype == BSS_F64) {
        e = launch_absmax<double>((const double *)d, cnt, &st->dnorm, s);
        if (e == cudaSuccess)
            e = launch_residual<double, double>((const double *)A, (const double *)B, (const double *)x,
                                                (const double *)d, nullptr, N, (int)n, (int)k, 1, st, s);
    } else {
        e = launch_absmax<float>((const float *)d, cnt, &st->dnorm, s);
        if (e == cudaSuccess)
            e = launch_residual<float, float>((const float *)A, (const float *)B, (const float *)x, (const float *)d,
                                              nullptr, N, (int)n, (int)k, 1, st, s);
    }
    if (e == cudaSuccess) e = launch_relres(st, 0.0, s);
    DevStatus hs;
    if (e == cudaSuccess) e = cudaMemcpyAsync(&hs, st, sizeof(DevStatus), cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    cudaFreeAsync(st, s);
    if (e != cudaSuccess) return cuda_fail(e, "bss_residual");
    *out = hs.relres;
    return BSS_OK;
}
