// Many independent block-tridiagonal systems of uneven N, n and k solved
// together (no counterpart in the reference, whose batching is over the
// partitions of one system, src/gpu_batched.jl).
//
// Every system is planned like a single handle (its own recursion levels),
// all systems share one device arena, and each recursion level of all
// systems runs as ONE persistent launch per block-size class: CTAs pull
// (system, partition) items from a device work queue, longest chains first.
// The assembly, refinement and vector steps are batched the same way.  The
// launch sequence is fixed at creation (descriptors and work items are
// uploaded once), so after the first call factorize/solve replay CUDA
// graphs; in mixed precision the refinement loop runs on the device while
// any system is unconverged.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstring>
#include <functional>
#include <numeric>
#include <string>
#include <vector>

#include "bss_internal.h"

using namespace bss;

namespace {

// small status kernels over all systems
enum { ST_FACTOR_INIT = 0, ST_SOLVE_INIT = 1 };

__global__ void batch_status_kernel(DevStatus *const *sts, int nsys, int mode)
{
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= nsys) return;
    DevStatus *st = sts[s];
    if (mode == ST_FACTOR_INIT) {
        st->bad_key = ~0ULL;
        st->anorm = 0ULL;
        st->need_anorm = 1;
        st->tc_timeout = 0;
    } else {
        st->dnorm = 0ULL;
        st->rnorm = 0ULL;
        st->xnorm = 0ULL;
        st->iters = 0;
        st->done = 0;
    }
}

__global__ void batch_gather_status_kernel(DevStatus *const *sts, DevStatus *out, int nsys)
{
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s < nsys) out[s] = *sts[s];
}

inline int grid1d(int n) { return (n + 127) / 128; }

struct Step {
    std::function<cudaError_t(cudaStream_t)> run;
    std::string what;  // kernel and launch shape, for error messages
};

}  // namespace

struct bss_batch {
    int nsys = 0;
    int dtype = F64;
    bss_options opt{};
    bool mixed = false;
    cudaStream_t stream = nullptr;
    cudaStream_t cap = nullptr, cap2 = nullptr;
    int device = 0;
    std::vector<bss_handle *> sys;
    char *arena = nullptr;
    char *meta = nullptr;  // descriptors, work items, queue heads, status pointers
    DevStatus **d_sts = nullptr;
    DevStatus *d_gather = nullptr;
    int *d_any = nullptr;   // [0] any system continues, [1] loop round
    std::vector<DevStatus> h_gather;
    std::vector<Step> factor_steps, solve_steps, resid_steps, corr_steps, pro_steps, epi_steps;
    cudaGraphExec_t g_factor = nullptr, g_solve = nullptr;
    int n_factor = 0, n_solve = 0;
    long long k_factor = 0, k_solve = 0;  // kernels per replay (mixed: prologue + epilogue)
    long long k_body = 0, k_corr = 0;     // mixed graph: per loop round, per correction
    long long graph_solves_unsynced = 0;
    bool factored = false;
    bool solve_pending = false;
    int sms = 152;
};

namespace {

// host blob of device metadata, laid out then uploaded once
struct Blob {
    std::vector<char> bytes;
    size_t put(const void *p, size_t n)
    {
        size_t off = (bytes.size() + 255) & ~(size_t)255;
        bytes.resize(off + n);
        if (p && n) std::memcpy(bytes.data() + off, p, n);
        return off;
    }
};


template <class T>
size_t put_vec(Blob &b, const std::vector<T> &v)
{
    return b.put(v.data(), v.size() * sizeof(T));
}

int nb_class(long long n) { return tile_for((int)n); }

// finest-level blocks per partition of every batch system: the caller's
// value, else the autotuner's for (n, dtype, precision), else 32 (mixed) /
// 128 (plain)
long long batch_chain_blocks(const bss_options &o, int n, int dtype)
{
    if (o.chain_blocks > 0) return o.chain_blocks;
    bss_tune_entry te{};
    if (tuned_plan(n, dtype, o.precision, &te) && te.chain_blocks > 0) return te.chain_blocks;
    return o.precision == BSS_PRECISION_MIXED ? 32 : 128;
}

// ------------------------------------------------------------------ launchers
template <class Tin, class T, int NB>
cudaError_t queue_factor_nb(const ChainFactorArgs<Tin, T> *descs, const WorkItem *items, int nitems, int *head,
                            int sms, cudaStream_t s)
{
    const size_t smem = chain_factor_smem<T, NB>();
    auto kern = chain_factor_queue_kernel<Tin, T, NB>;
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    int per = 1;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, kern, Tile<NB>::THREADS, smem);
    int grid = std::max(1, std::min(nitems, sms * std::max(per, 1)));
    e = cudaMemsetAsync(head, 0, sizeof(int), s);
    if (e != cudaSuccess) return e;
    kern<<<grid, Tile<NB>::THREADS, smem, s>>>(descs, items, nitems, head);
    count_launch();
    return cudaGetLastError();
}

template <class Tin, class T, bool TC>
cudaError_t queue_factor_wide(const ChainFactorArgs<Tin, T> *descs, const WorkItem *items, int nitems, int *head,
                              int sms, cudaStream_t s)
{
    const size_t smem = wide_factor_smem<T, TC>();
    auto kern = wide_chain_factor_queue_kernel<Tin, T, TC>;
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    cudaFuncSetAttribute(kern, cudaFuncAttributePreferredSharedMemoryCarveout, 100);
    const int per = ctas_per_sm(kern, WIDE_THREADS, smem);
    int grid = std::max(1, std::min(nitems, sms * per));
    e = cudaMemsetAsync(head, 0, sizeof(int), s);
    if (e != cudaSuccess) return e;
    kern<<<grid, WIDE_THREADS, smem, s>>>(descs, items, nitems, head);
    count_launch();
    return cudaGetLastError();
}

template <class Tin, class T>
cudaError_t queue_factor(int nb, const ChainFactorArgs<Tin, T> *descs, const WorkItem *items, int nitems, int *head,
                         int sms, cudaStream_t s)
{
    switch (nb) {
    case WIDE_CLASS: return queue_factor_wide<Tin, T, false>(descs, items, nitems, head, sms, s);
    case WIDE_CLASS + 1: return queue_factor_wide<Tin, T, std::is_same<T, float>::value>(descs, items, nitems, head,
                                                                                         sms, s);
    case 16: return queue_factor_nb<Tin, T, 16>(descs, items, nitems, head, sms, s);
    case 32: return queue_factor_nb<Tin, T, 32>(descs, items, nitems, head, sms, s);
    default: return queue_factor_nb<Tin, T, 64>(descs, items, nitems, head, sms, s);
    }
}

template <class T>
cudaError_t queue_fwd(const SolveArgs<T> *descs, const WorkItem *items, int nitems, int *head, size_t smem, int sms,
                      bool staged, cudaStream_t s)
{
    auto kern = staged ? chain_fwd_queue_kernel<T, true> : chain_fwd_queue_kernel<T, false>;
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    int per = 1;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, kern, SOLVE_THREADS, smem);
    const int grid = std::max(1, std::min(nitems, sms * std::max(per, 1)));
    e = cudaMemsetAsync(head, 0, sizeof(int), s);
    if (e != cudaSuccess) return e;
    kern<<<grid, SOLVE_THREADS, smem, s>>>(descs, items, nitems, head);
    count_launch();
    return cudaGetLastError();
}

template <class T, class Tsep>
cudaError_t queue_bwd(const SolveArgs<T> *descs, const WorkItem *items, int nitems, int *head, size_t smem, int sms,
                      bool staged, cudaStream_t s)
{
    auto kern = staged ? chain_bwd_queue_kernel<T, Tsep, true> : chain_bwd_queue_kernel<T, Tsep, false>;
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    int per = 1;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, kern, SOLVE_THREADS, smem);
    const int grid = std::max(1, std::min(nitems, sms * std::max(per, 1)));
    e = cudaMemsetAsync(head, 0, sizeof(int), s);
    if (e != cudaSuccess) return e;
    kern<<<grid, SOLVE_THREADS, smem, s>>>(descs, items, nitems, head);
    count_launch();
    return cudaGetLastError();
}

// ------------------------------------------------------------------ planning
struct Builder {
    bss_batch *b;
    Blob blob;
    // steps are recorded with blob offsets and bound to device addresses after upload
    std::vector<std::function<Step(char *)>> factor, solve, resid, corr, pro, epi;
};

template <class Tin, class T>
void plan_factor_level(Builder &B, int level, bool coarsest)
{
    bss_batch *b = B.b;
    // wide blocks: the tensor-core form (FP32, n <= 128) is its own launch class
    for (int nb : {16, 32, 64, (int)WIDE_CLASS, (int)WIDE_CLASS + 1}) {
        std::vector<ChainFactorArgs<Tin, T>> descs;
        std::vector<WorkItem> items;
        std::vector<long long> len;
        for (int s = 0; s < b->nsys; ++s) {
            bss_handle *h = b->sys[s];
            const int L = (int)h->levels.size();
            const int l = coarsest ? L - 1 : level;
            int cls = nb_class(h->n);
            if (cls == WIDE_CLASS && wide_uses_tc<T>((int)h->n)) cls = WIDE_CLASS + 1;
            if (cls != nb || l >= L) continue;
            const Level &lv = h->levels[l];
            if (lv.seq != coarsest) continue;
            if ((lv.tin == F64) != std::is_same<Tin, double>::value || (lv.t == F64) != std::is_same<T, double>::value)
                continue;
            const int di = (int)descs.size();
            descs.push_back(make_factor_args<Tin, T>(h, l));
            const long long q = lv.seq ? 1 : lv.Q;
            for (long long p = 0; p < q; ++p) {
                items.push_back(WorkItem{di, (int)p});
                len.push_back(lv.seq ? lv.N : (lv.N - 1) / lv.Q);
            }
        }
        if (items.empty()) continue;
        std::vector<int> ord(items.size());
        std::iota(ord.begin(), ord.end(), 0);
        std::stable_sort(ord.begin(), ord.end(), [&](int a, int c) { return len[a] > len[c]; });
        std::vector<WorkItem> sorted;
        for (int i : ord) sorted.push_back(items[i]);
        const size_t od = put_vec(B.blob, descs), oi = put_vec(B.blob, sorted), oh = B.blob.put(nullptr, 16);
        const int ni = (int)sorted.size();
        const int sms = b->sms;
        B.factor.push_back([=](char *base) {
            Step st;
            st.what = std::string("plan_factor_level") + " items=" + std::to_string(ni);
            st.run = [=](cudaStream_t s) {
                return queue_factor<Tin, T>(nb, (const ChainFactorArgs<Tin, T> *)(base + od),
                                            (const WorkItem *)(base + oi), ni, (int *)(base + oh), sms, s);
            };
            return st;
        });
    }
}

template <class Tsrc, class T, class Tdst>
void plan_asm_schur(Builder &B, int level)
{
    bss_batch *b = B.b;
    std::vector<AsmSchurDesc<Tsrc, T, Tdst>> descs;
    std::vector<WorkItem> items;
    for (int s = 0; s < b->nsys; ++s) {
        bss_handle *h = b->sys[s];
        if (level + 1 >= (int)h->levels.size() || h->levels[level].seq) continue;
        const Level &L = h->levels[level], &X = h->levels[level + 1];
        if ((L.tin == F64) != std::is_same<Tsrc, double>::value || (L.t == F64) != std::is_same<T, double>::value ||
            (X.t == F64) != std::is_same<Tdst, double>::value)
            continue;
        AsmSchurDesc<Tsrc, T, Tdst> d{(const Tsrc *)L.A, (const T *)L.C, (Tdst *)X.A, (Tdst *)X.B, L.N, L.Q,
                                      (int)h->n};
        const int di = (int)descs.size();
        descs.push_back(d);
        const long long total = (2 * L.Q + 1) * h->n * h->n;
        for (long long c = 0; c * BATCH_CHUNK < total; ++c) items.push_back(WorkItem{di, (int)c});
    }
    if (items.empty()) return;
    const size_t od = put_vec(B.blob, descs), oi = put_vec(B.blob, items);
    const int ni = (int)items.size();
    B.factor.push_back([=](char *base) {
        Step st;
        st.what = std::string("plan_asm_schur") + " items=" + std::to_string(ni);
        st.run = [=](cudaStream_t s) {
            assemble_schur_batch_kernel<Tsrc, T, Tdst><<<ni, 256, 0, s>>>(
                (const AsmSchurDesc<Tsrc, T, Tdst> *)(base + od), (const WorkItem *)(base + oi));
            count_launch();
            return cudaGetLastError();
        };
        return st;
    });
}

// forward sweeps (and the coarsest level's full solve) of one level
template <class T>
void plan_fwd(Builder &B, int level, bool coarsest, bool staged, int nb, std::vector<std::function<Step(char *)>> &dst)
{
    bss_batch *b = B.b;
    std::vector<SolveArgs<T>> descs;
    std::vector<WorkItem> items;
    std::vector<long long> len;
    size_t smem = 0;
    for (int s = 0; s < b->nsys; ++s) {
        bss_handle *h = b->sys[s];
        const int L = (int)h->levels.size();
        const int l = coarsest ? L - 1 : level;
        if (l >= L) continue;
        const Level &lv = h->levels[l];
        if (lv.seq != coarsest || (lv.t == F64) != std::is_same<T, double>::value) continue;
        if (solve_staged<T>((int)h->n, (int)h->k) != staged || nb_class(h->n) != nb) continue;
        const int di = (int)descs.size();
        descs.push_back(make_solve_args<T>(h, l, 0, (int)h->k));
        smem = std::max(smem, solve_smem_bytes<T>((int)h->n, (int)h->k, staged));
        const long long q = lv.seq ? 1 : lv.Q;
        for (long long p = 0; p < q; ++p) {
            items.push_back(WorkItem{di, (int)p});
            len.push_back(lv.seq ? lv.N : (lv.N - 1) / lv.Q);
        }
    }
    if (items.empty()) return;
    std::vector<int> ord(items.size());
    std::iota(ord.begin(), ord.end(), 0);
    std::stable_sort(ord.begin(), ord.end(), [&](int a, int c) { return len[a] > len[c]; });
    std::vector<WorkItem> sorted;
    for (int i : ord) sorted.push_back(items[i]);
    const size_t od = put_vec(B.blob, descs), oi = put_vec(B.blob, sorted), oh = B.blob.put(nullptr, 16);
    const int ni = (int)sorted.size();
    const int sms = b->sms;
    dst.push_back([=](char *base) {
        Step st;
        st.what = std::string("plan_fwd") + " items=" + std::to_string(ni) + " smem=" + std::to_string(smem) + (staged ? " staged" : " direct");
        st.run = [=](cudaStream_t s) {
            return queue_fwd<T>((const SolveArgs<T> *)(base + od), (const WorkItem *)(base + oi), ni,
                                (int *)(base + oh), smem, sms, staged, s);
        };
        return st;
    });
}

template <class T, class Tn>
void plan_asm_rhs(Builder &B, int level, std::vector<std::function<Step(char *)>> &dst)
{
    bss_batch *b = B.b;
    std::vector<AsmRhsDesc<T, Tn>> descs;
    std::vector<WorkItem> items;
    for (int s = 0; s < b->nsys; ++s) {
        bss_handle *h = b->sys[s];
        if (level + 1 >= (int)h->levels.size() || h->levels[level].seq) continue;
        const Level &L = h->levels[level], &X = h->levels[level + 1];
        if ((L.t == F64) != std::is_same<T, double>::value || (X.t == F64) != std::is_same<Tn, double>::value)
            continue;
        AsmRhsDesc<T, Tn> d{(const T *)L.d, (const T *)L.bvec, (Tn *)X.d, L.N, L.Q,
                            (int)h->n, (int)h->k, 0, (int)h->k};
        const int di = (int)descs.size();
        descs.push_back(d);
        const long long total = (L.Q + 1) * h->n * h->k;
        for (long long c = 0; c * BATCH_CHUNK < total; ++c) items.push_back(WorkItem{di, (int)c});
    }
    if (items.empty()) return;
    const size_t od = put_vec(B.blob, descs), oi = put_vec(B.blob, items);
    const int ni = (int)items.size();
    dst.push_back([=](char *base) {
        Step st;
        st.what = std::string("plan_asm_rhs") + " items=" + std::to_string(ni);
        st.run = [=](cudaStream_t s) {
            assemble_rhs_batch_kernel<T, Tn><<<ni, 256, 0, s>>>((const AsmRhsDesc<T, Tn> *)(base + od),
                                                               (const WorkItem *)(base + oi));
            count_launch();
            return cudaGetLastError();
        };
        return st;
    });
}

template <class T, class Tsep>
void plan_bwd(Builder &B, int level, bool staged, int nb, std::vector<std::function<Step(char *)>> &dst)
{
    bss_batch *b = B.b;
    std::vector<SolveArgs<T>> descs;
    std::vector<WorkItem> items;
    std::vector<long long> len;
    size_t smem = 0;
    for (int s = 0; s < b->nsys; ++s) {
        bss_handle *h = b->sys[s];
        if (level + 1 >= (int)h->levels.size() || h->levels[level].seq) continue;
        const Level &L = h->levels[level], &X = h->levels[level + 1];
        if ((L.t == F64) != std::is_same<T, double>::value || (X.t == F64) != std::is_same<Tsep, double>::value)
            continue;
        if (solve_staged<T>((int)h->n, (int)h->k) != staged || nb_class(h->n) != nb) continue;
        const int di = (int)descs.size();
        descs.push_back(make_solve_args<T>(h, level, 0, (int)h->k));
        smem = std::max(smem, solve_smem_bytes<T>((int)h->n, (int)h->k, staged));
        for (long long p = 0; p < L.Q; ++p) {
            items.push_back(WorkItem{di, (int)p});
            len.push_back((L.N - 1) / L.Q);
        }
    }
    if (items.empty()) return;
    std::vector<int> ord(items.size());
    std::iota(ord.begin(), ord.end(), 0);
    std::stable_sort(ord.begin(), ord.end(), [&](int a, int c) { return len[a] > len[c]; });
    std::vector<WorkItem> sorted;
    for (int i : ord) sorted.push_back(items[i]);
    const size_t od = put_vec(B.blob, descs), oi = put_vec(B.blob, sorted), oh = B.blob.put(nullptr, 16);
    const int ni = (int)sorted.size();
    const int sms = b->sms;
    dst.push_back([=](char *base) {
        Step st;
        st.what = std::string("plan_bwd") + " items=" + std::to_string(ni) + " smem=" + std::to_string(smem) + (staged ? " staged" : " direct");
        st.run = [=](cudaStream_t s) {
            return queue_bwd<T, Tsep>((const SolveArgs<T> *)(base + od), (const WorkItem *)(base + oi), ni,
                                      (int *)(base + oh), smem, sms, staged, s);
        };
        return st;
    });
}

// one full chain solve of every system on its level-0 RHS (levels[0].d)
void plan_chain_solve(Builder &B, int maxpart, std::vector<std::function<Step(char *)>> &dst)
{
    // one launch per (type, staged form, block-size class): the shared
    // memory of a launch is sized for its largest system, so mixing classes
    // would cap every CTA at the occupancy of the largest blocks
    static const int kClasses[] = {16, 32, 64, WIDE_CLASS};
    for (int l = 0; l < maxpart; ++l) {
        for (bool st : {true, false})
            for (int nb : kClasses) {
                plan_fwd<float>(B, l, false, st, nb, dst);
                plan_fwd<double>(B, l, false, st, nb, dst);
            }
        plan_asm_rhs<float, float>(B, l, dst);
        plan_asm_rhs<float, double>(B, l, dst);
        plan_asm_rhs<double, double>(B, l, dst);
    }
    for (bool st : {true, false})
        for (int nb : kClasses) {
            plan_fwd<float>(B, 0, true, st, nb, dst);
            plan_fwd<double>(B, 0, true, st, nb, dst);
        }
    for (int l = maxpart - 1; l >= 0; --l)
        for (bool st : {true, false})
            for (int nb : kClasses) {
                plan_bwd<float, float>(B, l, st, nb, dst);
                plan_bwd<float, double>(B, l, st, nb, dst);
                plan_bwd<double, double>(B, l, st, nb, dst);
            }
}

template <class Tc>
void plan_vec(Builder &B, int op, std::vector<std::function<Step(char *)>> &dst)
{
    bss_batch *b = B.b;
    std::vector<VecDesc<Tc>> descs;
    std::vector<WorkItem> items;
    for (int s = 0; s < b->nsys; ++s) {
        bss_handle *h = b->sys[s];
        if ((h->levels[0].t == F64) != std::is_same<Tc, double>::value) continue;
        const long long cnt = h->N * h->n * h->k;
        VecDesc<Tc> d{h->x64, (Tc *)h->c0, (double *)h->d, cnt, h->st};
        const int di = (int)descs.size();
        descs.push_back(d);
        for (long long c = 0; c * BATCH_CHUNK < cnt; ++c) items.push_back(WorkItem{di, (int)c});
    }
    if (items.empty()) return;
    const size_t od = put_vec(B.blob, descs), oi = put_vec(B.blob, items);
    const int ni = (int)items.size();
    dst.push_back([=](char *base) {
        Step st;
        st.what = std::string("plan_vec") + " items=" + std::to_string(ni);
        st.run = [=](cudaStream_t s) {
            vec_batch_kernel<Tc><<<ni, 256, 0, s>>>((const VecDesc<Tc> *)(base + od), (const WorkItem *)(base + oi), op);
            count_launch();
            return cudaGetLastError();
        };
        return st;
    });
}

// residual CTA shape per block-size class: 512 threads for the wide class
// (one CTA per SM fits its staged B_i), 256 otherwise
inline size_t res_smem(int nb, int n, int k)
{
    return nb == (int)WIDE_CLASS ? residual_df_smem_bytes<512>(n, k) : residual_df_smem_bytes<256>(n, k);
}

template <class Tr>
void plan_resid(Builder &B, int nb, std::vector<std::function<Step(char *)>> &dst)
{
    const bool wide = nb == (int)WIDE_CLASS;
    bss_batch *b = B.b;
    std::vector<ResidualDesc<Tr>> descs;
    std::vector<WorkItem> items;
    size_t smem = 0;
    for (int s = 0; s < b->nsys; ++s) {
        bss_handle *h = b->sys[s];
        if ((h->levels[0].t == F64) != std::is_same<Tr, double>::value || nb_class(h->n) != nb) continue;
        const long long per = std::max(1LL, std::min(h->N, 32LL));
        int kc = (int)h->k;  // column chunk whose shared memory fits
        while (kc > 1 && res_smem(nb, (int)h->n, kc) > (nb == (int)WIDE_CLASS ? residual_df_smem_cap<512>()
                                                                                 : residual_df_smem_cap<256>()))
            kc = (kc + 1) / 2;
        for (int j0 = 0; j0 < h->k; j0 += kc) {
            const int kk = (int)std::min<long long>(kc, h->k - j0);
            ResidualDesc<Tr> d{(const double *)h->A, (const double *)h->B, h->x64, (const double *)h->d,
                               (Tr *)h->c0, h->N, (int)h->n, (int)h->k, j0, kk, j0 == 0 ? -1 : 0, per, h->st};
            const int di = (int)descs.size();
            descs.push_back(d);
            smem = std::max(smem, res_smem(nb, (int)h->n, kk));
            for (long long c = 0; c * per < h->N; ++c) items.push_back(WorkItem{di, (int)c});
        }
    }
    if (items.empty()) return;
    const size_t od = put_vec(B.blob, descs), oi = put_vec(B.blob, items);
    const int ni = (int)items.size();
    dst.push_back([=](char *base) {
        Step st;
        st.what = std::string("plan_resid") + " items=" + std::to_string(ni) + " smem=" + std::to_string(smem);
        st.run = [=](cudaStream_t s) {
            auto run = [&](auto kern, int threads) {
                cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
                if (e != cudaSuccess) return e;
                e = cudaFuncSetAttribute(kern, cudaFuncAttributePreferredSharedMemoryCarveout, 100);
                if (e != cudaSuccess) return e;
                kern<<<ni, threads, smem, s>>>((const ResidualDesc<Tr> *)(base + od), (const WorkItem *)(base + oi));
                count_launch();
                return cudaGetLastError();
            };
            return wide ? run(residual_batch_kernel<Tr, 512>, 512) : run(residual_batch_kernel<Tr, 256>, 256);
        };
        return st;
    });
}

int run_steps(const std::vector<Step> &steps, cudaStream_t s)
{
    for (const Step &st : steps) {
        const cudaError_t e = st.run(s);
        if (e != cudaSuccess) return cuda_fail(e, ("batch step " + st.what).c_str());
    }
    return BSS_OK;
}

int build_batch(bss_batch *b)
{
    Builder B;
    B.b = b;
    int maxpart = 0;
    for (bss_handle *h : b->sys) maxpart = std::max(maxpart, (int)h->levels.size() - 1);
    // factorize: per partitioned level, the chain kernels then the assembly; then every coarsest level
    for (int l = 0; l < maxpart; ++l) {
        plan_factor_level<double, double>(B, l, false);
        plan_factor_level<double, float>(B, l, false);
        plan_factor_level<float, float>(B, l, false);
        plan_asm_schur<double, double, double>(B, l);
        plan_asm_schur<double, float, float>(B, l);
        plan_asm_schur<double, float, double>(B, l);
        plan_asm_schur<float, float, float>(B, l);
        plan_asm_schur<float, float, double>(B, l);
    }
    plan_factor_level<double, double>(B, 0, true);
    plan_factor_level<double, float>(B, 0, true);  // mixed systems short enough to have no partitioned level
    plan_factor_level<float, float>(B, 0, true);
    if (!b->mixed) {
        plan_chain_solve(B, maxpart, B.solve);
    } else {
        plan_vec<float>(B, VEC_ABSMAX, B.pro);
        plan_vec<double>(B, VEC_ABSMAX, B.pro);
        plan_vec<float>(B, VEC_TO_CORR, B.pro);
        plan_vec<double>(B, VEC_TO_CORR, B.pro);
        plan_chain_solve(B, maxpart, B.pro);
        plan_vec<float>(B, VEC_SET, B.pro);
        plan_vec<double>(B, VEC_SET, B.pro);
        for (int nb : {16, 32, 64, (int)WIDE_CLASS}) {
            plan_resid<float>(B, nb, B.resid);
            plan_resid<double>(B, nb, B.resid);
        }
        plan_chain_solve(B, maxpart, B.corr);
        plan_vec<float>(B, VEC_ADD, B.corr);
        plan_vec<double>(B, VEC_ADD, B.corr);
        plan_vec<float>(B, VEC_COPY_OUT, B.epi);
        plan_vec<double>(B, VEC_COPY_OUT, B.epi);
    }
    // status pointer array, gather buffer, loop flags
    std::vector<DevStatus *> sts;
    for (bss_handle *h : b->sys) sts.push_back(h->st);
    const size_t osts = put_vec(B.blob, sts);
    const size_t ogather = B.blob.put(nullptr, sizeof(DevStatus) * b->nsys);
    const size_t oany = B.blob.put(nullptr, 16);
    BSS_CUDA(cudaMalloc((void **)&b->meta, B.blob.bytes.size()));
    BSS_CUDA(cudaMemcpy(b->meta, B.blob.bytes.data(), B.blob.bytes.size(), cudaMemcpyHostToDevice));
    b->d_sts = (DevStatus **)(b->meta + osts);
    b->d_gather = (DevStatus *)(b->meta + ogather);
    b->d_any = (int *)(b->meta + oany);
    b->h_gather.assign(b->nsys, DevStatus{});
    auto bind = [&](std::vector<std::function<Step(char *)>> &src, std::vector<Step> &dst) {
        for (auto &f : src) dst.push_back(f(b->meta));
    };
    bind(B.factor, b->factor_steps);
    bind(B.solve, b->solve_steps);
    bind(B.pro, b->pro_steps);
    bind(B.resid, b->resid_steps);
    bind(B.corr, b->corr_steps);
    bind(B.epi, b->epi_steps);
    return BSS_OK;
}

int factor_body(bss_batch *b, cudaStream_t s)
{
    batch_status_kernel<<<grid1d(b->nsys), 128, 0, s>>>(b->d_sts, b->nsys, ST_FACTOR_INIT);
    count_launch();
    BSS_CUDA(cudaGetLastError());
    return run_steps(b->factor_steps, s);
}

int solve_plain_body(bss_batch *b, cudaStream_t s) { return run_steps(b->solve_steps, s); }

// eager mixed solve: host-driven loop (first call)
int solve_mixed_eager(bss_batch *b, cudaStream_t s)
{
    batch_status_kernel<<<grid1d(b->nsys), 128, 0, s>>>(b->d_sts, b->nsys, ST_SOLVE_INIT);
    count_launch();
    BSS_CUDA(cudaGetLastError());
    int rc = run_steps(b->pro_steps, s);
    if (rc) return rc;
    int flags[2] = {0, 0};
    BSS_CUDA(cudaMemsetAsync(b->d_any, 0, 2 * sizeof(int), s));
    for (int it = 0;; ++it) {
        rc = run_steps(b->resid_steps, s);
        if (rc) return rc;
        batch_decide_kernel<<<grid1d(b->nsys), 128, 0, s>>>(b->d_sts, b->nsys, b->opt.tol, b->opt.max_refine, b->d_any);
        count_launch();
        BSS_CUDA(cudaGetLastError());
        BSS_CUDA(cudaMemcpyAsync(flags, b->d_any, sizeof(int), cudaMemcpyDeviceToHost, s));
        BSS_CUDA(cudaStreamSynchronize(s));
        BSS_CUDA(cudaMemsetAsync(b->d_any, 0, sizeof(int), s));
        if (!flags[0] || it >= b->opt.max_refine) break;
        rc = run_steps(b->corr_steps, s);
        if (rc) return rc;
    }
    return run_steps(b->epi_steps, s);
}

// graph mixed solve: WHILE(any) { residual; decide; IF(any) { correction } }
int capture_mixed(bss_batch *b)
{
    cudaStream_t s = b->cap;
    batch_status_kernel<<<grid1d(b->nsys), 128, 0, s>>>(b->d_sts, b->nsys, ST_SOLVE_INIT);
    count_launch();
    BSS_CUDA(cudaGetLastError());
    BSS_CUDA(cudaMemsetAsync(b->d_any, 0, 2 * sizeof(int), s));
    int rc = run_steps(b->pro_steps, s);
    if (rc) return rc;
    cudaStreamCaptureStatus cst;
    cudaGraph_t g = nullptr;
    const cudaGraphNode_t *deps = nullptr;
    size_t nd = 0;
    BSS_CUDA(cudaStreamGetCaptureInfo(s, &cst, nullptr, &g, &deps, nullptr, &nd));
    cudaGraphConditionalHandle hloop, hcorr;
    BSS_CUDA(cudaGraphConditionalHandleCreate(&hloop, g, 1, cudaGraphCondAssignDefault));
    cudaGraphNodeParams wp = {cudaGraphNodeTypeConditional};
    wp.conditional.handle = hloop;
    wp.conditional.type = cudaGraphCondTypeWhile;
    wp.conditional.size = 1;
    cudaGraphNode_t wnode;
    BSS_CUDA(cudaGraphAddNode(&wnode, g, deps, nullptr, nd, &wp));
    cudaGraph_t wbody = wp.conditional.phGraph_out[0];
    BSS_CUDA(cudaStreamUpdateCaptureDependencies(s, &wnode, nullptr, 1, cudaStreamSetCaptureDependencies));
    BSS_CUDA(cudaGraphConditionalHandleCreate(&hcorr, wbody, 0, cudaGraphCondAssignDefault));
    cudaStream_t s2 = b->cap2;
    BSS_CUDA(cudaStreamBeginCaptureToGraph(s2, wbody, nullptr, nullptr, 0, cudaStreamCaptureModeRelaxed));
    const long long kb0 = launch_count();
    rc = run_steps(b->resid_steps, s2);
    if (rc == BSS_OK) {
        batch_decide_kernel<<<grid1d(b->nsys), 128, 0, s2>>>(b->d_sts, b->nsys, b->opt.tol, b->opt.max_refine, b->d_any);
        count_launch();
        batch_set_conditional_kernel<<<1, 32, 0, s2>>>(b->d_any, b->d_any + 1, b->opt.max_refine, hloop, hcorr);
        count_launch();
    }
    b->k_body = launch_count() - kb0;
    cudaGraph_t g2 = nullptr;
    BSS_CUDA(cudaStreamGetCaptureInfo(s2, &cst, nullptr, &g2, &deps, nullptr, &nd));
    cudaGraphNodeParams ip = {cudaGraphNodeTypeConditional};
    ip.conditional.handle = hcorr;
    ip.conditional.type = cudaGraphCondTypeIf;
    ip.conditional.size = 1;
    cudaGraphNode_t inode;
    BSS_CUDA(cudaGraphAddNode(&inode, g2, deps, nullptr, nd, &ip));
    cudaGraph_t ibody = ip.conditional.phGraph_out[0];
    BSS_CUDA(cudaStreamUpdateCaptureDependencies(s2, &inode, nullptr, 1, cudaStreamSetCaptureDependencies));
    cudaGraph_t tmp = nullptr;
    BSS_CUDA(cudaStreamEndCapture(s2, &tmp));
    if (rc) return rc;
    BSS_CUDA(cudaStreamBeginCaptureToGraph(s2, ibody, nullptr, nullptr, 0, cudaStreamCaptureModeRelaxed));
    const long long kc0 = launch_count();
    rc = run_steps(b->corr_steps, s2);
    b->k_corr = launch_count() - kc0;
    count_launches(-(b->k_body + b->k_corr));  // counted per round at synchronize
    BSS_CUDA(cudaStreamEndCapture(s2, &tmp));
    if (rc) return rc;
    return run_steps(b->epi_steps, s);
}

// kernels per replay: counted while capturing, added back per replay (the
// mixed solve's loop body per round at synchronize)
template <class F>
int run_graphed_batch(bss_batch *b, cudaGraphExec_t &exec, int &ncalls, long long &nkern, F eager,
                      std::function<int()> capture)
{
    if (!b->opt.use_graphs || ncalls++ == 0) return eager();
    if (!exec) {
        if (!b->cap) BSS_CUDA(cudaStreamCreateWithFlags(&b->cap, cudaStreamNonBlocking));
        if (!b->cap2) BSS_CUDA(cudaStreamCreateWithFlags(&b->cap2, cudaStreamNonBlocking));
        BSS_CUDA(cudaStreamBeginCapture(b->cap, cudaStreamCaptureModeRelaxed));
        const long long k0 = launch_count();
        const int rc = capture();
        nkern = launch_count() - k0;
        count_launches(-nkern);
        cudaGraph_t g = nullptr;
        const cudaError_t e = cudaStreamEndCapture(b->cap, &g);
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
    }
    BSS_CUDA(cudaGraphLaunch(exec, b->stream));
    count_launches(nkern);
    return BSS_OK;
}

}  // namespace

extern "C" int bss_batch_create(int32_t nsys, const int64_t *N, const int64_t *n, const int64_t *k, int32_t dtype,
                                void *stream, const bss_options *opt, bss_batch **out)
{
    if (!out || nsys < 1 || !N || !n || !k) return fail(BSS_ERR_ARG, "bss_batch_create: bad argument");
    *out = nullptr;
    if (dtype != BSS_F32 && dtype != BSS_F64) return fail(BSS_ERR_ARG, "dtype must be BSS_F32 or BSS_F64");
    bss_batch *b = new bss_batch();
    if (opt)
        b->opt = *opt;
    else
        bss_default_options(&b->opt);
    b->nsys = nsys;
    b->dtype = dtype;
    b->mixed = b->opt.precision == BSS_PRECISION_MIXED;
    b->stream = (cudaStream_t)stream;
    if (b->mixed && dtype != BSS_F64) {
        delete b;
        return fail(BSS_ERR_ARG, "mixed precision needs FP64 tensors");
    }
    cudaError_t e = cudaGetDevice(&b->device);
    if (e != cudaSuccess) {
        delete b;
        return cuda_fail(e, "cudaGetDevice");
    }
    cudaDeviceGetAttribute(&b->sms, cudaDevAttrMultiProcessorCount, b->device);
    size_t bytes = 0;
    int rc = BSS_OK;
    for (int s = 0; s < nsys && rc == BSS_OK; ++s) {
        if (N[s] < 1 || n[s] < 1 || k[s] < 1 || tile_for((int)n[s]) == 0) {
            rc = fail(BSS_ERR_ARG, "system " + std::to_string(s) + ": unsupported N, n or k");
            break;
        }
        bss_handle *h = new bss_handle();
        h->opt = b->opt;
        h->N_user = N[s];
        h->N = N[s];  // batch systems are not padded
        h->n = n[s];
        h->k = k[s];
        h->dtype = dtype;
        h->stream = b->stream;
        h->ls = b->stream;
        h->device = b->device;
        h->seq_api = false;
        h->external_arena = true;
        h->kc_max = solve_kc_max((int)n[s], (int)k[s], dtype == BSS_F64 ? 8 : 4);
        if (h->kc_max < k[s] ||
            (b->mixed && residual_smem_bytes<double>((int)n[s], 1) > (size_t)200 * 1024)) {
            delete h;
            rc = fail(BSS_ERR_UNSUPPORTED,
                      "system " + std::to_string(s) + ": k too large for one solve pass, or n > 128 in mixed precision");
            break;
        }
        // The plan of a system depends only on its own N and the chain length,
        // so its result is the same whichever systems share the batch.
        // Systems shorter than two chains run as one sequential chain (the
        // cheapest schedule; the batch supplies the parallelism).
        const long long chain = batch_chain_blocks(b->opt, (int)n[s], dtype);
        h->opt.plan = BSS_PLAN_AUTO;
        h->opt.coarsest_fp64 = 0;  // the batch's coarsest chains run in the factor dtype
        h->opt.target_partitions = (int)std::max<long long>(1, N[s] / chain);
        if (N[s] < 2 * chain) h->opt.seq_cutoff = (int)std::max<long long>(1, N[s]);
        rc = plan_handle(h);
        h->arena_bytes = (h->arena_bytes + 255) & ~(size_t)255;
        bytes += h->arena_bytes;
        b->sys.push_back(h);
    }
    if (rc == BSS_OK) {
        e = cudaMalloc((void **)&b->arena, bytes);
        if (e != cudaSuccess) rc = cuda_fail(e, "cudaMalloc(batch arena)");
    }
    size_t off = 0;
    for (size_t s = 0; rc == BSS_OK && s < b->sys.size(); ++s) {
        bss_handle *h = b->sys[s];
        h->arena = b->arena + off;
        rc = bind_handle(h, h->arena, false);
        off += h->arena_bytes;
    }
    if (rc == BSS_OK) rc = build_batch(b);
    if (rc != BSS_OK) {
        for (bss_handle *h : b->sys) delete h;
        if (b->arena) cudaFree(b->arena);
        if (b->meta) cudaFree(b->meta);
        delete b;
        return rc;
    }
    *out = b;
    return BSS_OK;
}

extern "C" int bss_batch_destroy(bss_batch *b)
{
    if (!b) return BSS_OK;
    if (b->stream)
        cudaStreamSynchronize(b->stream);
    else
        cudaDeviceSynchronize();
    if (b->g_factor) cudaGraphExecDestroy(b->g_factor);
    if (b->g_solve) cudaGraphExecDestroy(b->g_solve);
    if (b->cap) cudaStreamDestroy(b->cap);
    if (b->cap2) cudaStreamDestroy(b->cap2);
    for (bss_handle *h : b->sys) delete h;
    if (b->arena) cudaFree(b->arena);
    if (b->meta) cudaFree(b->meta);
    delete b;
    return BSS_OK;
}

extern "C" int bss_batch_get_tensors(bss_batch *b, int32_t s, void **A, void **B, void **d)
{
    if (!b || s < 0 || s >= b->nsys) return fail(BSS_ERR_ARG, "bad batch or system index");
    return bss_get_tensors(b->sys[s], A, B, d);
}

extern "C" int bss_batch_get_dims(bss_batch *b, int32_t s, int64_t *N, int64_t *n, int64_t *k)
{
    if (!b || s < 0 || s >= b->nsys) return fail(BSS_ERR_ARG, "bad batch or system index");
    return bss_get_dims(b->sys[s], N, n, k, nullptr);
}

extern "C" int bss_batch_factorize(bss_batch *b)
{
    if (!b) return fail(BSS_ERR_ARG, "batch is NULL");
    const int rc = run_graphed_batch(
        b, b->g_factor, b->n_factor, b->k_factor, [&]() { return factor_body(b, b->stream); },
        [&]() { return factor_body(b, b->cap); });
    if (rc == BSS_OK) b->factored = true;
    return rc;
}

extern "C" int bss_batch_solve(bss_batch *b)
{
    if (!b) return fail(BSS_ERR_ARG, "batch is NULL");
    if (!b->factored) return fail(BSS_ERR_STATE, "solve before factorize");
    int rc;
    const bool graph = b->opt.use_graphs && b->n_solve > 0;
    if (b->mixed)
        rc = run_graphed_batch(
            b, b->g_solve, b->n_solve, b->k_solve, [&]() { return solve_mixed_eager(b, b->stream); },
            [&]() { return capture_mixed(b); });
    else
        rc = run_graphed_batch(
            b, b->g_solve, b->n_solve, b->k_solve, [&]() { return solve_plain_body(b, b->stream); },
            [&]() { return solve_plain_body(b, b->cap); });
    if (rc == BSS_OK) {
        b->solve_pending = true;
        if (graph && b->mixed) ++b->graph_solves_unsynced;
    }
    return rc;
}

extern "C" int bss_batch_synchronize(bss_batch *b)
{
    if (!b) return fail(BSS_ERR_ARG, "batch is NULL");
    BSS_CUDA(cudaStreamSynchronize(b->stream));
    batch_gather_status_kernel<<<grid1d(b->nsys), 128, 0, b->stream>>>(b->d_sts, b->d_gather, b->nsys);
    BSS_CUDA(cudaGetLastError());
    BSS_CUDA(cudaMemcpyAsync(b->h_gather.data(), b->d_gather, sizeof(DevStatus) * b->nsys, cudaMemcpyDeviceToHost,
                             b->stream));
    int rounds = 0;
    BSS_CUDA(cudaMemcpyAsync(&rounds, b->d_any + 1, sizeof(int), cudaMemcpyDeviceToHost, b->stream));
    BSS_CUDA(cudaStreamSynchronize(b->stream));
    if (b->graph_solves_unsynced > 0) {
        // each device-loop solve ran `rounds` loop bodies and rounds-1 corrections
        // (the count of the last solve stands in for earlier unsynchronised ones)
        const long long per = rounds * b->k_body + std::max(rounds - 1, 0) * b->k_corr;
        count_launches(per * b->graph_solves_unsynced);
        b->graph_solves_unsynced = 0;
    }
    int rc = BSS_OK;
    for (int s = 0; s < b->nsys; ++s) {
        const DevStatus &st = b->h_gather[s];
        bss_info &inf = b->sys[s]->info;
        if (b->factored && st.tc_timeout && rc == BSS_OK)
            rc = fail(BSS_ERR_TIMEOUT, "a bounded tensor-core wait expired in system " + std::to_string(s));
        if (b->factored && st.bad_key != ~0ULL) {
            inf.failed_level = (int32_t)(st.bad_key >> 40);
            inf.failed_block = (int64_t)(st.bad_key & ((1ULL << 40) - 1));
            if (rc == BSS_OK) rc = fail(BSS_ERR_NOT_SPD, "pivot failed in system " + std::to_string(s));
        } else {
            inf.failed_level = -1;
            inf.failed_block = -1;
        }
        if (b->mixed && b->solve_pending) {
            inf.refine_steps = st.iters;
            inf.rel_residual = st.relres;
            if (!st.done && rc == BSS_OK)
                rc = fail(BSS_ERR_NOT_CONVERGED, "system " + std::to_string(s) + " missed the tolerance");
        }
    }
    b->solve_pending = false;
    return rc;
}

extern "C" int bss_batch_get_info(bss_batch *b, int32_t s, bss_info *info)
{
    if (!b || !info || s < 0 || s >= b->nsys) return fail(BSS_ERR_ARG, "bad batch or system index");
    *info = b->sys[s]->info;
    return BSS_OK;
}
