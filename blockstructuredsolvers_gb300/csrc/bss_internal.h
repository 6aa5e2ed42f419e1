// Internal host-side structures shared by the single-system handle
// (bss_api.cu) and the many-system batch (bss_batch.cu).  Not public ABI.
#pragma once

#include <cuda_runtime.h>

#include <string>
#include <vector>

#include "../../include/bss.h"
#include "bss_launch.h"

#define BSS_CUDA(call)                                       \
    do {                                                     \
        cudaError_t e__ = (call);                            \
        if (e__ != cudaSuccess) return cuda_fail(e__, #call); \
    } while (0)

namespace bss {

enum Ty { F32 = 0, F64 = 1 };

inline size_t tsize(int t) { return t == F64 ? 8 : 4; }

// one level of the recursion (finest = 0; the last one is the sequential
// coarsest level)
struct Level {
    long long N = 0;
    long long Q = 0;  // partitions (0 for the sequential level)
    bool seq = false;
    int tin = F64;    // dtype of A/B as read by the factor kernel
    int t = F64;      // dtype of factors, workspace and RHS at this level
    void *A = nullptr, *B = nullptr;    // level system (input)
    void *Af = nullptr, *Bf = nullptr;  // factor storage (== A/B when in place)
    void *d = nullptr;                  // level RHS (t), n x k per block
    void *Y = nullptr, *C = nullptr, *bvec = nullptr;
};


// byte offsets of every buffer of a handle inside its arena
struct Layout {
    size_t A = 0, B = 0, d = 0, c0 = 0, x = 0, st = 0;
    std::vector<size_t> lA, lB, ld, lAf, lBf, lY, lC, lb;
};

}  // namespace bss

struct bss_handle {
    bss::Layout layout;
    bool external_arena = false;  // arena owned by a bss_batch
    long long N_user = 0, N = 0, n = 0, k = 0;
    int dtype = bss::F64;
    bss_options opt{};
    bool seq_api = false;
    cudaStream_t stream = nullptr;
    int device = 0;
    char *arena = nullptr;
    size_t arena_bytes = 0;
    void *A = nullptr, *B = nullptr, *d = nullptr;  // user-visible tensors
    std::vector<bss::Level> levels;
    // mixed precision workspace
    void *c0 = nullptr;     // level-0 correction RHS (levels[0].t)
    double *x64 = nullptr;  // FP64 solution accumulator
    bss::DevStatus *st = nullptr;
    bss::DevStatus *h_st = nullptr;  // pinned mirror
    bool factored = false;
    bool need_anorm = false;  // the next residual also computes ||T||_inf
    int kc_max = 1;
    int variant = 0;  // FACTOR_* kernel variant bits of this handle's factorization
    bss_info info{};
    int sticky = BSS_OK;
    // CUDA graphs: the first call of each kind runs eagerly on `stream`; later
    // calls replay a graph captured on cap_stream and launched on `stream`
    cudaStream_t ls = nullptr;          // stream the launch code enqueues on
    cudaStream_t cap_stream = nullptr;  // private capture streams
    cudaStream_t cap_stream2 = nullptr;
    cudaGraphExec_t g_factor = nullptr, g_solve = nullptr;
    int n_factor = 0, n_solve = 0;
    // kernels per replay (captured launches); mixed solve: prologue, loop
    // body (residual + decision) and correction, combined at synchronize
    long long k_factor = 0, k_solve = 0, k_pro = 0, k_body = 0, k_corr = 0;
    long long graph_solves_unsynced = 0;        // device-loop solves launched since the last sync
    unsigned long long iters_total_seen = 0;    // st->iters_total at the last sync
    bool graph_solve_pending = false;   // a graph solve ran: read its outcome at synchronize
};

namespace bss {

int cuda_fail(cudaError_t e, const char *what);
int fail(int code, const std::string &msg);
// plan levels + layout (sets h->levels, h->layout, h->arena_bytes); no allocation
int plan_handle(bss_handle *h);
// bind the planned layout to memory at `base`, zero it and set the identity padding
int bind_handle(bss_handle *h, char *base, bool alloc_host_status);
template <class Tin, class T>
ChainFactorArgs<Tin, T> make_factor_args(bss_handle *h, int l);
template <class T>
SolveArgs<T> make_solve_args(bss_handle *h, int l, int j0, int kc);

// tuned plan for (n, dtype, precision), if the autotuner has one
bool tuned_plan(int n, int dtype, int precision, bss_tune_entry *out);

// asynchronous pieces of the mixed-precision solve (enqueue on h->ls; each
// of begin/correct ends with the status copied to the pinned h->h_st)
int mixed_begin(bss_handle *h);
int mixed_correct(bss_handle *h);
int mixed_finish(bss_handle *h);

}  // namespace bss
