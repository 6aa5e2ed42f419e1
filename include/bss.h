/*
 * bss.h -- C ABI of the GB300 (sm_103a) batched block-tridiagonal SPD solver.
 *
 * Drop-in for BlockStructuredSolvers.jl's batched GPU solver.  A Julia caller
 * binds these entry points with `ccall`; Python binds
 * them with ctypes (blockstructuredsolvers_gb300/_lib.py).  No torch or CUDA
 * C++ types appear in the signatures: streams are passed as `void*`
 * (a cudaStream_t), device buffers as `void*`.
 *
 * Matrix convention (reference test/utils.jl:32-74): the system matrix has
 * diagonal blocks A_i (n x n, SPD), super-diagonal blocks B_i (block (i,i+1))
 * and sub-diagonal blocks B_i^T.  All device tensors are Julia column-major:
 *   A_tensor  n x n x N      (block i at A + i*n*n, leading dimension n)
 *   B_tensor  n x n x (N-1)
 *   d_tensor  n x k x N      (block i at d + i*n*k, leading dimension n)
 *
 * Threading: a handle is used by one host thread at a time.  Every call that
 * launches work is asynchronous on the handle's stream; bss_synchronize()
 * waits and returns the sticky device status.
 */
#ifndef BSS_H_
#define BSS_H_

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes ------------------------------------------------------- */
#define BSS_OK 0
#define BSS_ERR_ARG 1            /* invalid argument / size                     */
#define BSS_ERR_OOM 2            /* device allocation failed                    */
#define BSS_ERR_CUDA 3           /* a CUDA runtime call failed                  */
#define BSS_ERR_NOT_SPD 4        /* a pivot was <= 0 or not finite              */
#define BSS_ERR_TIMEOUT 5        /* a bounded device wait gave up               */
#define BSS_ERR_UNSUPPORTED 6    /* block size / dtype combination not built    */
#define BSS_ERR_STATE 7          /* solve before factorize, etc.                */
#define BSS_ERR_NOT_CONVERGED 8  /* refinement stopped above its tolerance      */

/* ---- enums ---------------------------------------------------------------- */
#define BSS_F32 0
#define BSS_F64 1

#define BSS_PRECISION_PLAIN 0 /* factor and solve in the tensor dtype            */
#define BSS_PRECISION_MIXED 1 /* FP64 tensors; FP32 factor + FP64 refinement     */

#define BSS_PLAN_AUTO 0      /* partition count sized to the GPU                 */
#define BSS_PLAN_REFERENCE 1 /* the reference planner's (N, m, P) per level      */

typedef struct bss_handle bss_handle;

typedef struct {
    int32_t precision;         /* BSS_PRECISION_*                                  */
    int32_t plan;              /* BSS_PLAN_*                                       */
    int32_t max_refine;        /* mixed: cap on refinement steps (default 10)      */
    int32_t target_partitions; /* auto plan: partitions at the finest level (0 = auto) */
    int32_t seq_cutoff;        /* auto plan: coarsest level size (0 = auto)        */
    int32_t use_graphs;        /* capture factorize/solve into CUDA graphs (1)     */
    double tol;                /* mixed: target relative residual (default 1e-12)  */
    int32_t chain_blocks;      /* batch: blocks per partition at the finest level of
                                  every system (0 = auto per n and precision); a
                                  system's plan depends only on its own N, n and
                                  this value, never on the other systems        */
} bss_options;

typedef struct {
    int64_t failed_block;  /* -1, or the 0-based block index (finest numbering when
                              level == 0) whose pivot failed                          */
    int32_t failed_level;  /* recursion level of the failure (0 = finest)            */
    int32_t refine_steps;  /* mixed: refinement steps taken by the last solve        */
    double rel_residual;   /* mixed: ||d - A x||_inf / (||A||_inf ||x||_inf + ||d||_inf)
                              after the last solve; -1 when not computed              */
    int32_t levels;        /* number of partitioned levels (excl. coarsest)          */
    int64_t coarsest_blocks;
} bss_info;

/* Fill `opt` with the defaults listed above. */
void bss_default_options(bss_options *opt);

/* Replaces initialize_batched(N, n, T, CuArray)
 *   (reference src/gpu_batched.jl:165-182).
 * Allocates library-owned device memory on the current device: A_tensor
 * (n x n x N_use), B_tensor (n x n x (N_use-1)) and d_tensor (n x k x N_use),
 * where N_use >= N is the reference planner's padded size
 * (find_sequence_upper, gpu_batched.jl:155-162).  Padding blocks
 * (indices N-1 .. N_use-1, 0-based) of A are identity, B and d are zero,
 * as gpu_batched.jl:177-179 leaves them.  k >= 1 right-hand sides (the
 * reference batched path has k = 1).  `opt` may be NULL (defaults). */
int bss_create_batched(int64_t N, int64_t n, int64_t k, int32_t dtype, void *stream,
                       const bss_options *opt, bss_handle **out);

/* Replaces initialize_seq(N, n, T, CuArray) (reference src/gpu_seq.jl:45-59):
 * the sequential block Cholesky solver (no partitioning, no padding). */
int bss_create_seq(int64_t N, int64_t n, int64_t k, int32_t dtype, void *stream,
                   bss_handle **out);

/* Frees all device memory of the handle (Julia's finalizer calls this). */
int bss_destroy(bss_handle *h);

/* Device pointers of the handle-owned tensors (valid until bss_destroy):
 * the `A_tensor`, `B_tensor`, `d_tensor` fields of BlockTriDiagData_batched
 * (gpu_batched.jl:1-71) / BlockTriDiagData_seq (gpu_seq.jl:1-27). */
int bss_get_tensors(bss_handle *h, void **A, void **B, void **d);

/* N_use (the `N` field), n, k and dtype of the handle. */
int bss_get_dims(bss_handle *h, int64_t *N, int64_t *n, int64_t *k, int32_t *dtype);

/* Replaces factorize!(data) (gpu_batched.jl:184-227, gpu_seq.jl:61-71).
 * Asynchronous.  Plain precision factors in place like the reference (A and
 * B hold factors afterwards, so it is not idempotent).  Mixed precision keeps
 * A/B unchanged and stores FP32 factors in handle workspace. */
int bss_factorize(bss_handle *h);

/* Replaces solve!(data) (gpu_batched.jl:229-258, gpu_seq.jl:73-84).
 * Asynchronous; overwrites d_tensor with the solution.  Valid repeatedly
 * after one factorize.  Mixed precision: FP64 iterative refinement to
 * opt.tol (host waits on one scalar per refinement step). */
int bss_solve(bss_handle *h);

/* Wait for the handle's stream; returns BSS_ERR_NOT_SPD if a pivot failed
 * in the last factorize, BSS_ERR_NOT_CONVERGED if refinement missed its
 * tolerance, else BSS_OK (or the CUDA error). */
int bss_synchronize(bss_handle *h);

/* Details after bss_synchronize. */
int bss_get_info(bss_handle *h, bss_info *info);

/* Message of the last error returned on this host thread. */
const char *bss_last_error_string(void);

/* The reference level planner (find_sequence_upper/_build_sequence,
 * gpu_batched.jl:112-162).  Writes finest-first triples (N_l, m_l, P_l) into
 * levels[3*l .. 3*l+2] for l < *nlev (at most maxlev) and the coarsest
 * sequential size into *coarsest.  N_use = levels[0]. */
int bss_plan_reference(int64_t N, int64_t *levels, int32_t maxlev, int32_t *nlev,
                       int64_t *coarsest);

/* Relative residual ||d - T x||_inf / (||T||_inf ||x||_inf + ||d||_inf) of a
 * block-tridiagonal system held in caller device buffers (same layouts),
 * computed on the device: d - T x in FP64; ||T||_inf accumulated in FP32
 * from FP64 magnitudes (relative accuracy ~1e-6, which only scales the
 * ratio).  Blocks on `stream`; result in *out. */
int bss_residual(int64_t N, int64_t n, int64_t k, int32_t dtype, const void *A, const void *B,
                 const void *x, const void *d, void *stream, double *out);

/* Inspection (no counterpart in the reference; used by the parity tests to
 * compare intermediate separator systems with the reference's
 * NextData.A_tensor / B_tensor after factorize!, gpu_batched.jl:223-224).
 * bss_factorize_levels runs factorize for the first `nlevels` partitioned
 * levels only, leaving level `nlevels`'s separator system assembled and
 * unfactored.  bss_get_level returns a level's block count, partition count
 * (0 for the sequential coarsest level), device pointers and dtype; level 0
 * is the finest (its A/B are the user tensors). */
int bss_factorize_levels(bss_handle *h, int32_t nlevels);
int bss_get_level(bss_handle *h, int32_t level, int64_t *N, int64_t *Q, void **A, void **B, void **d,
                  int32_t *dtype);

/* ---- factorize + solve without any device allocation ------------------------
 * No counterpart in the reference.  For callers that cannot allocate device
 * memory: hosts whose memory manager owns the whole device pool (a Julia or
 * MATLAB process that hands out only its own buffers, a serving process
 * with a fixed memory budget, code running where cudaMalloc is forbidden).
 * Factors and solves one system in place on CALLER-OWNED device buffers A
 * (n x n x N), B (n x n x (N-1)) and d (n x k x N), in the dtype's own
 * precision (like factorize! followed by solve!: A and B hold factors and d
 * holds x afterwards).  The recursion workspace lives in one file-scope
 * `static __device__` array of BSS_NOALLOC_SCRATCH_BYTES bytes that every GPU
 * loading this library reserves until the process exits; this call performs
 * no cudaMalloc/cudaFree and calls no allocating library routine.  A problem
 * whose workspace does not fit is rejected with BSS_ERR_ARG before any work
 * is launched.  The first call on a device looks up the array's device
 * address with that device current; make that first call before any stream
 * capture.  All calls share the one array: calls that overlap on the GPU
 * (other streams, other host threads) race on it, so serialise them.
 * Blocks until the stream has finished; returns BSS_ERR_NOT_SPD on a failed
 * pivot. */
#define BSS_NOALLOC_SCRATCH_BYTES (8u << 20)
int bss_factor_solve_noalloc(int64_t N, int64_t n, int64_t k, int32_t dtype, void *A, void *B, void *d,
                             void *stream);

/* ---- many independent systems in one batch --------------------------------
 * No counterpart in the reference (its batching is over the partitions of
 * ONE system, src/gpu_batched.jl:184-258).  nsys systems of their own N[s],
 * n[s] (<= 64) and k[s] share one device arena; each recursion level of all
 * systems runs as one persistent launch per block-size class whose CTAs pull
 * (system, partition) items from a device work queue, longest chains first.
 * Systems are not padded (tensors hold exactly N[s] blocks).  Tensors per
 * system come from bss_batch_get_tensors (same layout as a handle's).  With
 * opt->precision = BSS_PRECISION_MIXED (FP64 tensors) every system is
 * refined to opt->tol; the refinement loop runs until all systems converge
 * or max_refine.  factorize/solve are asynchronous on `stream` and replay
 * CUDA graphs after their first call when opt->use_graphs.
 * bss_batch_synchronize waits and returns BSS_ERR_NOT_SPD (first failing
 * system) or BSS_ERR_NOT_CONVERGED; bss_batch_get_info gives each system's
 * outcome. */
typedef struct bss_batch bss_batch;
int bss_batch_create(int32_t nsys, const int64_t *N, const int64_t *n, const int64_t *k, int32_t dtype,
                     void *stream, const bss_options *opt, bss_batch **out);
int bss_batch_destroy(bss_batch *b);
int bss_batch_get_tensors(bss_batch *b, int32_t sys, void **A, void **B, void **d);
int bss_batch_get_dims(bss_batch *b, int32_t sys, int64_t *N, int64_t *n, int64_t *k);
int bss_batch_factorize(bss_batch *b);
int bss_batch_solve(bss_batch *b);
int bss_batch_synchronize(bss_batch *b);
int bss_batch_get_info(bss_batch *b, int32_t sys, bss_info *info);

/* Number of CUDA kernels this library has launched in this process, over
 * all handles (no counterpart in the reference; benchmarks report it). */
int64_t bss_kernel_launches(void);

/* Library build string (kernels compiled, arch). */
const char *bss_version(void);

#ifdef __cplusplus
}
#endif
#endif /* BSS_H_ */
