/*
 * bss.h -- C ABI of the GB300 (sm_103a) batched block-tridiagonal SPD solver.
 *
 * Drop-in for BlockStructuredSolvers.jl's batched GPU solver.  A Julia caller
 * binds these entry points with `ccall`; Python binds them with ctypes
 * (blockstructuredsolvers_gb300/_lib.py).  No torch or CUDA
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
    int32_t coarsest_fp64;     /* mixed, single-system handles: factor and solve the
                                  sequential coarsest level in FP64 (0 = FP32, the
                                  default; the FP64 refinement corrects the whole
                                  factorization either way).  Batches ignore it. */
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

/* ---- host upload / download --------------------------------------------------
 * Replaces the caller's `copyto!(data.A_tensor, A)`, `copyto!(data.B_tensor,
 * B)`, `copyto!(data.d_tensor, d)` before factorize! (reference
 * benchmark/benchmark_gpu.jl:129-131) from host arrays, and the read of the
 * solution out of d_tensor after solve!.  Host arrays hold the N blocks the handle was
 * created with (not N_use), in the device layout above and the handle's
 * dtype: A n x n x N, B n x n x (N-1), d (and x) n x k x N, column-major.
 * The caller guarantees those sizes.  Asynchronous on the handle's stream
 * when the host memory is page-locked; the padding blocks keep their values.
 *
 * flags BSS_UPLOAD_UPPER: only the upper triangle of each A_i defines the
 * block -- the triangle the reference's potrf(CUBLAS_FILL_MODE_UPPER) reads
 * (src/backbone_cuda.jl:21-33, 77-99) -- it is mirrored into the lower
 * triangle on the device, so the host's lower triangles may hold anything.
 * BSS_UPLOAD_FULL keeps the blocks as copied.  Each tensor is one contiguous
 * copy.  A, B or d may be NULL (that tensor is left as it is).  *host_bytes
 * (may be NULL) receives the bytes read from host memory. */
#define BSS_UPLOAD_FULL 0
#define BSS_UPLOAD_UPPER 1
int bss_upload(bss_handle *h, const void *A, const void *B, const void *d, int32_t flags, int64_t *host_bytes);

/* Copies d_tensor's first N blocks (the solution after bss_solve) into host
 * memory x (n x k x N); asynchronous on the handle's stream: x is complete
 * after bss_synchronize. */
int bss_download(bss_handle *h, void *x);

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
 * is launched, as are N >= 2^40 and k > INT32_MAX.  The first call on a
 * device looks up the array's device address with that device current and
 * keeps it for the life of the process; make that first call before any
 * stream capture, and do not call this entry point on a device after
 * cudaDeviceReset (the kept address belonged to the reset context).  All
 * calls share the one array: calls that overlap on the GPU (other streams,
 * other host threads) race on it, so serialise them.  Blocks until the
 * stream has finished; returns BSS_ERR_NOT_SPD on a failed pivot and
 * BSS_ERR_TIMEOUT when a bounded tensor-core wait of the wide FP32 path
 * (64 < n <= 128) expired (the result is then void). */
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

/* ---- Kalman-smoother blocks built on the device ------------------------------
 * Replaces build_kf_blocks (reference benchmark/benchmark_kf.jl:105-154),
 * which assembles the normal equations of a linear-Gaussian state-space
 * model on the host.  All pointers are DEVICE memory, column-major, FP64:
 *   F (n x n), H (m x n), Qinv (n x n) = Q^{-1}, Rinv (m x m) = R^{-1},
 *   P0inv (n x n) or NULL, x0 (n) or NULL, y (m x k x N): k observation
 *   sequences (the reference has k = 1).
 * Output A (n x n x N), B (n x n x (N-1)), d (n x k x N):
 *   B_i = -F^T Q^{-1};  d_i = H^T R^{-1} y_i  (+ P0^{-1} x0 at i = 0)
 *   with P0inv: A_0 = H^T R^{-1} H + P0^{-1} + F^T Q^{-1} F,
 *               A_{N-1} = H^T R^{-1} H + Q^{-1}, the others
 *               H^T R^{-1} H + Q^{-1} + F^T Q^{-1} F   (the reference's form);
 *   P0inv NULL: every A_i = H^T R^{-1} H + Q^{-1} + F^T Q^{-1} F.
 * A_i is symmetrised from its upper triangle (the reference's
 * Symmetric(Akk)).  Asynchronous on `stream`. */
int bss_kf_build(int64_t N, int64_t n, int64_t m, int64_t k, const double *F, const double *H, const double *Qinv,
                 const double *Rinv, const double *P0inv, const double *x0, const double *y, double *A, double *B,
                 double *d, void *stream);

/* ---- request server: continuous batching under an HBM budget ------------------
 * No counterpart in the reference.  A worker thread owns the GPU work:
 * requests are admitted as streams and memory free up (FIFO on memory; a
 * request larger than the whole budget fails with BSS_ERR_OOM), each runs on
 * one of `streams` CUDA streams so the work of concurrent requests overlaps
 * on the device, and the mixed-precision refinement loop of every request
 * advances on completion events (no host thread blocks on a stream).  Each
 * request's system gets its own plan and workspace, so its result is the
 * same alone and in any mix.  Factors of requests submitted with `keep`
 * stay resident for repeat right-hand sides until released, or until the
 * budget needs their memory (least recently used first; an RHS request on
 * an evicted factor fails with BSS_ERR_STATE, at submit or, if the factor
 * was evicted while the request queued, in its result).
 * Host buffers passed to submit calls (inputs and x_out) must stay valid and
 * unchanged until bss_server_wait returns for that request; page-locked
 * buffers make the copies asynchronous.  All tensors are FP64, column-major
 * as above; x_out receives x (n x k x N). */
typedef struct bss_server bss_server;

typedef struct {
    int64_t hbm_budget_bytes;  /* device memory for all requests (default 100 GB)  */
    int32_t streams;           /* concurrent CUDA streams (default 8)               */
    int32_t max_inflight;      /* requests on the GPU at once (default 64)          */
    int32_t precision;         /* BSS_PRECISION_MIXED (default) or _PLAIN (FP64)    */
    int32_t max_refine;        /* default 10                                        */
    double tol;                /* default 1e-12                                     */
} bss_server_options;

typedef struct {
    int32_t status;        /* BSS_OK, BSS_ERR_NOT_SPD, BSS_ERR_NOT_CONVERGED, ...   */
    int32_t refine_steps;
    double rel_residual;   /* mixed: relative residual of x; -1 in plain precision  */
    double latency_ms;     /* submit -> result in x_out                             */
    double queue_ms;       /* submit -> admitted to the GPU                         */
    uint64_t factor_id;    /* resident factor (0 if none)                           */
} bss_request_info;

typedef struct {
    int64_t submitted, completed, failed, evictions;
    int64_t resident_factors;
    int64_t bytes_in_use, bytes_peak;
    double p50_ms, p99_ms, mean_ms, max_ms;  /* latency over completed requests  */
    double busy_s;                            /* first submit -> last completion  */
} bss_server_stats;

void bss_server_default_options(bss_server_options *opt);
int bss_server_create(const bss_server_options *opt, bss_server **out);
/* Waits for every request, frees all device memory and stops the worker. */
int bss_server_destroy(bss_server *s);
/* A new system (A, B, d host arrays). keep != 0: its factor stays resident;
 * *factor_id names it (also returned in the info). */
int bss_server_submit(bss_server *s, int64_t N, int64_t n, int64_t k, const double *A, const double *B,
                      const double *d, int32_t keep, double *x_out, uint64_t *request_id, uint64_t *factor_id);
/* A new Kalman-smoother system from its model and observations (host
 * arrays, meaning as in bss_kf_build); blocks are built on the device. */
int bss_server_submit_kalman(bss_server *s, int64_t N, int64_t n, int64_t m, int64_t k, const double *F,
                             const double *H, const double *Qinv, const double *Rinv, const double *P0inv,
                             const double *x0, const double *y, int32_t keep, double *x_out, uint64_t *request_id,
                             uint64_t *factor_id);
/* A repeat right-hand side on a resident factor: d (n x k x N) for a
 * system factor, or y (m x k x N) for a Kalman factor (d rebuilt on the
 * device).  Runs after the factor's earlier requests. */
int bss_server_submit_rhs(bss_server *s, uint64_t factor_id, const double *d_or_y, double *x_out,
                          uint64_t *request_id);
/* Blocks until the request finished; fills *info (may be NULL); returns its
 * status.  A request id can be waited on once. */
int bss_server_wait(bss_server *s, uint64_t request_id, bss_request_info *info);
/* *done = 1 when the request finished (does not consume it). */
int bss_server_poll(bss_server *s, uint64_t request_id, int32_t *done);
/* Drops a resident factor (after its pending requests). */
int bss_server_release(bss_server *s, uint64_t factor_id);
int bss_server_get_stats(bss_server *s, bss_server_stats *stats);
/* Clears the latency record and counters (not the resident factors). */
int bss_server_reset_stats(bss_server *s);

/* ---- CPU block Cholesky (host memory) ---------------------------------------
 * Replaces initialize_cpu / factorize! / solve! of BlockTriDiagData_cpu
 * (reference src/cpu.jl:12-50 over src/backbone_cpu.jl:5-33) with host C++:
 * the sequential block recursion potrf('U') / trsm('L','U','T','N') /
 * gemm('T','N') and its two sweeps.  Tensors are HOST memory in the same
 * column-major layouts (A n x n x N, B n x n x (N-1), d n x k x N), zeroed
 * at creation.  factorize leaves U_i in A_i's upper triangle and
 * U_i^{-T} B_i in B_i, like the reference; a non-positive pivot returns
 * BSS_ERR_NOT_SPD (the reference ignores potrf's info) and
 * bss_cpu_failed_block names the block.  No GPU is used. */
typedef struct bss_cpu_handle bss_cpu_handle;
int bss_cpu_create(int64_t N, int64_t n, int64_t k, int32_t dtype, bss_cpu_handle **out);
int bss_cpu_destroy(bss_cpu_handle *h);
int bss_cpu_get_tensors(bss_cpu_handle *h, void **A, void **B, void **d);
int bss_cpu_factorize(bss_cpu_handle *h);
int bss_cpu_solve(bss_cpu_handle *h);
int bss_cpu_failed_block(bss_cpu_handle *h, int64_t *block);

/* ---- plan autotuner per (n, dtype, precision) ------------------------------
 * No counterpart in the reference.  Tile shapes and CTA sizes are fixed per
 * block-size class; the tuner picks the plan: finest-level partitions as a
 * multiple of one wave of resident chain CTAs (wave_mult_x4 / 4), the
 * sequential cutoff, and the batch chain length, by timing factorize+solve
 * of a device-generated SPD system of N_probe blocks (0: 16384) and of a
 * batch of 256 systems of 512 blocks.  Results go to a process-wide table
 * that the planners consult whenever the caller leaves target_partitions,
 * seq_cutoff or chain_blocks at 0 (so tuning changes the partitioning, and
 * with it the rounding, of later handles).  Blocks while it runs (seconds). */
typedef struct {
    int32_t n, dtype, precision;
    int32_t wave_mult_x4;   /* finest-level partitions = waves x 4 / 4 */
    int32_t seq_cutoff;
    int32_t chain_blocks;
    double single_ms;       /* best factorize+solve time of the probe system */
    double batch_ms;        /* best factorize+solve time of the probe batch  */
    int32_t factor_variant; /* BSS_FACTOR_* bits of the chain kernel          */
} bss_tune_entry;

int bss_autotune(int64_t n, int32_t dtype, int32_t precision, int64_t N_probe, bss_tune_entry *out);
int bss_autotune_lookup(int64_t n, int32_t dtype, int32_t precision, bss_tune_entry *out);
void bss_autotune_clear(void);
/* text cache: one line per entry (n dtype precision wave_mult_x4 seq_cutoff
 * chain_blocks single_ms batch_ms) */
int bss_autotune_save(const char *path);
int bss_autotune_load(const char *path);

/* ---- the reference's algorithm on this GPU (comparison) ---------------------
 * A restatement of factorize!/solve! of BlockTriDiagData_batched
 * (src/gpu_batched.jl:184-258) over the same batched cuSOLVER/cuBLAS calls
 * (potrfBatched, trsmBatched, gemmBatched; src/backbone_cuda.jl:14-184), the
 * same n x 2n fill F = T^{-1} G and M_2n Schur products, the reference
 * planner's padded size and levels, and a sequential coarsest level.  For
 * timing the reference's own GPU algorithm beside this library's kernels;
 * it is not a path of bss_create_batched.  Tensors (device, column-major,
 * N_use blocks, identity padding) as for bss_create_batched; factorize
 * leaves the reference's factors in A/B; solve overwrites d.  Asynchronous
 * on `stream`; pivot failures are not checked (as in the reference). */
typedef struct bss_refalgo bss_refalgo;
int bss_refalgo_create(int64_t N, int64_t n, int64_t k, int32_t dtype, void *stream, bss_refalgo **out);
int bss_refalgo_destroy(bss_refalgo *h);
int bss_refalgo_get_tensors(bss_refalgo *h, void **A, void **B, void **d);
int bss_refalgo_get_dims(bss_refalgo *h, int64_t *N, int64_t *n, int64_t *k);
int bss_refalgo_factorize(bss_refalgo *h);
int bss_refalgo_solve(bss_refalgo *h);

/* ---- sparse assembly and a general sparse Cholesky (comparison) ------------
 * bss_csr_assemble replaces construct_block_tridiagonal
 * (benchmark/utils.jl:59-103): from N column-major n x n blocks A (device)
 * and N-1 blocks B it writes the (N n) x (N n) matrix with A_i on the
 * diagonal, B_i at block (i, i+1) and B_i^T at block (i+1, i) as CSR --
 * 0-based int32 row_ptr (N n + 1) and col_idx (nnz), column indices ascending
 * in every row, every entry of every block stored (explicit zeros kept, as
 * the reference's sparse(I, J, V) keeps them), values copied bit for bit.
 * nnz = bss_csr_nnz(N, n) = n^2 (3N - 2) must be below 2^31.  Asynchronous
 * on `stream`.
 *
 * bss_spchol_* replaces the reference's sparse direct-solver comparison
 * (benchmark/benchmark_gpu.jl:75-117: analysis, factorization, solve of the
 * assembled SPD matrix with cuDSS).  cuDSS is not in this toolkit; the
 * phases run on cuSOLVER's GPU sparse Cholesky (csrcholAnalysis,
 * csrcholFactor, csrcholSolve) over the bss_csr_assemble matrix.  Tensors
 * as for bss_create_batched without padding (A n x n x N, B n x n x (N-1),
 * d n x k x N, column-major, device); analyze assembles the CSR matrix and
 * runs the symbolic phase (again: refreshes the values only); factorize
 * re-assembles the values (analyzing first if needed) and factors, returning
 * BSS_ERR_NOT_SPD on a non-positive pivot; solve overwrites d with the
 * solution and returns BSS_ERR_STATE unless a factorization succeeded since
 * the last analyze.  The library phases synchronise the stream. */
int64_t bss_csr_nnz(int64_t N, int64_t n);
int bss_csr_assemble(int64_t N, int64_t n, int32_t dtype, const void *A, const void *B, int32_t *row_ptr,
                     int32_t *col_idx, void *vals, void *stream);
typedef struct bss_spchol bss_spchol;
int bss_spchol_create(int64_t N, int64_t n, int64_t k, int32_t dtype, void *stream, bss_spchol **out);
int bss_spchol_destroy(bss_spchol *h);
int bss_spchol_get_tensors(bss_spchol *h, void **A, void **B, void **d);
int bss_spchol_get_csr(bss_spchol *h, int32_t **row_ptr, int32_t **col_idx, void **vals, int64_t *nnz);
int bss_spchol_get_dims(bss_spchol *h, int64_t *N, int64_t *n, int64_t *k);
int bss_spchol_analyze(bss_spchol *h);
int bss_spchol_factorize(bss_spchol *h);
int bss_spchol_solve(bss_spchol *h);

/* Diagnostic (no counterpart in the reference): one tensor-core product
 * C = X^T Y of n x n FP32 blocks (n <= 128) through the wide kernel's
 * tcgen05 3xTF32 path, compared with an FP64 product of the same inputs;
 * *max_rel_err = max |C - C64| / max |C64|.  Allocates and synchronises. */
int bss_tc_selftest(int64_t n, double *max_rel_err);

/* Diagnostic (no counterpart in the reference): the planner's occupancy
 * query for the tensor-core wide kernel.  out[0..5]: the CUDA error codes of
 * the two attribute calls and of the query, blocks per SM, registers per
 * thread, dynamic shared memory bytes. */
int bss_diag_wide_occupancy(int64_t *out);

/* Diagnostic (no counterpart in the reference): r = d - T x of an FP64
 * system (A, B, x, d, r device, column-major n x n / n x k blocks) by the
 * exact FP64 residual kernel (method 0) or by the double-float kernel on
 * the FP32 pipe that the mixed-precision refinement uses (method 1).
 * Synchronises `stream`. */
int bss_diag_residual(int64_t N, int64_t n, int64_t k, int32_t method, const double *A, const double *B,
                      const double *x, const double *d, double *r, void *stream);

/* Diagnostic (no counterpart in the reference): the bounded mbarrier wait of
 * the tensor-core kernels, run on a barrier that nothing arrives on with at
 * most `polls` (1 .. 2^18) polls.  *timed_out = 1 when the wait gave up (as
 * it must), *cycles = the SM clock cycles it took.  Synchronises. */
int bss_diag_wait_timeout(int64_t polls, int64_t *timed_out, int64_t *cycles);

/* Diagnostic (no counterpart in the reference): the FMA-pipe peak of the
 * current GPU in TFLOP/s for BSS_F32 or BSS_F64 (one FMA = 2 flops), measured
 * by a kernel of independent FMA chains on every SM (best of three timed
 * launches, CUDA events).  The benchmark's roofline fractions use it as the
 * compute peak of the FP32 and FP64 paths.  Synchronises the device. */
int bss_diag_fma_peak(int32_t dtype, double *tflops);

/* Kernel variants of the chain factorization (bits; no counterpart in the
 * reference).  BSS_FACTOR_FMA_CHAIN: partitioned levels of 33 <= n <= 64
 * blocks with FP32 factors (plain FP32, and every level of the mixed path)
 * run on the CUDA-core chain kernel instead of the tensor-core one (tcgen05
 * 3xTF32 products, bulk-copied block tiles).  A handle takes the autotuner's
 * variant for its (n, dtype, precision) when there is one, else the
 * process-wide default set here (0 at start).  Applies to handles and
 * batches created after the call.  BSS_FACTOR_WIDE_L2: partitioned levels
 * of 65 <= n <= 128 blocks with FP32 factors run on the wide kernel whose
 * tensor-core operands are re-staged from L2 per product (two CTAs per SM)
 * instead of the kernel that keeps a chain step on chip (one CTA per SM,
 * factors carried in shared and tensor memory between steps). */
#define BSS_FACTOR_FMA_CHAIN 1
#define BSS_FACTOR_WIDE_L2 2
int bss_diag_set_factor_variant(int32_t variant);
int32_t bss_diag_get_factor_variant(void);

/* Number of CUDA kernels this library has launched in this process, over
 * all handles (no counterpart in the reference; benchmarks report it). */
int64_t bss_kernel_launches(void);

/* Library build string (kernels compiled, arch). */
const char *bss_version(void);

#ifdef __cplusplus
}
#endif
#endif /* BSS_H_ */
