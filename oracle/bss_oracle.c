/*
 * CPU oracle: sequential block Cholesky of a block-tridiagonal SPD matrix.
 *
 * TEST INFRASTRUCTURE ONLY.  Used by tests/ to check results and by bench.py as
 * the timed CPU baseline (the reference's own CPU path); never linked into or
 * called by the product library.
 *
 * Restates BlockStructuredSolvers.jl src/backbone_cpu.jl:5-33 (wrapped by
 * src/cpu.jl:30-50):
 *   factorize:  potrf!('U', A_1)
 *               for i = 2..N: trsm!('L','U','T','N', 1, A_{i-1}, B_{i-1})
 *                             gemm!('T','N', -1, B_{i-1}, B_{i-1}, 1, A_i)
 *                             potrf!('U', A_i)
 *   solve:      trsm!('L','U','T','N', 1, A_1, d_1)
 *               for i = 2..N: gemm!('T','N',-1,B_{i-1},d_{i-1},1,d_i); trsm!(LUTN, A_i, d_i)
 *               trsm!('L','U','N','N', 1, A_N, d_N)
 *               for i = N-1..1: gemm!('N','N',-1,B_i,d_{i+1},1,d_i); trsm!(LUNN, A_i, d_i)
 *
 * The reference reaches LAPACK/BLAS through Julia's LinearAlgebra (OpenBLAS).
 * Here the same LAPACK/BLAS routines are reached through function pointers the
 * caller registers (scipy.linalg.cython_lapack / cython_blas export them, so
 * the oracle links OpenBLAS on both x86-64 and aarch64 without a system BLAS).
 * If no pointers are registered, plain C loops implementing the same LAPACK /
 * BLAS semantics are used instead ("port" mode).
 *
 * Storage: Julia column-major blocks.  A is n x n x N (block i at A + i*n*n,
 * lda = n), B is n x n x (N-1), d is n x k x N (block i at d + i*n*k, ld = n).
 */
#include <math.h>
#include <pthread.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

typedef void (*potrf_d_t)(char *, int *, double *, int *, int *);
typedef void (*trsm_d_t)(char *, char *, char *, char *, int *, int *, double *, double *, int *,
                         double *, int *);
typedef void (*gemm_d_t)(char *, char *, int *, int *, int *, double *, double *, int *, double *,
                         int *, double *, double *, int *);
typedef void (*potrf_s_t)(char *, int *, float *, int *, int *);
typedef void (*trsm_s_t)(char *, char *, char *, char *, int *, int *, float *, float *, int *,
                         float *, int *);
typedef void (*gemm_s_t)(char *, char *, int *, int *, int *, float *, float *, int *, float *,
                         int *, float *, float *, int *);

static potrf_d_t g_dpotrf = 0;
static trsm_d_t g_dtrsm = 0;
static gemm_d_t g_dgemm = 0;
static potrf_s_t g_spotrf = 0;
static trsm_s_t g_strsm = 0;
static gemm_s_t g_sgemm = 0;

int bsso_set_blas(void *dpotrf, void *dtrsm, void *dgemm, void *spotrf, void *strsm, void *sgemm)
{
    g_dpotrf = (potrf_d_t)dpotrf;
    g_dtrsm = (trsm_d_t)dtrsm;
    g_dgemm = (gemm_d_t)dgemm;
    g_spotrf = (potrf_s_t)spotrf;
    g_strsm = (trsm_s_t)strsm;
    g_sgemm = (gemm_s_t)sgemm;
    return 0;
}

int bsso_has_blas(void) { return g_dpotrf && g_dtrsm && g_dgemm && g_spotrf && g_strsm && g_sgemm; }

/* ---------------------------------------------------------------------------
 * Plain C loops with the LAPACK/BLAS semantics used above (column-major).
 * ------------------------------------------------------------------------- */
#define DEFINE_PORT(T, SUF, SQRT)                                                                   \
    /* potrf 'U': upper triangle of a replaced by U with U^T U = a. */                              \
    static int port_potrf_##SUF(int n, T *a, int lda)                                               \
    {                                                                                               \
        for (int j = 0; j < n; ++j) {                                                               \
            T s = a[j + (size_t)j * lda];                                                           \
            for (int p = 0; p < j; ++p) s -= a[p + (size_t)j * lda] * a[p + (size_t)j * lda];       \
            if (!(s > 0)) return j + 1;                                                             \
            T ujj = SQRT(s);                                                                        \
            a[j + (size_t)j * lda] = ujj;                                                           \
            for (int c = j + 1; c < n; ++c) {                                                       \
                T t = a[j + (size_t)c * lda];                                                       \
                for (int p = 0; p < j; ++p) t -= a[p + (size_t)j * lda] * a[p + (size_t)c * lda];   \
                a[j + (size_t)c * lda] = t / ujj;                                                   \
            }                                                                                       \
        }                                                                                           \
        return 0;                                                                                   \
    }                                                                                               \
    /* trsm L,U,trans,N: solve op(U) X = b in place (b is n x nrhs). */                             \
    static void port_trsm_##SUF(int trans, int n, int nrhs, const T *a, int lda, T *b, int ldb)     \
    {                                                                                               \
        for (int c = 0; c < nrhs; ++c) {                                                            \
            T *x = b + (size_t)c * ldb;                                                             \
            if (trans) { /* U^T x = b: forward */                                                   \
                for (int i = 0; i < n; ++i) {                                                       \
                    T t = x[i];                                                                     \
                    for (int p = 0; p < i; ++p) t -= a[p + (size_t)i * lda] * x[p];                 \
                    x[i] = t / a[i + (size_t)i * lda];                                              \
                }                                                                                   \
            } else { /* U x = b: backward */                                                        \
                for (int i = n - 1; i >= 0; --i) {                                                  \
                    T t = x[i];                                                                     \
                    for (int p = i + 1; p < n; ++p) t -= a[i + (size_t)p * lda] * x[p];             \
                    x[i] = t / a[i + (size_t)i * lda];                                              \
                }                                                                                   \
            }                                                                                       \
        }                                                                                           \
    }                                                                                               \
    /* c = c - op(a) * b ; op = transpose if ta (a is n x n, b is n x nrhs). */                     \
    static void port_gemm_sub_##SUF(int ta, int n, int nrhs, const T *a, int lda, const T *b,       \
                                    int ldb, T *c, int ldc)                                         \
    {                                                                                               \
        for (int j = 0; j < nrhs; ++j)                                                              \
            for (int i = 0; i < n; ++i) {                                                           \
                T t = 0;                                                                            \
                if (ta)                                                                             \
                    for (int p = 0; p < n; ++p) t += a[p + (size_t)i * lda] * b[p + (size_t)j * ldb]; \
                else                                                                                \
                    for (int p = 0; p < n; ++p) t += a[i + (size_t)p * lda] * b[p + (size_t)j * ldb]; \
                c[i + (size_t)j * ldc] -= t;                                                        \
            }                                                                                       \
    }

DEFINE_PORT(double, d, sqrt)
DEFINE_PORT(float, s, sqrtf)

/* ---------------------------------------------------------------------------
 * backbone_cpu.jl:5-33, one system.
 * ------------------------------------------------------------------------- */
#define DEFINE_CHOL(T, SUF)                                                                         \
    static int potrf_##SUF(int n, T *a)                                                             \
    {                                                                                               \
        if (g_##SUF##potrf) {                                                                       \
            char u = 'U';                                                                           \
            int nn = n, lda = n, info = 0;                                                          \
            g_##SUF##potrf(&u, &nn, a, &lda, &info);                                                \
            return info;                                                                            \
        }                                                                                           \
        return port_potrf_##SUF(n, a, n);                                                           \
    }                                                                                               \
    static void trsm_##SUF(int trans, int n, int nrhs, T *a, T *b)                                  \
    {                                                                                               \
        if (g_##SUF##trsm) {                                                                        \
            char side = 'L', up = 'U', tr = trans ? 'T' : 'N', dg = 'N';                            \
            int mm = n, nn = nrhs, lda = n, ldb = n;                                                \
            T one = 1;                                                                              \
            g_##SUF##trsm(&side, &up, &tr, &dg, &mm, &nn, &one, a, &lda, b, &ldb);                  \
            return;                                                                                 \
        }                                                                                           \
        port_trsm_##SUF(trans, n, nrhs, a, n, b, n);                                                \
    }                                                                                               \
    /* c -= op(a) b, a n x n, b/c n x nrhs */                                                       \
    static void gemm_sub_##SUF(int ta, int n, int nrhs, T *a, T *b, T *c)                           \
    {                                                                                               \
        if (g_##SUF##gemm) {                                                                        \
            char tA = ta ? 'T' : 'N', tB = 'N';                                                     \
            int mm = n, nn = nrhs, kk = n, lda = n, ldb = n, ldc = n;                               \
            T alpha = -1, beta = 1;                                                                 \
            g_##SUF##gemm(&tA, &tB, &mm, &nn, &kk, &alpha, a, &lda, b, &ldb, &beta, c, &ldc);       \
            return;                                                                                 \
        }                                                                                           \
        port_gemm_sub_##SUF(ta, n, nrhs, a, n, b, n, c, n);                                         \
    }                                                                                               \
    /* returns 0, or 1-based index of the first block whose potrf failed */                        \
    int64_t bsso_factorize_##SUF(int64_t N, int n, T *A, T *B)                                      \
    {                                                                                               \
        const size_t nn = (size_t)n * n;                                                            \
        if (N <= 0 || n <= 0) return 0;                                                             \
        if (potrf_##SUF(n, A)) return 1;                                                            \
        for (int64_t i = 1; i < N; ++i) {                                                           \
            trsm_##SUF(1, n, n, A + (i - 1) * nn, B + (i - 1) * nn);                                \
            gemm_sub_##SUF(1, n, n, B + (i - 1) * nn, B + (i - 1) * nn, A + i * nn);                \
            if (potrf_##SUF(n, A + i * nn)) return i + 1;                                           \
        }                                                                                           \
        return 0;                                                                                   \
    }                                                                                               \
    void bsso_solve_##SUF(int64_t N, int n, int k, T *A, T *B, T *d)                                \
    {                                                                                               \
        const size_t nn = (size_t)n * n, nk = (size_t)n * k;                                        \
        if (N <= 0 || n <= 0 || k <= 0) return;                                                     \
        trsm_##SUF(1, n, k, A, d);                                                                  \
        for (int64_t i = 1; i < N; ++i) {                                                           \
            gemm_sub_##SUF(1, n, k, B + (i - 1) * nn, d + (i - 1) * nk, d + i * nk);                \
            trsm_##SUF(1, n, k, A + i * nn, d + i * nk);                                            \
        }                                                                                           \
        trsm_##SUF(0, n, k, A + (N - 1) * nn, d + (N - 1) * nk);                                    \
        for (int64_t i = N - 2; i >= 0; --i) {                                                      \
            gemm_sub_##SUF(0, n, k, B + i * nn, d + (i + 1) * nk, d + i * nk);                      \
            trsm_##SUF(0, n, k, A + i * nn, d + i * nk);                                            \
        }                                                                                           \
    }

DEFINE_CHOL(double, d)
DEFINE_CHOL(float, s)

/* ---------------------------------------------------------------------------
 * Many independent systems (uneven N and n), one worker thread per system
 * at a time.  Each system: factorize + solve in place.  Used as the CPU
 * baseline for batched workloads.  info_out[s] = bsso_factorize result.
 * ------------------------------------------------------------------------- */
typedef struct {
    int nsys;
    const int64_t *N;
    const int *n;
    const int *k;
    double **A;
    double **B;
    double **d;
    int64_t *info;
    int next;
    pthread_mutex_t mu;
} many_job_t;

static void *many_worker(void *arg)
{
    many_job_t *j = (many_job_t *)arg;
    for (;;) {
        pthread_mutex_lock(&j->mu);
        int s = j->next++;
        pthread_mutex_unlock(&j->mu);
        if (s >= j->nsys) break;
        int64_t info = bsso_factorize_d(j->N[s], j->n[s], j->A[s], j->B[s]);
        if (j->info) j->info[s] = info;
        if (!info) bsso_solve_d(j->N[s], j->n[s], j->k[s], j->A[s], j->B[s], j->d[s]);
    }
    return 0;
}

int bsso_solve_many_d(int nsys, const int64_t *N, const int *n, const int *k, double **A,
                      double **B, double **d, int64_t *info, int nthreads)
{
    many_job_t job;
    memset(&job, 0, sizeof(job));
    job.nsys = nsys;
    job.N = N;
    job.n = n;
    job.k = k;
    job.A = A;
    job.B = B;
    job.d = d;
    job.info = info;
    pthread_mutex_init(&job.mu, 0);
    if (nthreads < 1) nthreads = 1;
    if (nthreads > 256) nthreads = 256;
    pthread_t th[256];
    int started = 0;
    for (int t = 0; t < nthreads; ++t)
        if (pthread_create(&th[t], 0, many_worker, &job) == 0) ++started;
    if (!started) many_worker(&job);
    for (int t = 0; t < started; ++t) pthread_join(th[t], 0);
    pthread_mutex_destroy(&job.mu);
    return 0;
}
