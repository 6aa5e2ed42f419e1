// Sparse assembly of the block-tridiagonal matrix and a general-purpose
// sparse Cholesky on this GPU, for comparison -- the reference's sparse
// harness: construct_block_tridiagonal (benchmark/utils.jl:59-103) builds
// the (N n) x (N n) matrix with A_i on the diagonal, B_i at block (i, i+1)
// and B_i^T at block (i+1, i), every entry of every block stored; the
// reference then times a sparse direct solver on it in three phases --
// analysis, factorization, solve (benchmark/benchmark_gpu.jl:75-117, cuDSS
// with an "SPD" view).  cuDSS is not part of this toolkit; the stand-in is
// the GPU sparse Cholesky of cuSOLVER (csrcholAnalysis / csrcholFactor /
// csrcholSolve), which has the same three phases, called as a library.
//
// CSR layout (0-based, int32, column indices ascending in every row):
// row R = i n + r of block-row i has length L_i = n (1 + [i > 0] + [i < N-1])
// and holds, in order, B_{i-1}(:, r)^T (columns (i-1) n ..), A_i(r, :)
// (columns i n ..) and B_i(r, :) (columns (i+1) n ..); block-row i starts at
// n^2 (3 i - 1) for i > 0 (0 for i = 0), row r of it at that + r L_i.
// Assembly is a copy: the stored values are the input bits.
#define DISABLE_CUSOLVER_DEPRECATED
#include <cuda_runtime.h>
#include <cusolverSp.h>
#include <cusolverSp_LOWLEVEL_PREVIEW.h>
#include <cusparse.h>

#include <algorithm>
#include <string>
#include <type_traits>
#include <vector>

#include "bss_internal.h"

using namespace bss;

namespace {

constexpr int CSR_TR = 64;    // tile rows of the assembly kernel
constexpr int CSR_TC = 32;    // tile columns (one warp across)
constexpr int CSR_ROWS = 8;   // warps per CTA (32 x 8 threads)

__host__ __device__ inline long long csr_block_row_start(long long i, long long n)
{
    return i == 0 ? 0 : n * n * (3 * i - 1);
}

__host__ __device__ inline long long csr_row_len(long long i, long long N, long long n)
{
    return n * (1 + (i > 0 ? 1 : 0) + (i < N - 1 ? 1 : 0));
}

long long csr_nnz(long long N, long long n) { return n * n * (N + 2 * (N - 1)); }

// row pointers: one thread per row, plus the closing nnz
__global__ void csr_rowptr_kernel(long long N, int n, int *row_ptr)
{
    const long long rows = N * n;
    for (long long R = blockIdx.x * (long long)blockDim.x + threadIdx.x; R <= rows;
         R += (long long)gridDim.x * blockDim.x) {
        if (R == rows) {
            row_ptr[R] = (int)((long long)n * n * (N + 2 * (N - 1)));
        } else {
            const long long i = R / n, r = R - i * n;
            row_ptr[R] = (int)(csr_block_row_start(i, n) + r * csr_row_len(i, N, n));
        }
    }
}

// One CTA per 64-row x 32-column tile of one source block: grid = N x 3
// parts x ceil(n/64) x ceil(n/32) tiles, parts 0 = B_{i-1}^T, 1 = A_i, 2 = B_i.
// Every thread issues its 8 loads before its first store (8 elements in
// flight per thread).  Values are written row by row (coalesced along the
// CSR row); the column-major A_i / B_i tiles pass through shared memory,
// while B_{i-1}^T is already row-contiguous in column-major B_{i-1} and is
// copied directly.
template <class T>
__global__ void __launch_bounds__(CSR_TC *CSR_ROWS)
    csr_values_kernel(long long N, int n, const T *__restrict__ A, const T *__restrict__ B, int *__restrict__ col,
                      T *__restrict__ val, int write_idx)
{
    constexpr int PER = CSR_TR / CSR_ROWS;  // elements per thread
    __shared__ T tile[CSR_TC][CSR_TR + 1];
    const int tnr = (n + CSR_TR - 1) / CSR_TR, tnc = (n + CSR_TC - 1) / CSR_TC;
    long long t = blockIdx.x;
    const int tc = (int)(t % tnc);
    t /= tnc;
    const int tr = (int)(t % tnr);
    t /= tnr;
    const int part = (int)(t % 3);
    const long long i = t / 3;
    if (i >= N || (part == 0 && i == 0) || (part == 2 && i == N - 1)) return;
    const long long nn = (long long)n * n;
    const T *S = part == 1 ? A + i * nn : B + (part == 0 ? i - 1 : i) * nn;
    const long long L = csr_row_len(i, N, n);
    const long long start = csr_block_row_start(i, n);
    const long long pofs = part == 0 ? 0 : (part == 1 ? (i > 0 ? n : 0) : (i > 0 ? 2 * n : n));
    const long long cbase = (i + part - 1) * n;
    const int tx = threadIdx.x % CSR_TC, ty = threadIdx.x / CSR_TC;
    const int r0 = tr * CSR_TR, c0 = tc * CSR_TC;
    if (part == 0) {
        // value (r, c) = B_{i-1}(c, r) = S[c + r n]: contiguous in c
        T v[PER];
        const int c = c0 + tx;
#pragma unroll
        for (int q = 0; q < PER; ++q) {
            const int r = r0 + ty + CSR_ROWS * q;
            if (r < n && c < n) v[q] = S[c + (long long)r * n];
        }
#pragma unroll
        for (int q = 0; q < PER; ++q) {
            const int r = r0 + ty + CSR_ROWS * q;
            if (r < n && c < n) {
                const long long pos = start + r * L + pofs + c;
                val[pos] = v[q];
                if (write_idx) col[pos] = (int)(cbase + c);
            }
        }
        return;
    }
    // value (r, c) = S[r + c n]: load coalesced along r (two 32-row halves),
    // write along c
#pragma unroll
    for (int q = 0; q < PER; ++q) {
        const int cl = ty + CSR_ROWS * (q >> 1), rl = tx + 32 * (q & 1);
        const int r = r0 + rl, c = c0 + cl;
        if (r < n && c < n) tile[cl][rl] = S[r + (long long)c * n];
    }
    __syncthreads();
#pragma unroll
    for (int q = 0; q < PER; ++q) {
        const int rl = ty + CSR_ROWS * q;
        const int r = r0 + rl, c = c0 + tx;
        if (r < n && c < n) {
            const long long pos = start + r * L + pofs + c;
            val[pos] = tile[tx][rl];
            if (write_idx) col[pos] = (int)(cbase + c);
        }
    }
}

template <class T>
int assemble(long long N, int n, const T *A, const T *B, int *row_ptr, int *col, T *val, bool write_idx,
             cudaStream_t s)
{
    if (write_idx) {
        const long long rows = N * n + 1;
        const int grid = (int)std::min<long long>((rows + 255) / 256, 152LL * 16);
        csr_rowptr_kernel<<<grid, 256, 0, s>>>(N, n, row_ptr);
        count_launch();
        BSS_CUDA(cudaGetLastError());
    }
    const long long tiles = N * 3 * ((n + CSR_TR - 1) / CSR_TR) * ((n + CSR_TC - 1) / CSR_TC);
    csr_values_kernel<T><<<(unsigned)tiles, CSR_TC * CSR_ROWS, 0, s>>>(N, n, A, B, col, val, write_idx ? 1 : 0);
    count_launch();
    BSS_CUDA(cudaGetLastError());
    return BSS_OK;
}

// d (n x k per block, column-major) <-> k vectors of length N n
template <class T>
__global__ void rhs_gather_kernel(long long N, int n, int k, const T *d, T *v, int to_vectors)
{
    const long long Nn = N * n, total = Nn * k;
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < total;
         e += (long long)gridDim.x * blockDim.x) {
        const long long c = e / Nn, q = e - c * Nn, i = q / n, r = q - i * n;
        const long long di = i * n * k + c * n + r;
        if (to_vectors)
            v[e] = d[di];
        else
            ((T *)d)[di] = v[e];
    }
}

template <class T>
int rhs_move(long long N, int n, int k, T *d, T *v, bool to_vectors, cudaStream_t s)
{
    const long long total = N * n * k;
    const int grid = (int)std::min<long long>((total + 255) / 256, 152LL * 16);
    rhs_gather_kernel<T><<<grid, 256, 0, s>>>(N, n, k, d, v, to_vectors ? 1 : 0);
    count_launch();
    BSS_CUDA(cudaGetLastError());
    return BSS_OK;
}

int sp_fail(cusolverStatus_t st, const char *what)
{
    return fail(st == CUSOLVER_STATUS_ALLOC_FAILED ? BSS_ERR_OOM : BSS_ERR_CUDA,
                std::string(what) + " failed (cusolverStatus " + std::to_string((int)st) + ")");
}

#define BSS_SP(call)                                             \
    do {                                                         \
        cusolverStatus_t s__ = (call);                           \
        if (s__ != CUSOLVER_STATUS_SUCCESS) return sp_fail(s__, #call); \
    } while (0)

bool args_ok(long long N, long long n) { return N >= 1 && n >= 1 && n <= 4096 && csr_nnz(N, n) < (1LL << 31) && N * n < (1LL << 31); }

}  // namespace

struct bss_spchol {
    int dtype = BSS_F64;
    long long N = 0, n = 0, k = 1, nnz = 0;
    cudaStream_t stream = nullptr;
    cusolverSpHandle_t sp = nullptr;
    cusparseMatDescr_t descr = nullptr;
    csrcholInfo_t info = nullptr;
    std::vector<void *> allocs;
    void *A = nullptr, *B = nullptr, *d = nullptr;  // user tensors (column-major blocks)
    int *row_ptr = nullptr, *col = nullptr;
    void *val = nullptr, *rhs = nullptr, *sol = nullptr, *work = nullptr;
    bool analyzed = false;  // symbolic phase done (pattern and workspace fixed)
    bool factored = false;  // a numeric factorization of the current values exists
};

namespace {

int sp_alloc(bss_spchol *h, void **p, size_t bytes)
{
    const cudaError_t e = cudaMalloc(p, bytes ? bytes : 16);
    if (e != cudaSuccess) return cuda_fail(e, "cudaMalloc(spchol)");
    h->allocs.push_back(*p);
    return cudaMemsetAsync(*p, 0, bytes ? bytes : 16, h->stream) == cudaSuccess ? BSS_OK : BSS_ERR_CUDA;
}

template <class T>
int sp_analyze(bss_spchol *h)
{
    const int m = (int)(h->N * h->n);
    h->factored = false;
    if (h->analyzed)  // the pattern is fixed by (N, n): refresh the values only
        return assemble<T>(h->N, (int)h->n, (const T *)h->A, (const T *)h->B, h->row_ptr, h->col, (T *)h->val, false,
                           h->stream);
    int rc = assemble<T>(h->N, (int)h->n, (const T *)h->A, (const T *)h->B, h->row_ptr, h->col, (T *)h->val, true,
                         h->stream);
    if (rc) return rc;
    BSS_SP(cusolverSpXcsrcholAnalysis(h->sp, m, (int)h->nnz, h->descr, h->row_ptr, h->col, h->info));
    size_t internal = 0, work = 0;
    if constexpr (std::is_same<T, double>::value)
        BSS_SP(cusolverSpDcsrcholBufferInfo(h->sp, m, (int)h->nnz, h->descr, (const double *)h->val, h->row_ptr,
                                            h->col, h->info, &internal, &work));
    else
        BSS_SP(cusolverSpScsrcholBufferInfo(h->sp, m, (int)h->nnz, h->descr, (const float *)h->val, h->row_ptr,
                                            h->col, h->info, &internal, &work));
    rc = sp_alloc(h, &h->work, work);
    if (rc) return rc;
    h->analyzed = true;
    return BSS_OK;
}

template <class T>
int sp_factor(bss_spchol *h)
{
    const int m = (int)(h->N * h->n);
    if (!h->analyzed) {
        const int rc = sp_analyze<T>(h);
        if (rc) return rc;
    } else {
        const int rc = assemble<T>(h->N, (int)h->n, (const T *)h->A, (const T *)h->B, h->row_ptr, h->col,
                                   (T *)h->val, false, h->stream);
        if (rc) return rc;
    }
    int pos = -1;
    h->factored = false;
    if constexpr (std::is_same<T, double>::value) {
        BSS_SP(cusolverSpDcsrcholFactor(h->sp, m, (int)h->nnz, h->descr, (const double *)h->val, h->row_ptr, h->col,
                                        h->info, h->work));
        BSS_SP(cusolverSpDcsrcholZeroPivot(h->sp, h->info, 0.0, &pos));
    } else {
        BSS_SP(cusolverSpScsrcholFactor(h->sp, m, (int)h->nnz, h->descr, (const float *)h->val, h->row_ptr, h->col,
                                        h->info, h->work));
        BSS_SP(cusolverSpScsrcholZeroPivot(h->sp, h->info, 0.0f, &pos));
    }
    // the library reports the pivot position counted from 1 (measured with a
    // zero-based matrix descriptor: a failed first row reads 1); -1 = none
    if (pos >= 0) {
        const long long row = pos > 0 ? pos - 1 : 0;
        return fail(BSS_ERR_NOT_SPD, "sparse Cholesky: non-positive pivot at row " + std::to_string(row) +
                                         " (block " + std::to_string(row / h->n) + ")");
    }
    h->factored = true;
    return BSS_OK;
}

template <class T>
int sp_solve(bss_spchol *h)
{
    if (!h->factored) return fail(BSS_ERR_STATE, "bss_spchol_solve: not factorized");
    const long long Nn = h->N * h->n;
    int rc = rhs_move<T>(h->N, (int)h->n, (int)h->k, (T *)h->d, (T *)h->rhs, true, h->stream);
    if (rc) return rc;
    for (long long c = 0; c < h->k; ++c) {
        const T *b = (const T *)h->rhs + c * Nn;
        T *x = (T *)h->sol + c * Nn;
        if constexpr (std::is_same<T, double>::value)
            BSS_SP(cusolverSpDcsrcholSolve(h->sp, (int)Nn, b, x, h->info, h->work));
        else
            BSS_SP(cusolverSpScsrcholSolve(h->sp, (int)Nn, b, x, h->info, h->work));
    }
    return rhs_move<T>(h->N, (int)h->n, (int)h->k, (T *)h->d, (T *)h->sol, false, h->stream);
}

}  // namespace

extern "C" int64_t bss_csr_nnz(int64_t N, int64_t n)
{
    if (N < 1 || n < 1) return -1;
    return csr_nnz(N, n);
}

extern "C" int bss_csr_assemble(int64_t N, int64_t n, int32_t dtype, const void *A, const void *B, int32_t *row_ptr,
                                int32_t *col_idx, void *vals, void *stream)
{
    if (!args_ok(N, n) || (dtype != BSS_F32 && dtype != BSS_F64) || !A || (N > 1 && !B) || !row_ptr || !col_idx ||
        !vals)
        return fail(BSS_ERR_ARG, "bss_csr_assemble: bad argument");
    const cudaStream_t s = (cudaStream_t)stream;
    return dtype == BSS_F64 ? assemble<double>(N, (int)n, (const double *)A, (const double *)B, row_ptr, col_idx,
                                               (double *)vals, true, s)
                            : assemble<float>(N, (int)n, (const float *)A, (const float *)B, row_ptr, col_idx,
                                              (float *)vals, true, s);
}

extern "C" int bss_spchol_create(int64_t N, int64_t n, int64_t k, int32_t dtype, void *stream, bss_spchol **out)
{
    if (!out || !args_ok(N, n) || k < 1 || (dtype != BSS_F32 && dtype != BSS_F64))
        return fail(BSS_ERR_ARG, "bss_spchol_create: bad argument");
    *out = nullptr;
    bss_spchol *h = new bss_spchol();
    h->dtype = dtype;
    h->N = N;
    h->n = n;
    h->k = k;
    h->nnz = csr_nnz(N, n);
    h->stream = (cudaStream_t)stream;
    const size_t es = dtype == BSS_F64 ? 8 : 4;
    int rc = BSS_OK;
    if (cusolverSpCreate(&h->sp) != CUSOLVER_STATUS_SUCCESS || cusparseCreateMatDescr(&h->descr) != CUSPARSE_STATUS_SUCCESS ||
        cusolverSpCreateCsrcholInfo(&h->info) != CUSOLVER_STATUS_SUCCESS)
        rc = fail(BSS_ERR_CUDA, "cuSOLVER sparse handle creation failed");
    if (!rc) {
        cusolverSpSetStream(h->sp, h->stream);
        cusparseSetMatType(h->descr, CUSPARSE_MATRIX_TYPE_GENERAL);
        cusparseSetMatIndexBase(h->descr, CUSPARSE_INDEX_BASE_ZERO);
        const size_t nn = (size_t)n * n;
        rc = sp_alloc(h, &h->A, es * nn * N);
        if (!rc) rc = sp_alloc(h, &h->B, es * nn * (N - 1));
        if (!rc) rc = sp_alloc(h, &h->d, es * (size_t)n * k * N);
        if (!rc) rc = sp_alloc(h, (void **)&h->row_ptr, 4 * (size_t)(N * n + 1));
        if (!rc) rc = sp_alloc(h, (void **)&h->col, 4 * (size_t)h->nnz);
        if (!rc) rc = sp_alloc(h, &h->val, es * (size_t)h->nnz);
        if (!rc) rc = sp_alloc(h, &h->rhs, es * (size_t)n * k * N);
        if (!rc) rc = sp_alloc(h, &h->sol, es * (size_t)n * k * N);
    }
    if (rc) {
        bss_spchol_destroy(h);
        return rc;
    }
    *out = h;
    return BSS_OK;
}

extern "C" int bss_spchol_destroy(bss_spchol *h)
{
    if (!h) return BSS_OK;
    if (h->stream)
        cudaStreamSynchronize(h->stream);
    else
        cudaDeviceSynchronize();
    for (void *p : h->allocs) cudaFree(p);
    if (h->info) cusolverSpDestroyCsrcholInfo(h->info);
    if (h->descr) cusparseDestroyMatDescr(h->descr);
    if (h->sp) cusolverSpDestroy(h->sp);
    delete h;
    return BSS_OK;
}

extern "C" int bss_spchol_get_tensors(bss_spchol *h, void **A, void **B, void **d)
{
    if (!h) return fail(BSS_ERR_ARG, "handle is NULL");
    if (A) *A = h->A;
    if (B) *B = h->B;
    if (d) *d = h->d;
    return BSS_OK;
}

extern "C" int bss_spchol_get_csr(bss_spchol *h, int32_t **row_ptr, int32_t **col_idx, void **vals, int64_t *nnz)
{
    if (!h) return fail(BSS_ERR_ARG, "handle is NULL");
    if (row_ptr) *row_ptr = h->row_ptr;
    if (col_idx) *col_idx = h->col;
    if (vals) *vals = h->val;
    if (nnz) *nnz = h->nnz;
    return BSS_OK;
}

extern "C" int bss_spchol_get_dims(bss_spchol *h, int64_t *N, int64_t *n, int64_t *k)
{
    if (!h) return fail(BSS_ERR_ARG, "handle is NULL");
    if (N) *N = h->N;
    if (n) *n = h->n;
    if (k) *k = h->k;
    return BSS_OK;
}

extern "C" int bss_spchol_analyze(bss_spchol *h)
{
    if (!h) return fail(BSS_ERR_ARG, "handle is NULL");
    return h->dtype == BSS_F64 ? sp_analyze<double>(h) : sp_analyze<float>(h);
}

extern "C" int bss_spchol_factorize(bss_spchol *h)
{
    if (!h) return fail(BSS_ERR_ARG, "handle is NULL");
    return h->dtype == BSS_F64 ? sp_factor<double>(h) : sp_factor<float>(h);
}

extern "C" int bss_spchol_solve(bss_spchol *h)
{
    if (!h) return fail(BSS_ERR_ARG, "handle is NULL");
    return h->dtype == BSS_F64 ? sp_solve<double>(h) : sp_solve<float>(h);
}
