// The reference's own GPU algorithm on this GPU, for comparison: a C++
// restatement of factorize!/solve! of BlockTriDiagData_batched
// (src/gpu_batched.jl:184-258) over the batched cuSOLVER/cuBLAS calls of
// src/backbone_cuda.jl:14-184 -- per level: potrfBatched / trsmBatched /
// gemmBatched along each partition's chain (batch = partitions), the n x 2n
// fill F = T^{-1} G by the same chain solve, M_2n = sum G^T F, the separator
// system LHS_A/LHS_B, recursion, and a sequential coarsest level -- with the
// reference planner's padding and level sizes (find_sequence_upper).  The
// calls, their order and operands follow the reference; the strided
// gathers it performs with copyto!/broadcasts are small kernels here, and
// the per-call pointer vectors it materialises are uploaded once.
// Comparator only: the library's own path is bss_create_batched.
#include <cublas_v2.h>
#include <cuda_runtime.h>
#include <cusolverDn.h>

#include <string>
#include <vector>

#include "bss_internal.h"

using namespace bss;

namespace {

// dst(r, c) (+)= alpha * op(src)(r, c) for rows x cols sub-blocks of nb
// block pairs: block b of dst at dst + doff + b * dstr (leading dim dld),
// of src at src + soff + b * sstr (leading dim sld); op = transpose or not
template <class T>
__global__ void blkop_kernel(T *dst, long long doff, long long dstr, int dld, const T *src, long long soff,
                             long long sstr, int sld, int rows, int cols, long long nb, int transpose, T alpha,
                             int accumulate)
{
    const long long per = (long long)rows * cols, total = per * nb;
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < total;
         e += (long long)gridDim.x * blockDim.x) {
        const long long b = e / per, q = e - b * per;
        const int r = (int)(q % rows), c = (int)(q / rows);
        const T v = src[soff + b * sstr + (transpose ? (long long)c + (long long)r * sld : (long long)r + (long long)c * sld)];
        T *o = dst + doff + b * dstr + r + (long long)c * dld;
        *o = accumulate ? *o + alpha * v : alpha * v;
    }
}

template <class T>
__global__ void identity_kernel(T *A, long long first, long long last, int n)
{
    const long long nn = (long long)n * n, total = (last - first) * nn;
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < total;
         e += (long long)gridDim.x * blockDim.x) {
        const long long q = e % nn;
        A[first * nn + e] = ((q % n) == (q / n)) ? T(1) : T(0);
    }
}

// library calls per type
inline cusolverStatus_t potrf_b(cusolverDnHandle_t h, int n, double **A, int *info, int bs)
{
    return cusolverDnDpotrfBatched(h, CUBLAS_FILL_MODE_UPPER, n, A, n, info, bs);
}
inline cusolverStatus_t potrf_b(cusolverDnHandle_t h, int n, float **A, int *info, int bs)
{
    return cusolverDnSpotrfBatched(h, CUBLAS_FILL_MODE_UPPER, n, A, n, info, bs);
}
inline cublasStatus_t trsm_b(cublasHandle_t h, cublasOperation_t op, int m, int nd, const double *one,
                             double *const *A, double *const *X, int bs)
{
    return cublasDtrsmBatched(h, CUBLAS_SIDE_LEFT, CUBLAS_FILL_MODE_UPPER, op, CUBLAS_DIAG_NON_UNIT, m, nd, one,
                              (const double *const *)A, m, X, m, bs);
}
inline cublasStatus_t trsm_b(cublasHandle_t h, cublasOperation_t op, int m, int nd, const float *one,
                             float *const *A, float *const *X, int bs)
{
    return cublasStrsmBatched(h, CUBLAS_SIDE_LEFT, CUBLAS_FILL_MODE_UPPER, op, CUBLAS_DIAG_NON_UNIT, m, nd, one,
                              (const float *const *)A, m, X, m, bs);
}
inline cublasStatus_t gemm_b(cublasHandle_t h, cublasOperation_t ta, cublasOperation_t tb, int m, int nn, int k,
                             const double *alpha, double *const *A, int lda, double *const *B, int ldb,
                             const double *beta, double *const *C, int ldc, int bs)
{
    return cublasDgemmBatched(h, ta, tb, m, nn, k, alpha, (const double *const *)A, lda, (const double *const *)B,
                              ldb, beta, C, ldc, bs);
}
inline cublasStatus_t gemm_b(cublasHandle_t h, cublasOperation_t ta, cublasOperation_t tb, int m, int nn, int k,
                             const float *alpha, float *const *A, int lda, float *const *B, int ldb,
                             const float *beta, float *const *C, int ldc, int bs)
{
    return cublasSgemmBatched(h, ta, tb, m, nn, k, alpha, (const float *const *)A, lda, (const float *const *)B,
                              ldb, beta, C, ldc, bs);
}

}  // namespace

struct bss_refalgo {
    int dtype = BSS_F64;
    long long N_user = 0, N = 0, n = 0, k = 1;
    cudaStream_t stream = nullptr;
    cublasHandle_t cb = nullptr;
    cusolverDnHandle_t cs = nullptr;
    std::vector<void *> allocs;
    void *A = nullptr, *B = nullptr, *d = nullptr;  // user-visible tensors (level 0)
    struct Lvl {
        long long N = 0, m = 0, P = 0;
        void *A = nullptr, *B = nullptr, *d = nullptr;  // level system (A, B: previous level's LHS)
        void *M1 = nullptr, *M2 = nullptr, *LA = nullptr, *LB = nullptr, *G = nullptr, *F = nullptr;
        void *M2n = nullptr, *b = nullptr, *dn = nullptr;
        // device pointer arrays: per interior position j (0 .. m-1), P-1 entries
        void **pA = nullptr, **pBint = nullptr, **pF = nullptr, **pG = nullptr, **pd = nullptr;
        void **pM2n = nullptr, **pb = nullptr, **pM1 = nullptr, **pM2 = nullptr;
        void **pdSep = nullptr, **pdSepR = nullptr, **pdFirst = nullptr, **pdLast = nullptr;
    };
    std::vector<Lvl> lv;
    long long Nc = 0;  // coarsest (sequential) size
    void *cA = nullptr, *cB = nullptr, *cd = nullptr;
    void **cpA = nullptr, **cpB = nullptr, **cpd = nullptr;  // one pointer per coarsest block
    int *info = nullptr;
};

namespace {

int ra_alloc(bss_refalgo *h, void **p, size_t bytes)
{
    const cudaError_t e = cudaMalloc(p, bytes ? bytes : 16);
    if (e != cudaSuccess) return cuda_fail(e, "cudaMalloc(refalgo)");
    h->allocs.push_back(*p);
    return cudaMemsetAsync(*p, 0, bytes ? bytes : 16, h->stream) == cudaSuccess ? BSS_OK : BSS_ERR_CUDA;
}

int upload_ptrs(bss_refalgo *h, void ***dst, const std::vector<void *> &v)
{
    int rc = ra_alloc(h, (void **)dst, v.size() * sizeof(void *));
    if (rc) return rc;
    BSS_CUDA(cudaMemcpy(*dst, v.data(), v.size() * sizeof(void *), cudaMemcpyHostToDevice));
    return BSS_OK;
}

template <class T>
cudaError_t blkop(cudaStream_t s, T *dst, long long doff, long long dstr, int dld, const T *src, long long soff,
                  long long sstr, int sld, int rows, int cols, long long nb, bool transpose, T alpha, bool acc)
{
    const long long total = (long long)rows * cols * nb;
    if (total <= 0) return cudaSuccess;
    const int grid = (int)std::min<long long>((total + 255) / 256, 152LL * 16);
    blkop_kernel<T><<<grid, 256, 0, s>>>(dst, doff, dstr, dld, src, soff, sstr, sld, rows, cols, nb,
                                         transpose ? 1 : 0, alpha, acc ? 1 : 0);
    count_launch();
    return cudaGetLastError();
}

template <class T>
int build(bss_refalgo *h)
{
    const long long n = h->n, nn = n * n, k = h->k;
    const size_t ts = sizeof(T);
    std::vector<int64_t> lev(3 * 64);
    int32_t nl = 0;
    int64_t coarsest = 0;
    int rc = bss_plan_reference(h->N_user, lev.data(), 64, &nl, &coarsest);
    if (rc) return rc;
    h->N = nl > 0 ? lev[0] : coarsest;
    rc = ra_alloc(h, &h->A, h->N * nn * ts);
    if (!rc) rc = ra_alloc(h, &h->B, std::max(h->N - 1, 1LL) * nn * ts);
    if (!rc) rc = ra_alloc(h, &h->d, h->N * n * k * ts);
    if (rc) return rc;
    void *curA = h->A, *curB = h->B, *curd = h->d;
    for (int l = 0; l < nl; ++l) {
        bss_refalgo::Lvl L;
        L.N = lev[3 * l];
        L.m = lev[3 * l + 1];
        L.P = lev[3 * l + 2];
        L.A = curA;
        L.B = curB;
        L.d = curd;
        const long long P1 = L.P - 1, m = L.m;
        rc = ra_alloc(h, &L.M1, P1 * nn * ts);
        if (!rc) rc = ra_alloc(h, &L.M2, P1 * nn * ts);
        if (!rc) rc = ra_alloc(h, &L.LA, L.P * nn * ts);
        if (!rc) rc = ra_alloc(h, &L.LB, std::max(P1, 1LL) * nn * ts);
        if (!rc) rc = ra_alloc(h, &L.G, L.N * 2 * nn * ts);
        if (!rc) rc = ra_alloc(h, &L.F, L.N * 2 * nn * ts);
        if (!rc) rc = ra_alloc(h, &L.M2n, P1 * 4 * nn * ts);
        if (!rc) rc = ra_alloc(h, &L.b, P1 * 2 * n * k * ts);
        if (!rc) rc = ra_alloc(h, &L.dn, L.P * n * k * ts);
        if (rc) return rc;
        std::vector<void *> pA, pBint, pF, pG, pd, pM2n, pb, pM1, pM2, pdSep, pdSepR, pdFirst, pdLast;
        T *A = (T *)L.A, *B = (T *)L.B, *d = (T *)L.d, *F = (T *)L.F, *G = (T *)L.G;
        for (long long j = 0; j < m; ++j)
            for (long long p = 0; p < P1; ++p) {
                const long long blk = p * (m + 1) + 1 + j;  // interior position j of partition p
                pA.push_back(A + blk * nn);
                pF.push_back(F + blk * 2 * nn);
                pG.push_back(G + blk * 2 * nn);
                pd.push_back(d + blk * n * k);
                pBint.push_back(B + blk * nn);  // couples interior j and j + 1 (used for j < m - 1)
            }
        for (long long p = 0; p < P1; ++p) {
            pM2n.push_back((T *)L.M2n + p * 4 * nn);
            pb.push_back((T *)L.b + p * 2 * n * k);
            pM1.push_back((T *)L.M1 + p * nn);
            pM2.push_back((T *)L.M2 + p * nn);
            pdSep.push_back(d + p * (m + 1) * n * k);
            pdSepR.push_back(d + (p + 1) * (m + 1) * n * k);
            pdFirst.push_back(d + (p * (m + 1) + 1) * n * k);
            pdLast.push_back(d + (p * (m + 1) + m) * n * k);
        }
        rc = upload_ptrs(h, &L.pA, pA);
        if (!rc) rc = upload_ptrs(h, &L.pBint, pBint);
        if (!rc) rc = upload_ptrs(h, &L.pF, pF);
        if (!rc) rc = upload_ptrs(h, &L.pG, pG);
        if (!rc) rc = upload_ptrs(h, &L.pd, pd);
        if (!rc) rc = upload_ptrs(h, &L.pM2n, pM2n);
        if (!rc) rc = upload_ptrs(h, &L.pb, pb);
        if (!rc) rc = upload_ptrs(h, &L.pM1, pM1);
        if (!rc) rc = upload_ptrs(h, &L.pM2, pM2);
        if (!rc) rc = upload_ptrs(h, &L.pdSep, pdSep);
        if (!rc) rc = upload_ptrs(h, &L.pdSepR, pdSepR);
        if (!rc) rc = upload_ptrs(h, &L.pdFirst, pdFirst);
        if (!rc) rc = upload_ptrs(h, &L.pdLast, pdLast);
        if (rc) return rc;
        h->lv.push_back(L);
        curA = L.LA;  // the next level's system is this level's LHS_A / LHS_B
        curB = L.LB;
        curd = L.dn;
    }
    h->Nc = coarsest;
    h->cA = curA;
    h->cB = curB;
    h->cd = curd;
    std::vector<void *> cpA, cpB, cpd;
    for (long long i = 0; i < h->Nc; ++i) {
        cpA.push_back((T *)h->cA + i * nn);
        cpB.push_back((T *)h->cB + i * nn);
        cpd.push_back((T *)h->cd + i * n * k);
    }
    rc = upload_ptrs(h, &h->cpA, cpA);
    if (!rc) rc = upload_ptrs(h, &h->cpB, cpB);
    if (!rc) rc = upload_ptrs(h, &h->cpd, cpd);
    if (!rc) rc = ra_alloc(h, (void **)&h->info, sizeof(int) * (size_t)std::max(h->N, 1LL));
    if (rc) return rc;
    // identity padding of A (gpu_batched.jl:177-179, 1-based i = N .. N_use)
    const long long first = h->N_user - 1;
    if (h->N > first) {
        identity_kernel<T><<<152 * 4, 256, 0, h->stream>>>((T *)h->A, first, h->N, (int)n);
        count_launch();
        BSS_CUDA(cudaGetLastError());
    }
    return BSS_OK;
}

#define CBX(call)                                                                                         \
    do {                                                                                                  \
        if ((call) != 0) return fail(BSS_ERR_CUDA, std::string("library call failed: ") + #call);         \
    } while (0)

// cholesky_factorize_batched! (backbone_cuda.jl:70-101) over the partitions
template <class T>
int chain_factor(bss_refalgo *h, const bss_refalgo::Lvl &L)
{
    const int n = (int)h->n, bs = (int)(L.P - 1);
    const T one = T(1), mone = T(-1);
    T **pA = (T **)L.pA, **pB = (T **)L.pBint;
    CBX(potrf_b(h->cs, n, pA, h->info, bs));
    for (long long j = 1; j < L.m; ++j) {
        CBX(trsm_b(h->cb, CUBLAS_OP_T, n, n, &one, pA + (j - 1) * bs, pB + (j - 1) * bs, bs));
        CBX(gemm_b(h->cb, CUBLAS_OP_T, CUBLAS_OP_N, n, n, n, &mone, pB + (j - 1) * bs, n, pB + (j - 1) * bs, n, &one,
                   pA + j * bs, n, bs));
        CBX(potrf_b(h->cs, n, pA + j * bs, h->info, bs));
    }
    return BSS_OK;
}

// cholesky_solve_batched! (backbone_cuda.jl:103-141) with nd right-hand columns
template <class T>
int chain_solve(bss_refalgo *h, const bss_refalgo::Lvl &L, T **pX, int nd)
{
    const int n = (int)h->n, bs = (int)(L.P - 1);
    const T one = T(1), mone = T(-1);
    T **pA = (T **)L.pA, **pB = (T **)L.pBint;
    CBX(trsm_b(h->cb, CUBLAS_OP_T, n, nd, &one, pA, pX, bs));
    for (long long j = 1; j < L.m; ++j) {
        CBX(gemm_b(h->cb, CUBLAS_OP_T, CUBLAS_OP_N, n, nd, n, &mone, pB + (j - 1) * bs, n, pX + (j - 1) * bs, n, &one,
                   pX + j * bs, n, bs));
        CBX(trsm_b(h->cb, CUBLAS_OP_T, n, nd, &one, pA + j * bs, pX + j * bs, bs));
    }
    for (long long j = L.m - 1; j >= 1; --j) {
        CBX(trsm_b(h->cb, CUBLAS_OP_N, n, nd, &one, pA + j * bs, pX + j * bs, bs));
        CBX(gemm_b(h->cb, CUBLAS_OP_N, CUBLAS_OP_N, n, nd, n, &mone, pB + (j - 1) * bs, n, pX + j * bs, n, &one,
                   pX + (j - 1) * bs, n, bs));
    }
    CBX(trsm_b(h->cb, CUBLAS_OP_N, n, nd, &one, pA, pX, bs));
    return BSS_OK;
}

// sequential coarsest level: cholesky_factorize! / cholesky_solve!
// (backbone_cuda.jl:14-61), one block per call
template <class T>
int seq_factor(bss_refalgo *h)
{
    const int n = (int)h->n;
    const T one = T(1), mone = T(-1);
    T **pA = (T **)h->cpA, **pB = (T **)h->cpB;
    CBX(potrf_b(h->cs, n, pA, h->info, 1));
    for (long long i = 1; i < h->Nc; ++i) {
        CBX(trsm_b(h->cb, CUBLAS_OP_T, n, n, &one, pA + i - 1, pB + i - 1, 1));
        CBX(gemm_b(h->cb, CUBLAS_OP_T, CUBLAS_OP_N, n, n, n, &mone, pB + i - 1, n, pB + i - 1, n, &one, pA + i, n, 1));
        CBX(potrf_b(h->cs, n, pA + i, h->info, 1));
    }
    return BSS_OK;
}

template <class T>
int seq_solve(bss_refalgo *h)
{
    const int n = (int)h->n, k = (int)h->k;
    const T one = T(1), mone = T(-1);
    T **pA = (T **)h->cpA, **pB = (T **)h->cpB, **pd = (T **)h->cpd;
    const long long N = h->Nc;
    CBX(trsm_b(h->cb, CUBLAS_OP_T, n, k, &one, pA, pd, 1));
    for (long long i = 1; i < N; ++i) {
        CBX(gemm_b(h->cb, CUBLAS_OP_T, CUBLAS_OP_N, n, k, n, &mone, pB + i - 1, n, pd + i - 1, n, &one, pd + i, n, 1));
        CBX(trsm_b(h->cb, CUBLAS_OP_T, n, k, &one, pA + i, pd + i, 1));
    }
    CBX(trsm_b(h->cb, CUBLAS_OP_N, n, k, &one, pA + N - 1, pd + N - 1, 1));
    for (long long i = N - 2; i >= 0; --i) {
        CBX(gemm_b(h->cb, CUBLAS_OP_N, CUBLAS_OP_N, n, k, n, &mone, pB + i, n, pd + i + 1, n, &one, pd + i, n, 1));
        CBX(trsm_b(h->cb, CUBLAS_OP_N, n, k, &one, pA + i, pd + i, 1));
    }
    return BSS_OK;
}

// factorize! (gpu_batched.jl:184-227), level by level
template <class T>
int factorize_t(bss_refalgo *h)
{
    const long long n = h->n, nn = n * n;
    const T one = T(1);
    cudaStream_t s = h->stream;
    for (const auto &L : h->lv) {
        const long long P1 = L.P - 1, m = L.m, step = (m + 1) * nn;
        T *A = (T *)L.A, *B = (T *)L.B;
        BSS_CUDA(cudaMemsetAsync(L.LA, 0, L.P * nn * sizeof(T), s));
        BSS_CUDA(cudaMemsetAsync(L.LB, 0, std::max(P1, 1LL) * nn * sizeof(T), s));
        BSS_CUDA(cudaMemsetAsync(L.M2n, 0, P1 * 4 * nn * sizeof(T), s));
        BSS_CUDA(cudaMemsetAsync(L.G, 0, L.N * 2 * nn * sizeof(T), s));
        // M_1 = B[1:(m+1):N-1], M_2 = B[(m+1):(m+1):N-1], LHS_A = A[1:(m+1):N]
        BSS_CUDA(blkop<T>(s, (T *)L.M1, 0, nn, (int)n, B, 0, step, (int)n, (int)n, (int)n, P1, false, one, false));
        BSS_CUDA(blkop<T>(s, (T *)L.M2, 0, nn, (int)n, B, m * nn, step, (int)n, (int)n, (int)n, P1, false, one, false));
        BSS_CUDA(blkop<T>(s, (T *)L.LA, 0, nn, (int)n, A, 0, step, (int)n, (int)n, (int)n, L.P, false, one, false));
        // G[:, 1:n, 2:(m+1):N] = M_1^T ; G[:, n+1:2n, (m+1):(m+1):N] = M_2 ; F = G
        BSS_CUDA(blkop<T>(s, (T *)L.G, 2 * nn, (m + 1) * 2 * nn, (int)n, (T *)L.M1, 0, nn, (int)n, (int)n, (int)n, P1,
                          true, one, false));
        BSS_CUDA(blkop<T>(s, (T *)L.G, m * 2 * nn + nn, (m + 1) * 2 * nn, (int)n, (T *)L.M2, 0, nn, (int)n, (int)n,
                          (int)n, P1, false, one, false));
        BSS_CUDA(cudaMemcpyAsync(L.F, L.G, L.N * 2 * nn * sizeof(T), cudaMemcpyDeviceToDevice, s));
        int rc = chain_factor<T>(h, L);
        if (!rc) rc = chain_solve<T>(h, L, (T **)L.pF, (int)(2 * n));
        if (rc) return rc;
        // compute_schur_complement! (backbone_cuda.jl:143-157)
        for (long long j = 0; j < m; ++j)
            CBX(gemm_b(h->cb, CUBLAS_OP_T, CUBLAS_OP_N, (int)(2 * n), (int)(2 * n), (int)n, &one, (T **)L.pG + j * P1,
                       (int)n, (T **)L.pF + j * P1, (int)n, &one, (T **)L.pM2n, (int)(2 * n), (int)P1));
        const T mone = T(-1);
        BSS_CUDA(blkop<T>(s, (T *)L.LA, 0, nn, (int)n, (T *)L.M2n, 0, 4 * nn, (int)(2 * n), (int)n, (int)n, P1, false,
                          mone, true));
        BSS_CUDA(blkop<T>(s, (T *)L.LA, nn, nn, (int)n, (T *)L.M2n, n + 2 * nn, 4 * nn, (int)(2 * n), (int)n, (int)n,
                          P1, false, mone, true));
        BSS_CUDA(blkop<T>(s, (T *)L.LB, 0, nn, (int)n, (T *)L.M2n, 2 * nn, 4 * nn, (int)(2 * n), (int)n, (int)n, P1,
                          false, mone, true));
    }
    return seq_factor<T>(h);
}

// solve! (gpu_batched.jl:229-258)
template <class T>
int solve_level(bss_refalgo *h, size_t l)
{
    if (l == h->lv.size()) return seq_solve<T>(h);
    const auto &L = h->lv[l];
    const long long n = h->n, k = h->k, nk = n * k, P1 = L.P - 1, m = L.m;
    const T one = T(1), mone = T(-1);
    cudaStream_t s = h->stream;
    T *d = (T *)L.d;
    BSS_CUDA(cudaMemsetAsync(L.b, 0, P1 * 2 * nk * sizeof(T), s));
    // compute_schur_RHS! (backbone_cuda.jl:159-171)
    for (long long j = 0; j < m; ++j)
        CBX(gemm_b(h->cb, CUBLAS_OP_T, CUBLAS_OP_N, (int)(2 * n), (int)k, (int)n, &mone, (T **)L.pF + j * P1, (int)n,
                   (T **)L.pd + j * P1, (int)n, &one, (T **)L.pb, (int)(2 * n), (int)P1));
    BSS_CUDA(blkop<T>(s, d, 0, (m + 1) * nk, (int)n, (T *)L.b, 0, 2 * nk, (int)(2 * n), (int)n, (int)k, P1, false,
                      one, true));
    BSS_CUDA(blkop<T>(s, d, (m + 1) * nk, (m + 1) * nk, (int)n, (T *)L.b, n, 2 * nk, (int)(2 * n), (int)n, (int)k,
                      P1, false, one, true));
    // separators down, recurse, back
    BSS_CUDA(blkop<T>(s, (T *)L.dn, 0, nk, (int)n, d, 0, (m + 1) * nk, (int)n, (int)n, (int)k, L.P, false, one, false));
    int rc = solve_level<T>(h, l + 1);
    if (rc) return rc;
    BSS_CUDA(blkop<T>(s, d, 0, (m + 1) * nk, (int)n, (T *)L.dn, 0, nk, (int)n, (int)n, (int)k, L.P, false, one, false));
    // update_boundary! (backbone_cuda.jl:173-184)
    CBX(gemm_b(h->cb, CUBLAS_OP_T, CUBLAS_OP_N, (int)n, (int)k, (int)n, &mone, (T **)L.pM1, (int)n, (T **)L.pdSep,
               (int)n, &one, (T **)L.pdFirst, (int)n, (int)P1));
    CBX(gemm_b(h->cb, CUBLAS_OP_N, CUBLAS_OP_N, (int)n, (int)k, (int)n, &mone, (T **)L.pM2, (int)n, (T **)L.pdSepR,
               (int)n, &one, (T **)L.pdLast, (int)n, (int)P1));
    return chain_solve<T>(h, L, (T **)L.pd, (int)k);
}

}  // namespace

extern "C" int bss_refalgo_create(int64_t N, int64_t n, int64_t k, int32_t dtype, void *stream, bss_refalgo **out)
{
    if (!out || N < 1 || n < 1 || k < 1 || (dtype != BSS_F32 && dtype != BSS_F64))
        return fail(BSS_ERR_ARG, "bss_refalgo_create: bad argument");
    *out = nullptr;
    bss_refalgo *h = new bss_refalgo();
    h->dtype = dtype;
    h->N_user = N;
    h->n = n;
    h->k = k;
    h->stream = (cudaStream_t)stream;
    int rc = BSS_OK;
    if (cublasCreate(&h->cb) != CUBLAS_STATUS_SUCCESS || cusolverDnCreate(&h->cs) != CUSOLVER_STATUS_SUCCESS)
        rc = fail(BSS_ERR_CUDA, "cuBLAS/cuSOLVER handle creation failed");
    if (!rc) {
        cublasSetStream(h->cb, h->stream);
        cusolverDnSetStream(h->cs, h->stream);
        rc = dtype == BSS_F64 ? build<double>(h) : build<float>(h);
    }
    if (rc) {
        bss_refalgo_destroy(h);
        return rc;
    }
    *out = h;
    return BSS_OK;
}

extern "C" int bss_refalgo_destroy(bss_refalgo *h)
{
    if (!h) return BSS_OK;
    if (h->stream)
        cudaStreamSynchronize(h->stream);
    else
        cudaDeviceSynchronize();
    for (void *p : h->allocs) cudaFree(p);
    if (h->cb) cublasDestroy(h->cb);
    if (h->cs) cusolverDnDestroy(h->cs);
    delete h;
    return BSS_OK;
}

extern "C" int bss_refalgo_get_tensors(bss_refalgo *h, void **A, void **B, void **d)
{
    if (!h) return fail(BSS_ERR_ARG, "handle is NULL");
    if (A) *A = h->A;
    if (B) *B = h->B;
    if (d) *d = h->d;
    return BSS_OK;
}

extern "C" int bss_refalgo_get_dims(bss_refalgo *h, int64_t *N, int64_t *n, int64_t *k)
{
    if (!h) return fail(BSS_ERR_ARG, "handle is NULL");
    if (N) *N = h->N;
    if (n) *n = h->n;
    if (k) *k = h->k;
    return BSS_OK;
}

extern "C" int bss_refalgo_factorize(bss_refalgo *h)
{
    if (!h) return fail(BSS_ERR_ARG, "handle is NULL");
    return h->dtype == BSS_F64 ? factorize_t<double>(h) : factorize_t<float>(h);
}

extern "C" int bss_refalgo_solve(bss_refalgo *h)
{
    if (!h) return fail(BSS_ERR_ARG, "handle is NULL");
    return h->dtype == BSS_F64 ? solve_level<double>(h, 0) : solve_level<float>(h, 0);
}
