// Host (CPU) block Cholesky: the reference's CPU API initialize_cpu /
// factorize! / solve! (src/cpu.jl:12-50) over the sequential block
// recursion of src/backbone_cpu.jl:5-33, in plain C++ (host code only; no
// GPU is touched).  Storage is the same column-major n x n x N / n x k x N
// layout as the GPU handles.  After factorize, A_i holds U_i in its upper
// triangle (the strictly lower part holds A_i - B_{i-1}^T B_{i-1}: the
// update touches the whole block and potrf 'U' leaves the lower part, as
// in the reference) and B_i holds U_i^{-T} B_i; after solve, d holds x.
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <string>

#include "bss_internal.h"

using namespace bss;

struct bss_cpu_handle {
    long long N = 0, n = 0, k = 0;
    int dtype = BSS_F64;
    void *A = nullptr, *B = nullptr, *d = nullptr;
    bool factored = false;
    long long failed_block = -1;
};

namespace {

// upper Cholesky in place: A = U^T U, upper triangle of A (ld n) -> U;
// returns false on a non-positive or non-finite pivot
template <class T>
bool potrf_upper(T *a, long long n)
{
    for (long long j = 0; j < n; ++j) {
        T *cj = a + j * n;
        // U(0:j, j) = U(0:j,0:j)^{-T} A(0:j, j)  (column j above the diagonal)
        for (long long i = 0; i < j; ++i) {
            const T *ci = a + i * n;
            T s = cj[i];
            for (long long p = 0; p < i; ++p) s -= ci[p] * cj[p];
            cj[i] = s / ci[i];
        }
        T dsum = cj[j];
        for (long long p = 0; p < j; ++p) dsum -= cj[p] * cj[p];
        if (!(dsum > T(0)) || !std::isfinite((double)dsum)) return false;
        cj[j] = std::sqrt(dsum);
    }
    return true;
}

// X <- U^{-T} X   (U upper n x n, X n x m, both ld n): forward substitution
template <class T>
void trsm_ut(const T *u, T *x, long long n, long long m)
{
    for (long long c = 0; c < m; ++c) {
        T *xc = x + c * n;
        for (long long i = 0; i < n; ++i) {
            const T *ui = u + i * n;  // column i of U: U(0:i, i)
            T s = xc[i];
            for (long long p = 0; p < i; ++p) s -= ui[p] * xc[p];
            xc[i] = s / ui[i];
        }
    }
}

// X <- U^{-1} X: backward substitution, column-oriented
template <class T>
void trsm_un(const T *u, T *x, long long n, long long m)
{
    for (long long c = 0; c < m; ++c) {
        T *xc = x + c * n;
        for (long long i = n - 1; i >= 0; --i) {
            const T *ui = u + i * n;
            xc[i] /= ui[i];
            const T xi = xc[i];
            for (long long p = 0; p < i; ++p) xc[p] -= ui[p] * xi;
        }
    }
}

// C(n x m) -= X^T Y   (X n x n, Y n x m; all ld n)
template <class T>
void gemm_tn_sub(const T *x, const T *y, T *c, long long n, long long m)
{
    for (long long j = 0; j < m; ++j) {
        const T *yj = y + j * n;
        T *cj = c + j * n;
        for (long long i = 0; i < n; ++i) {
            const T *xi = x + i * n;
            T s = T(0);
            for (long long p = 0; p < n; ++p) s += xi[p] * yj[p];
            cj[i] -= s;
        }
    }
}

// C(n x m) -= X Y   (X n x n, Y n x m)
template <class T>
void gemm_nn_sub(const T *x, const T *y, T *c, long long n, long long m)
{
    for (long long j = 0; j < m; ++j) {
        const T *yj = y + j * n;
        T *cj = c + j * n;
        for (long long p = 0; p < n; ++p) {
            const T *xp = x + p * n;
            const T yp = yj[p];
            for (long long i = 0; i < n; ++i) cj[i] -= xp[i] * yp;
        }
    }
}

// A_i -= B^T B on the whole block, as the reference's gemm!('T', 'N') does
// (potrf 'U' then reads only the upper triangle)
template <class T>
void syrk_full_sub(const T *b, T *a, long long n)
{
    for (long long j = 0; j < n; ++j) {
        const T *bj = b + j * n;
        T *aj = a + j * n;
        for (long long i = 0; i < n; ++i) {
            const T *bi = b + i * n;
            T s = T(0);
            for (long long p = 0; p < n; ++p) s += bi[p] * bj[p];
            aj[i] -= s;
        }
    }
}

template <class T>
int factorize_t(bss_cpu_handle *h)
{
    const long long n = h->n, nn = n * n;
    T *A = (T *)h->A, *B = (T *)h->B;
    h->failed_block = -1;
    if (!potrf_upper<T>(A, n)) h->failed_block = 0;
    for (long long i = 1; i < h->N && h->failed_block < 0; ++i) {
        trsm_ut<T>(A + (i - 1) * nn, B + (i - 1) * nn, n, n);    // B_{i-1} <- U_{i-1}^{-T} B_{i-1}
        syrk_full_sub<T>(B + (i - 1) * nn, A + i * nn, n);      // A_i -= B^T B
        if (!potrf_upper<T>(A + i * nn, n)) h->failed_block = i;
    }
    h->factored = true;
    if (h->failed_block >= 0)
        return fail(BSS_ERR_NOT_SPD, "pivot failed at block " + std::to_string(h->failed_block));
    return BSS_OK;
}

template <class T>
int solve_t(bss_cpu_handle *h)
{
    const long long n = h->n, k = h->k, nn = n * n, nk = n * k, N = h->N;
    const T *A = (const T *)h->A, *B = (const T *)h->B;
    T *d = (T *)h->d;
    trsm_ut<T>(A, d, n, k);
    for (long long i = 1; i < N; ++i) {
        gemm_tn_sub<T>(B + (i - 1) * nn, d + (i - 1) * nk, d + i * nk, n, k);
        trsm_ut<T>(A + i * nn, d + i * nk, n, k);
    }
    trsm_un<T>(A + (N - 1) * nn, d + (N - 1) * nk, n, k);
    for (long long i = N - 2; i >= 0; --i) {
        gemm_nn_sub<T>(B + i * nn, d + (i + 1) * nk, d + i * nk, n, k);
        trsm_un<T>(A + i * nn, d + i * nk, n, k);
    }
    return BSS_OK;
}

}  // namespace

extern "C" int bss_cpu_create(int64_t N, int64_t n, int64_t k, int32_t dtype, bss_cpu_handle **out)
{
    if (!out) return fail(BSS_ERR_ARG, "out is NULL");
    *out = nullptr;
    if (N < 1 || n < 1 || k < 1) return fail(BSS_ERR_ARG, "N, n and k must be >= 1");
    if (dtype != BSS_F32 && dtype != BSS_F64) return fail(BSS_ERR_ARG, "dtype must be BSS_F32 or BSS_F64");
    const size_t ts = dtype == BSS_F64 ? 8 : 4;
    bss_cpu_handle *h = new bss_cpu_handle();
    h->N = N;
    h->n = n;
    h->k = k;
    h->dtype = dtype;
    // zero-initialised like initialize_cpu's zeros(n, n)
    h->A = std::calloc((size_t)(N * n * n), ts);
    h->B = std::calloc((size_t)(std::max<int64_t>(N - 1, 1) * n * n), ts);
    h->d = std::calloc((size_t)(N * n * k), ts);
    if (!h->A || !h->B || !h->d) {
        std::free(h->A);
        std::free(h->B);
        std::free(h->d);
        delete h;
        return fail(BSS_ERR_OOM, "host allocation failed");
    }
    *out = h;
    return BSS_OK;
}

extern "C" int bss_cpu_destroy(bss_cpu_handle *h)
{
    if (!h) return BSS_OK;
    std::free(h->A);
    std::free(h->B);
    std::free(h->d);
    delete h;
    return BSS_OK;
}

extern "C" int bss_cpu_get_tensors(bss_cpu_handle *h, void **A, void **B, void **d)
{
    if (!h) return fail(BSS_ERR_ARG, "handle is NULL");
    if (A) *A = h->A;
    if (B) *B = h->B;
    if (d) *d = h->d;
    return BSS_OK;
}

extern "C" int bss_cpu_factorize(bss_cpu_handle *h)
{
    if (!h) return fail(BSS_ERR_ARG, "handle is NULL");
    return h->dtype == BSS_F64 ? factorize_t<double>(h) : factorize_t<float>(h);
}

extern "C" int bss_cpu_solve(bss_cpu_handle *h)
{
    if (!h) return fail(BSS_ERR_ARG, "handle is NULL");
    if (!h->factored) return fail(BSS_ERR_STATE, "solve before factorize");
    return h->dtype == BSS_F64 ? solve_t<double>(h) : solve_t<float>(h);
}

extern "C" int bss_cpu_failed_block(bss_cpu_handle *h, int64_t *block)
{
    if (!h || !block) return fail(BSS_ERR_ARG, "bad argument");
    *block = h->failed_block;
    return BSS_OK;
}
