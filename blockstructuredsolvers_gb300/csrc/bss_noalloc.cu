// bss_factor_solve_noalloc: factorize + solve on caller-owned buffers with
// the recursion workspace in a static device array (no device allocation).
//
// For callers that cannot allocate device memory (a host runtime whose own
// memory manager owns the device pool, a fixed-budget serving process).  The
// kernels are the library's chain kernels; only where their workspace lives
// differs from the handle path in bss_api.cu.
#include <cuda_runtime.h>

#include <mutex>
#include <string>

#include "../../include/bss.h"
#include "bss_launch.h"

using namespace bss;

// Workspace of every call of bss_factor_solve_noalloc.  Each GPU that loads
// the library holds these bytes until the process exits.
static __device__ __align__(256) unsigned char g_noalloc_scratch[BSS_NOALLOC_SCRATCH_BYTES];

namespace {

constexpr int kMaxDevices = 64;
constexpr int kMaxLevels = 40;
std::mutex g_addr_mu;
void *g_addr[kMaxDevices];  // device address of g_noalloc_scratch, per device

thread_local std::string g_noalloc_err;  // message of the failing call, copied to bss_last_error_string()

// In host code the array's name is only a host-side stand-in; the kernels
// need its device address, looked up once per device with that device
// current.
int scratch_address(char **out)
{
    int dev = -1;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) {
        g_noalloc_err = std::string("cudaGetDevice: ") + cudaGetErrorString(e);
        return BSS_ERR_CUDA;
    }
    if (dev < 0 || dev >= kMaxDevices) {
        g_noalloc_err = "device index out of range";
        return BSS_ERR_ARG;
    }
    std::lock_guard<std::mutex> lk(g_addr_mu);
    if (!g_addr[dev]) {
        void *p = nullptr;
        e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess || !p) {
            g_noalloc_err = std::string("cudaGetSymbolAddress: ") + cudaGetErrorString(e);
            return BSS_ERR_CUDA;
        }
        g_addr[dev] = p;
    }
    *out = static_cast<char *>(g_addr[dev]);
    return BSS_OK;
}

struct NaLevel {
    long long N, Q;
    bool seq;
    void *A, *B, *d, *Y, *C, *bvec;
};

inline size_t align256(size_t b) { return (b + 255) & ~(size_t)255; }

template <class T>
int run(long long N, int n, int k, T *A, T *B, T *d, cudaStream_t s)
{
    const size_t ts = sizeof(T);
    const long long nn = (long long)n * n;
    const int kc_max = solve_kc_max(n, k, (int)ts);
    // plan: partitions per level capped so the workspace stays small; the
    // chain kernels do not depend on the partition count for correctness
    NaLevel lv[kMaxLevels];
    int nlev = 0;
    long long ncur = N;
    while (ncur > 8 && nlev < kMaxLevels - 1) {
        long long q = (ncur - 1) / 2;
        if (q > 64) q = 64;
        lv[nlev++] = NaLevel{ncur, q, false, nullptr, nullptr, nullptr, nullptr, nullptr, nullptr};
        ncur = q + 1;
    }
    lv[nlev++] = NaLevel{ncur, 0, true, nullptr, nullptr, nullptr, nullptr, nullptr, nullptr};

    // workspace layout: status, then per level (Y, C, bvec) and the next
    // level's system (A, B, d)
    size_t off = align256(sizeof(DevStatus));
    size_t offs[kMaxLevels][6];
    for (int l = 0; l < nlev; ++l) {
        for (int q = 0; q < 6; ++q) offs[l][q] = 0;
        if (l > 0) {
            offs[l][0] = off;
            off += align256((size_t)lv[l].N * nn * ts);
            offs[l][1] = off;
            off += align256((size_t)(lv[l].N > 1 ? lv[l].N - 1 : 1) * nn * ts);
            offs[l][2] = off;
            off += align256((size_t)lv[l].N * n * k * ts);
        }
        if (!lv[l].seq) {
            offs[l][3] = off;
            off += align256((size_t)lv[l].N * nn * ts);
            offs[l][4] = off;
            off += align256((size_t)lv[l].Q * 3 * nn * ts);
            offs[l][5] = off;
            off += align256((size_t)lv[l].Q * 2 * n * kc_max * ts);
        }
    }
    if (off > (size_t)BSS_NOALLOC_SCRATCH_BYTES) {
        g_noalloc_err = "bss_factor_solve_noalloc: N=" + std::to_string(N) + ", n=" + std::to_string(n) +
                        ", k=" + std::to_string(k) + " needs " + std::to_string(off) +
                        " bytes of workspace; the static workspace holds " +
                        std::to_string((size_t)BSS_NOALLOC_SCRATCH_BYTES);
        return BSS_ERR_ARG;
    }
    char *base = nullptr;
    int rc = scratch_address(&base);
    if (rc) return rc;
    DevStatus *st = reinterpret_cast<DevStatus *>(base);
    for (int l = 0; l < nlev; ++l) {
        if (l == 0) {
            lv[l].A = A;
            lv[l].B = B;
            lv[l].d = d;
        } else {
            lv[l].A = base + offs[l][0];
            lv[l].B = base + offs[l][1];
            lv[l].d = base + offs[l][2];
        }
        if (!lv[l].seq) {
            lv[l].Y = base + offs[l][3];
            lv[l].C = base + offs[l][4];
            lv[l].bvec = base + offs[l][5];
        }
    }

    cudaError_t e;
#define NA_CHECK(x)                                                                     \
    do {                                                                                \
        e = (x);                                                                        \
        if (e != cudaSuccess) {                                                         \
            g_noalloc_err = std::string(#x) + ": " + cudaGetErrorString(e);             \
            return BSS_ERR_CUDA;                                                        \
        }                                                                               \
    } while (0)
    // the array keeps the previous call's contents: reset the status words
    // (every other workspace byte is written before it is read)
    NA_CHECK(cudaMemsetAsync(st, 0, sizeof(DevStatus), s));
    NA_CHECK(cudaMemsetAsync(&st->bad_key, 0xFF, sizeof(unsigned long long), s));
    for (int l = 0; l < nlev; ++l) {
        ChainFactorArgs<T, T> a;
        a.A_in = (const T *)lv[l].A;
        a.B_in = (const T *)lv[l].B;
        a.A_f = (T *)lv[l].A;
        a.B_f = (T *)lv[l].B;
        a.Y = (T *)lv[l].Y;
        a.C = (T *)lv[l].C;
        a.N = lv[l].N;
        a.Q = lv[l].Q;
        a.n = n;
        a.seq = lv[l].seq ? 1 : 0;
        a.level = l;
        a.st = st;
        a.variant = default_factor_variant();
        NA_CHECK((launch_chain_factor<T, T>(a, s)));
        if (!lv[l].seq)
            NA_CHECK((launch_assemble_schur<T, T, T>((const T *)lv[l].A, (const T *)lv[l].C, (T *)lv[l + 1].A,
                                                     (T *)lv[l + 1].B, lv[l].N, lv[l].Q, n, s)));
    }
    for (int j0 = 0; j0 < k; j0 += kc_max) {
        const int kc = (k - j0 < kc_max) ? k - j0 : kc_max;
        for (int l = 0; l < nlev; ++l) {
            SolveArgs<T> a;
            a.Af = (const T *)lv[l].A;
            a.Bf = (const T *)lv[l].B;
            a.Y = (const T *)lv[l].Y;
            a.d = (T *)lv[l].d;
            a.bvec = (T *)lv[l].bvec;
            a.xsep = (l + 1 < nlev) ? lv[l + 1].d : nullptr;
            a.N = lv[l].N;
            a.Q = lv[l].Q;
            a.n = n;
            a.k = k;
            a.j0 = j0;
            a.kc = kc;
            a.seq = lv[l].seq ? 1 : 0;
            a.st = st;
            NA_CHECK(launch_chain_fwd<T>(a, s));
            if (!lv[l].seq)
                NA_CHECK((launch_assemble_rhs<T, T>((const T *)lv[l].d, (const T *)lv[l].bvec, (T *)lv[l + 1].d,
                                                    lv[l].N, lv[l].Q, n, k, j0, kc, s)));
        }
        for (int l = nlev - 2; l >= 0; --l) {
            SolveArgs<T> a;
            a.Af = (const T *)lv[l].A;
            a.Bf = (const T *)lv[l].B;
            a.Y = (const T *)lv[l].Y;
            a.d = (T *)lv[l].d;
            a.bvec = (T *)lv[l].bvec;
            a.xsep = lv[l + 1].d;
            a.N = lv[l].N;
            a.Q = lv[l].Q;
            a.n = n;
            a.k = k;
            a.j0 = j0;
            a.kc = kc;
            a.seq = 0;
            a.st = st;
            NA_CHECK((launch_chain_bwd<T, T>(a, s)));
        }
    }
    // one copy of the whole status: the failed-pivot key and the flag the
    // tensor-core kernels set when a bounded wait expired
    DevStatus hs;
    NA_CHECK(cudaMemcpyAsync(&hs, st, sizeof(hs), cudaMemcpyDeviceToHost, s));
    NA_CHECK(cudaStreamSynchronize(s));
#undef NA_CHECK
    if (hs.tc_timeout) {
        g_noalloc_err = "a bounded tensor-core wait expired during factorize; the factors are void";
        return BSS_ERR_TIMEOUT;
    }
    const unsigned long long key = hs.bad_key;
    if (key != ~0ULL) {
        g_noalloc_err = "pivot failed at level " + std::to_string(key >> 40) + ", block " +
                        std::to_string(key & ((1ULL << 40) - 1));
        return BSS_ERR_NOT_SPD;
    }
    return BSS_OK;
}

}  // namespace

extern "C" int bss_factor_solve_noalloc(int64_t N, int64_t n, int64_t k, int32_t dtype, void *A, void *B, void *d,
                                        void *stream)
{
    if (N < 1 || n < 1 || k < 1 || !A || !d || (N > 1 && !B)) {
        set_last_error("bss_factor_solve_noalloc: bad argument");
        return BSS_ERR_ARG;
    }
    // range checks before the narrowing casts below: block indices are
    // reported in 40 bits, n and k are int in the kernels
    if (N >= (1LL << 40) || k > 0x7FFFFFFFLL) {
        set_last_error("bss_factor_solve_noalloc: N=" + std::to_string(N) + " or k=" + std::to_string(k) +
                       " out of range");
        return BSS_ERR_ARG;
    }
    if (n > MAX_WIDE_N || tile_for((int)n) == 0) {
        set_last_error("bss_factor_solve_noalloc: block size n=" + std::to_string(n) + " is not supported");
        return BSS_ERR_UNSUPPORTED;
    }
    cudaStream_t s = (cudaStream_t)stream;
    int rc;
    if (dtype == BSS_F64)
        rc = run<double>(N, (int)n, (int)k, (double *)A, (double *)B, (double *)d, s);
    else if (dtype == BSS_F32)
        rc = run<float>(N, (int)n, (int)k, (float *)A, (float *)B, (float *)d, s);
    else {
        g_noalloc_err = "bss_factor_solve_noalloc: dtype must be BSS_F32 or BSS_F64";
        rc = BSS_ERR_ARG;
    }
    if (rc != BSS_OK) set_last_error(g_noalloc_err);
    return rc;
}
