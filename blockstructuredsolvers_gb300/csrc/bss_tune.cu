// Autotuner of the chain kernel and the recursion plan per (n, dtype,
// precision).  Kernel: for FP32 factors of 33..64-wide blocks, the
// tensor-core chain kernel (one 128-row tcgen05 tile, bulk-copied block
// tiles, 100 KB of shared memory per CTA) or the CUDA-core one (4 x 4
// register tiles over 256 threads, 105 KB).  Plan: how many partitions the
// finest level gets (in units of one wave of resident CTAs of the chosen
// kernel), where the halving levels stop (the sequential cutoff), and, for
// many-system batches, the chain length per partition.  The tuner times
// factorize+solve of a device-generated SPD system for each candidate with
// CUDA events and keeps the fastest; results live in a process-wide table
// (consulted by the planners whenever the caller leaves the corresponding
// option at 0) and can be saved to / loaded from a text file.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdio>
#include <cstring>
#include <map>
#include <mutex>
#include <tuple>
#include <vector>

#include "bss_internal.h"

using namespace bss;

namespace {

std::mutex g_tune_mu;
std::map<std::tuple<int, int, int>, bss_tune_entry> g_tune;

// splitmix64 -> uniform in [-1, 1)
__device__ __forceinline__ double hash_unit(unsigned long long x)
{
    x += 0x9E3779B97F4A7C15ULL;
    x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ULL;
    x = (x ^ (x >> 27)) * 0x94D049BB133111EBULL;
    x ^= x >> 31;
    return (double)(x >> 11) * (2.0 / 9007199254740992.0) - 1.0;
}

// A_i = 4n I + sym(0.5 U), B_i = U' (U, U' uniform in [-1, 1)): strictly
// diagonally dominant (row sums of |off-diagonal| < 3n), hence SPD
template <class T>
__global__ void tune_gen_kernel(T *A, T *B, T *d, long long N, int n, int k, unsigned long long seed)
{
    const long long nn = (long long)n * n;
    const long long tA = N * nn, tB = (N - 1) * nn, tD = N * n * k;
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < tA + tB + tD;
         e += (long long)gridDim.x * blockDim.x) {
        if (e < tA) {
            const long long i = e / nn, q = e - i * nn;
            const int r = (int)(q % n), c = (int)(q / n);
            const int lo = r < c ? r : c, hi = r < c ? c : r;
            const double u = hash_unit(seed ^ (unsigned long long)(i * nn + lo + (long long)hi * n));
            A[e] = (T)((r == c ? 4.0 * n : 0.0) + 0.5 * u);
        } else if (e < tA + tB) {
            B[e - tA] = (T)hash_unit(seed * 31 + (unsigned long long)e);
        } else {
            d[e - tA - tB] = (T)hash_unit(seed * 77 + (unsigned long long)e);
        }
    }
}

template <class T>
cudaError_t tune_fill(void *A, void *B, void *d, long long N, int n, int k, cudaStream_t s)
{
    tune_gen_kernel<T><<<152 * 8, 256, 0, s>>>((T *)A, (T *)B, (T *)d, N, n, k, 12345ULL);
    count_launch();
    return cudaGetLastError();
}

// median ms of factorize+solve of one handle (inputs refilled before each rep)
int time_handle(long long N, int n, int dtype, const bss_options &o, int reps, double *ms)
{
    bss_handle *h = nullptr;
    cudaStream_t s;
    BSS_CUDA(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking));
    int rc = bss_create_batched(N, n, 1, dtype, s, &o, &h);
    if (rc) {
        cudaStreamDestroy(s);
        return rc;
    }
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    std::vector<float> ts;
    for (int r = 0; r <= reps && rc == BSS_OK; ++r) {
        void *A, *B, *d;
        bss_get_tensors(h, &A, &B, &d);
        long long Nu = 0;
        int64_t Nq = 0;
        bss_get_dims(h, &Nq, nullptr, nullptr, nullptr);
        Nu = Nq;
        const cudaError_t ge = dtype == BSS_F64 ? tune_fill<double>(A, B, d, Nu, n, 1, s)
                                                : tune_fill<float>(A, B, d, Nu, n, 1, s);
        if (ge != cudaSuccess) {
            rc = cuda_fail(ge, "tune_fill");
            break;
        }
        cudaEventRecord(e0, s);
        rc = bss_factorize(h);
        if (rc == BSS_OK) rc = bss_solve(h);
        cudaEventRecord(e1, s);
        const int sr = bss_synchronize(h);
        if (rc == BSS_OK && sr != BSS_OK && sr != BSS_ERR_NOT_CONVERGED) rc = sr;
        float t = 0.f;
        cudaEventElapsedTime(&t, e0, e1);
        if (r > 0) ts.push_back(t);  // the first call runs eagerly and captures nothing yet
    }
    bss_destroy(h);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaStreamDestroy(s);
    if (rc) return rc;
    std::sort(ts.begin(), ts.end());
    *ms = ts.empty() ? 0.0 : ts[ts.size() / 2];
    return BSS_OK;
}

// median ms of factorize+solve of a batch of `nsys` systems of N blocks
int time_batch(int nsys, long long N, int n, int dtype, const bss_options &o, int reps, double *ms)
{
    std::vector<int64_t> Ns(nsys, N), ns(nsys, n), ks(nsys, 1);
    cudaStream_t s;
    BSS_CUDA(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking));
    bss_batch *b = nullptr;
    int rc = bss_batch_create(nsys, Ns.data(), ns.data(), ks.data(), dtype, s, &o, &b);
    if (rc) {
        cudaStreamDestroy(s);
        return rc;
    }
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    std::vector<float> ts;
    for (int r = 0; r <= reps && rc == BSS_OK; ++r) {
        for (int i = 0; i < nsys && rc == BSS_OK; ++i) {
            void *A, *B, *d;
            bss_batch_get_tensors(b, i, &A, &B, &d);
            const cudaError_t ge = dtype == BSS_F64 ? tune_fill<double>(A, B, d, N, n, 1, s)
                                                    : tune_fill<float>(A, B, d, N, n, 1, s);
            if (ge != cudaSuccess) rc = cuda_fail(ge, "tune_fill");
        }
        if (rc) break;
        cudaEventRecord(e0, s);
        rc = bss_batch_factorize(b);
        if (rc == BSS_OK) rc = bss_batch_solve(b);
        cudaEventRecord(e1, s);
        const int sr = bss_batch_synchronize(b);
        if (rc == BSS_OK && sr != BSS_OK && sr != BSS_ERR_NOT_CONVERGED) rc = sr;
        float t = 0.f;
        cudaEventElapsedTime(&t, e0, e1);
        if (r > 0) ts.push_back(t);
    }
    bss_batch_destroy(b);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaStreamDestroy(s);
    if (rc) return rc;
    std::sort(ts.begin(), ts.end());
    *ms = ts.empty() ? 0.0 : ts[ts.size() / 2];
    return BSS_OK;
}

}  // namespace

bool bss::tuned_plan(int n, int dtype, int precision, bss_tune_entry *out)
{
    std::lock_guard<std::mutex> lk(g_tune_mu);
    auto it = g_tune.find(std::make_tuple(n, dtype, precision));
    if (it == g_tune.end()) return false;
    if (out) *out = it->second;
    return true;
}

extern "C" int bss_autotune(int64_t n, int32_t dtype, int32_t precision, int64_t N_probe, bss_tune_entry *out)
{
    if (n < 1 || tile_for((int)n) == 0 || (dtype != BSS_F32 && dtype != BSS_F64) ||
        (precision != BSS_PRECISION_PLAIN && precision != BSS_PRECISION_MIXED) ||
        (precision == BSS_PRECISION_MIXED && dtype != BSS_F64))
        return fail(BSS_ERR_ARG, "bss_autotune: bad (n, dtype, precision)");
    if (N_probe <= 0) N_probe = 16384;
    bss_tune_entry best{};
    best.n = (int32_t)n;
    best.dtype = dtype;
    best.precision = precision;
    // single system: partitions per wave x cutoff
    const int mults4[] = {2, 4, 8, 16};  // wave multiplier x 4: 0.5, 1, 2, 4
    std::vector<int> cutoffs = precision == BSS_PRECISION_MIXED ? std::vector<int>{2, 3, 4}
                                                                : std::vector<int>{2, 4, 8, 16};
    double best_ms = 1e300;
    int sms = 152, dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    const int t0 = precision == BSS_PRECISION_MIXED ? BSS_F32 : dtype;
    // kernel variants worth timing: FP32 factors of 33..64-wide and of
    // 65..128-wide blocks have two chain kernels each
    std::vector<int> variants{0};
    if (t0 == BSS_F32 && tile_for((int)n) == 64) variants = {0, FACTOR_FMA_CHAIN};
    if (t0 == BSS_F32 && tile_for((int)n) == WIDE_CLASS && n <= 128) variants = {0, FACTOR_WIDE_L2};
    // candidates run with the process-wide default variant set to theirs and
    // no table entry for this key (the default is restored afterwards)
    const int saved_default = default_factor_variant();
    {
        std::lock_guard<std::mutex> lk(g_tune_mu);
        g_tune.erase(std::make_tuple((int)n, (int)dtype, (int)precision));
    }
    int rc_all = BSS_OK;
    for (int v : variants) {
        set_default_factor_variant(v);
        int ctas = 1;
        if (dtype == BSS_F64 && t0 == BSS_F32)
            ctas = chain_factor_ctas_per_sm<double, float>((int)n, v);
        else if (t0 == BSS_F32)
            ctas = chain_factor_ctas_per_sm<float, float>((int)n, v);
        else
            ctas = chain_factor_ctas_per_sm<double, double>((int)n, v);
        for (int m4 : mults4)
            for (int c : cutoffs) {
                if (rc_all) break;
                bss_options o;
                bss_default_options(&o);
                o.precision = precision;
                o.target_partitions = std::max(1, (sms * ctas * m4) / 4);
                o.seq_cutoff = c;
                double ms = 0.0;
                rc_all = time_handle(N_probe, (int)n, dtype, o, 3, &ms);
                if (rc_all == BSS_OK && ms < best_ms) {
                    best_ms = ms;
                    best.wave_mult_x4 = m4;
                    best.seq_cutoff = c;
                    best.factor_variant = v;
                }
            }
    }
    if (rc_all) {
        set_default_factor_variant(saved_default);
        return rc_all;
    }
    best.single_ms = best_ms;
    // batch: chain length per partition (256 systems of 512 blocks)
    set_default_factor_variant(best.factor_variant);  // the batch runs with the winner's kernel
    const int chains[] = {16, 32, 64, 128, 256};
    double best_b = 1e300;
    for (int ch : chains) {
        bss_options o;
        bss_default_options(&o);
        o.precision = precision;
        o.chain_blocks = ch;
        double ms = 0.0;
        const int rc = time_batch(256, 512, (int)n, dtype, o, 2, &ms);
        if (rc) {
            set_default_factor_variant(saved_default);
            return rc;
        }
        if (ms < best_b) {
            best_b = ms;
            best.chain_blocks = ch;
        }
    }
    set_default_factor_variant(saved_default);
    best.batch_ms = best_b;
    {
        std::lock_guard<std::mutex> lk(g_tune_mu);
        g_tune[std::make_tuple((int)n, (int)dtype, (int)precision)] = best;
    }
    if (out) *out = best;
    return BSS_OK;
}

extern "C" int bss_autotune_lookup(int64_t n, int32_t dtype, int32_t precision, bss_tune_entry *out)
{
    if (!tuned_plan((int)n, dtype, precision, out)) return fail(BSS_ERR_STATE, "no tuned plan for this key");
    return BSS_OK;
}

extern "C" void bss_autotune_clear(void)
{
    std::lock_guard<std::mutex> lk(g_tune_mu);
    g_tune.clear();
}

extern "C" int bss_autotune_save(const char *path)
{
    if (!path) return fail(BSS_ERR_ARG, "path is NULL");
    FILE *f = std::fopen(path, "w");
    if (!f) return fail(BSS_ERR_ARG, std::string("cannot write ") + path);
    std::lock_guard<std::mutex> lk(g_tune_mu);
    std::fprintf(f, "# n dtype precision wave_mult_x4 seq_cutoff chain_blocks single_ms batch_ms factor_variant\n");
    for (auto &kv : g_tune) {
        const bss_tune_entry &e = kv.second;
        std::fprintf(f, "%d %d %d %d %d %d %.17g %.17g %d\n", e.n, e.dtype, e.precision, e.wave_mult_x4, e.seq_cutoff,
                     e.chain_blocks, e.single_ms, e.batch_ms, e.factor_variant);
    }
    std::fclose(f);
    return BSS_OK;
}

extern "C" int bss_autotune_load(const char *path)
{
    if (!path) return fail(BSS_ERR_ARG, "path is NULL");
    FILE *f = std::fopen(path, "r");
    if (!f) return fail(BSS_ERR_ARG, std::string("cannot read ") + path);
    char line[512];
    int loaded = 0;
    std::lock_guard<std::mutex> lk(g_tune_mu);
    while (std::fgets(line, sizeof line, f)) {
        if (line[0] == '#') continue;
        bss_tune_entry e{};
        // 9 columns; files written before the variant column have 8 (variant 0)
        const int got = std::sscanf(line, "%d %d %d %d %d %d %lf %lf %d", &e.n, &e.dtype, &e.precision,
                                    &e.wave_mult_x4, &e.seq_cutoff, &e.chain_blocks, &e.single_ms, &e.batch_ms,
                                    &e.factor_variant);
        if (got == 8) e.factor_variant = 0;
        if ((got == 8 || got == 9) && e.n > 0 && e.wave_mult_x4 > 0 && e.seq_cutoff > 0 && e.chain_blocks > 0 &&
            e.factor_variant >= 0 && (e.factor_variant & ~FACTOR_VARIANTS) == 0) {
            g_tune[std::make_tuple(e.n, e.dtype, e.precision)] = e;
            ++loaded;
        }
    }
    std::fclose(f);
    return loaded > 0 ? BSS_OK : fail(BSS_ERR_ARG, "no entries in the tuning file");
}
