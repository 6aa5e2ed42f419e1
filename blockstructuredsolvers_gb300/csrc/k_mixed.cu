// Kernel instantiations that cross precisions: FP32 factorization reading
// FP64 tensors, FP64 residuals written as FP32 corrections, conversions.
#include <atomic>

#include "bss_launch_impl.cuh"

namespace bss {
template cudaError_t launch_chain_factor<double, float>(const ChainFactorArgs<double, float> &, cudaStream_t);
template int chain_factor_ctas_per_sm<double, float>(int, int);
template cudaError_t launch_assemble_schur<double, float, float>(const double *, const float *, float *, float *,
                                                                 long long, long long, int, cudaStream_t);
template cudaError_t launch_assemble_schur<double, float, double>(const double *, const float *, double *,
                                                                  double *, long long, long long, int,
                                                                  cudaStream_t);
template cudaError_t launch_residual<double, float>(const double *, const double *, const double *,
                                                    const double *, float *, long long, int, int, int, DevStatus *,
                                                    cudaStream_t);
template cudaError_t launch_residual_df<float>(const double *, const double *, const double *, const double *,
                                               float *, long long, int, int, int, DevStatus *, cudaStream_t);
template cudaError_t launch_residual_df<double>(const double *, const double *, const double *, const double *,
                                                double *, long long, int, int, int, DevStatus *, cudaStream_t);
template cudaError_t launch_convert<double, float>(float *, const double *, long long, cudaStream_t);
template cudaError_t launch_convert<double, double>(double *, const double *, long long, cudaStream_t);
template cudaError_t launch_convert<float, float>(float *, const float *, long long, cudaStream_t);

static std::atomic<long long> g_launches{0};
void count_launch() { g_launches.fetch_add(1, std::memory_order_relaxed); }
void count_launches(long long n) { g_launches.fetch_add(n, std::memory_order_relaxed); }
long long launch_count() { return g_launches.load(std::memory_order_relaxed); }

cudaError_t launch_relres(DevStatus *st, double tol, cudaStream_t s)
{
    relres_kernel<<<1, 32, 0, s>>>(st, tol);
    count_launch();
    return cudaGetLastError();
}

cudaError_t launch_relres_control(DevStatus *st, double tol, int max_refine, cudaGraphConditionalHandle hloop,
                                  cudaGraphConditionalHandle hcorr, cudaStream_t s)
{
    relres_control_kernel<<<1, 32, 0, s>>>(st, tol, max_refine, hloop, hcorr);
    count_launch();
    return cudaGetLastError();
}

static std::atomic<int> g_factor_variant{0};
int default_factor_variant() { return g_factor_variant.load(std::memory_order_relaxed); }
void set_default_factor_variant(int v) { g_factor_variant.store(v & FACTOR_VARIANTS); }

int tile_for(int n)
{
    if (n <= 0) return 0;
    if (n <= 16) return 16;
    if (n <= 32) return 32;
    if (n <= 64) return 64;
    if (n <= MAX_WIDE_N) return WIDE_CLASS;
    return 0;
}

int solve_kc_max(int n, int k, int elem_bytes)
{
    // largest column chunk (<= 32) whose solve kernels fit in shared memory:
    // in the staged form when that fits for one column, else reading the
    // blocks from global memory (the launch picks the staged form whenever
    // it fits the chunk, for levels of either precision)
    const bool staged = elem_bytes == 8 ? solve_staged<double>(n, 1) : solve_staged<float>(n, 1);
    int best = 1;
    for (int kc = 1; kc <= 32 && kc <= k; ++kc) {
        const size_t need = elem_bytes == 8 ? solve_smem_bytes<double>(n, kc, staged)
                                            : solve_smem_bytes<float>(n, kc, staged);
        if (need > SOLVE_SMEM_MAX) break;
        best = kc;
    }
    return best;
}
}  // namespace bss
