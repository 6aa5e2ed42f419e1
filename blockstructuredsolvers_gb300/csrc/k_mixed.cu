// Kernel instantiations that cross precisions: FP32 factorization reading
// FP64 tensors, FP64 residuals written as FP32 corrections, conversions.
#include "bss_launch_impl.cuh"

namespace bss {
template cudaError_t launch_chain_factor<double, float>(const ChainFactorArgs<double, float> &, cudaStream_t);
template int chain_factor_ctas_per_sm<double, float>(int);
template cudaError_t launch_assemble_schur<double, float, float>(const double *, const float *, float *, float *,
                                                                 long long, long long, int, cudaStream_t);
template cudaError_t launch_assemble_schur<double, float, double>(const double *, const float *, double *,
                                                                  double *, long long, long long, int,
                                                                  cudaStream_t);
template cudaError_t launch_residual<double, float>(const double *, const double *, const double *,
                                                    const double *, float *, long long, int, int, DevStatus *,
                                                    cudaStream_t);
template cudaError_t launch_convert<double, float>(float *, const double *, long long, cudaStream_t);
template cudaError_t launch_convert<double, double>(double *, const double *, long long, cudaStream_t);
template cudaError_t launch_convert<float, float>(float *, const float *, long long, cudaStream_t);

cudaError_t launch_relres(DevStatus *st, double tol, cudaStream_t s)
{
    relres_kernel<<<1, 32, 0, s>>>(st, tol);
    return cudaGetLastError();
}

int tile_for(int n)
{
    if (n <= 0) return 0;
    if (n <= 16) return 16;
    if (n <= 32) return 32;
    if (n <= 64) return 64;
    return 0;
}

int solve_kc_max(int n, int k, int elem_bytes)
{
    const long long budget = 200 * 1024;
    long long kc = (budget / elem_bytes - 3LL * n * n) / (5LL * n);
    if (kc > 32) kc = 32;
    if (kc > k) kc = k;
    if (kc < 1) kc = 1;
    return (int)kc;
}
}  // namespace bss
