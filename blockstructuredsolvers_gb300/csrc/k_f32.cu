// Kernel instantiations: FP32 factor/solve (plain FP32 and the FP32 levels of
// the mixed-precision path).
#include "bss_launch_impl.cuh"

namespace bss {
template cudaError_t launch_chain_factor<float, float>(const ChainFactorArgs<float, float> &, cudaStream_t);
template int chain_factor_ctas_per_sm<float, float>(int, int);
template cudaError_t launch_assemble_schur<float, float, float>(const float *, const float *, float *, float *,
                                                                long long, long long, int, cudaStream_t);
template cudaError_t launch_assemble_schur<float, float, double>(const float *, const float *, double *, double *,
                                                                 long long, long long, int, cudaStream_t);
template cudaError_t launch_chain_fwd<float>(const SolveArgs<float> &, cudaStream_t);
template cudaError_t launch_chain_bwd<float, float>(const SolveArgs<float> &, cudaStream_t);
template cudaError_t launch_chain_bwd<float, double>(const SolveArgs<float> &, cudaStream_t);
template cudaError_t launch_assemble_rhs<float, float>(const float *, const float *, float *, long long, long long,
                                                       int, int, int, int, cudaStream_t);
template cudaError_t launch_assemble_rhs<float, double>(const float *, const float *, double *, long long,
                                                        long long, int, int, int, int, cudaStream_t);
template cudaError_t launch_opnorm<float>(const float *, const float *, long long, int, DevStatus *, cudaStream_t);
template cudaError_t launch_absmax<float>(const float *, long long, unsigned long long *, cudaStream_t);
template cudaError_t launch_residual<float, float>(const float *, const float *, const float *, const float *,
                                                   float *, long long, int, int, int, DevStatus *, cudaStream_t);
template cudaError_t launch_update<float>(double *, const float *, long long, int, cudaStream_t);
template cudaError_t launch_convert<float, double>(double *, const float *, long long, cudaStream_t);
template cudaError_t launch_init_identity<float>(float *, long long, long long, int, cudaStream_t);
}  // namespace bss
