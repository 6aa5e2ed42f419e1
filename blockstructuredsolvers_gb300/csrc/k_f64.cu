// Kernel instantiations: FP64 factor/solve (the plain FP64 path).
#include "bss_launch_impl.cuh"

namespace bss {
template cudaError_t launch_chain_factor<double, double>(const ChainFactorArgs<double, double> &, cudaStream_t);
template int chain_factor_ctas_per_sm<double, double>(int, int);
template cudaError_t launch_assemble_schur<double, double, double>(const double *, const double *, double *,
                                                                   double *, long long, long long, int,
                                                                   cudaStream_t);
template cudaError_t launch_chain_fwd<double>(const SolveArgs<double> &, cudaStream_t);
template cudaError_t launch_chain_bwd<double, double>(const SolveArgs<double> &, cudaStream_t);
template cudaError_t launch_assemble_rhs<double, double>(const double *, const double *, double *, long long,
                                                         long long, int, int, int, int, cudaStream_t);
template cudaError_t launch_opnorm<double>(const double *, const double *, long long, int, DevStatus *,
                                           cudaStream_t);
template cudaError_t launch_absmax<double>(const double *, long long, unsigned long long *, cudaStream_t);
template cudaError_t launch_residual<double, double>(const double *, const double *, const double *,
                                                     const double *, double *, long long, int, int, int, DevStatus *,
                                                     cudaStream_t);
template cudaError_t launch_update<double>(double *, const double *, long long, int, cudaStream_t);
template cudaError_t launch_init_identity<double>(double *, long long, long long, int, cudaStream_t);
}  // namespace bss
