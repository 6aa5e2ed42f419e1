// Internal launcher interface between the C-ABI host code (bss_api.cu) and
// the kernel translation units (k_*.cu).  Not part of the public ABI.
#pragma once

#include <cuda_runtime.h>

#include <string>

#include "bss_kernels.cuh"

namespace bss {

// largest block size the fused chain kernel handles in one CTA; larger
// blocks (up to MAX_WIDE_N) take the wide, tile-streamed path
constexpr int MAX_FUSED_N = 64;
constexpr int MAX_WIDE_N = 1024;
constexpr int WIDE_CLASS = 128;  // tile_for() code of the wide path

int tile_for(int n);  // NB in {16, 32, 64}, WIDE_CLASS, or 0 if unsupported

template <class Tin, class T>
cudaError_t launch_chain_factor(const ChainFactorArgs<Tin, T> &a, cudaStream_t s);
template <class Tin, class T>
int chain_factor_ctas_per_sm(int n, int variant);

// FACTOR_* variant bits that handles take when the autotuner has no entry
// for their (n, dtype, precision); process-wide
int default_factor_variant();
void set_default_factor_variant(int v);

template <class Tsrc, class T, class Tdst>
cudaError_t launch_assemble_schur(const Tsrc *A_src, const T *C, Tdst *A_next, Tdst *B_next, long long N,
                                  long long Q, int n, cudaStream_t s);

template <class T>
cudaError_t launch_chain_fwd(const SolveArgs<T> &a, cudaStream_t s);
template <class T, class Tsep>
cudaError_t launch_chain_bwd(const SolveArgs<T> &a, cudaStream_t s);
template <class T, class Tn>
cudaError_t launch_assemble_rhs(const T *d, const T *bvec, Tn *dn, long long N, long long Q, int n, int k, int j0,
                                int kc, cudaStream_t s);

template <class T>
cudaError_t launch_opnorm(const T *A, const T *B, long long N, int n, DevStatus *st, cudaStream_t s);
template <class T>
cudaError_t launch_absmax(const T *v, long long count, unsigned long long *dst, cudaStream_t s);
template <class T, class Tr>
cudaError_t launch_residual(const T *A, const T *B, const T *x, const T *d, Tr *r, long long N, int n, int k,
                            int with_norm, DevStatus *st, cudaStream_t s);
// the refinement residual of FP64 systems in double-float on the FP32 pipe
// (residual_df_kernel); same arguments as launch_residual<double, Tr>
template <class Tr>
cudaError_t launch_residual_df(const double *A, const double *B, const double *x, const double *d, Tr *r,
                               long long N, int n, int k, int with_norm, DevStatus *st, cudaStream_t s);
cudaError_t launch_relres(DevStatus *st, double tol, cudaStream_t s);
cudaError_t launch_relres_control(DevStatus *st, double tol, int max_refine, cudaGraphConditionalHandle hloop,
                                  cudaGraphConditionalHandle hcorr, cudaStream_t s);
template <class Tc>
cudaError_t launch_update(double *x, const Tc *c, long long count, int assign, cudaStream_t s);
template <class Ts, class Td>
cudaError_t launch_convert(Td *dst, const Ts *src, long long count, cudaStream_t s);
template <class T>
cudaError_t launch_init_identity(T *A, long long first_blk, long long last_blk, int n, cudaStream_t s);

int solve_kc_max(int n, int k, int elem_bytes);

// resident CTAs per SM of a kernel: the larger of the occupancy query and
// the count from its registers and shared memory (the query reports one CTA
// per SM for the tensor-core wide kernel although its resources admit two)
template <class K>
inline int ctas_per_sm(K kern, int threads, size_t smem)
{
    int nblk = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nblk, kern, threads, smem) != cudaSuccess) nblk = 1;
    int dev = 0, smem_sm = 0, reserved = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&smem_sm, cudaDevAttrMaxSharedMemoryPerMultiprocessor, dev);
    cudaDeviceGetAttribute(&reserved, cudaDevAttrReservedSharedMemoryPerBlock, dev);
    cudaFuncAttributes fa{};
    if (cudaFuncGetAttributes(&fa, kern) == cudaSuccess && fa.numRegs > 0) {
        const int by_smem = smem_sm / (int)(smem + fa.sharedSizeBytes + reserved);
        const int by_regs = 65536 / (fa.numRegs * threads);
        const int by_res = by_smem < by_regs ? by_smem : by_regs;
        if (by_res > nblk) nblk = by_res;
    }
    return nblk > 0 ? nblk : 1;
}

// message returned by bss_last_error_string() on this host thread
void set_last_error(const std::string &msg);

// process-wide count of kernels this library launched (all handles)
void count_launch();
void count_launches(long long n);  // kernels run by a graph replay
long long launch_count();

}  // namespace bss
