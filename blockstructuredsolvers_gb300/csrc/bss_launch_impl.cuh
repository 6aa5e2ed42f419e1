// Launcher definitions, included by the per-dtype kernel translation units.
#pragma once

#include <cstring>

#include "bss_launch.h"

namespace bss {

inline int grid_for(long long work, int threads, int cap = 152 * 16)
{
    long long g = (work + threads - 1) / threads;
    if (g < 1) g = 1;
    if (g > cap) g = cap;
    return (int)g;
}

// partitioned levels of 64-wide blocks with FP32 factors: the tensor-core
// chain kernel (bss_chain64_tc.cuh), unless the CUDA-core variant is chosen
template <class Tin>
static cudaError_t chain64_tc(const ChainFactorArgs<Tin, float> &a, cudaStream_t s)
{
    const size_t smem = chain64_tc_smem();
    auto kern = chain64_tc_kernel<Tin>;
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    cudaFuncSetAttribute(kern, cudaFuncAttributePreferredSharedMemoryCarveout, 100);
    kern<<<(unsigned)a.Q, C64_THREADS, smem, s>>>(a);
    count_launch();
    return cudaGetLastError();
}

template <class Tin, class T, int NB>
static cudaError_t chain_factor_nb(const ChainFactorArgs<Tin, T> &a, cudaStream_t s)
{
    if constexpr (std::is_same<T, float>::value && NB == 64) {
        if (!a.seq && !(a.variant & FACTOR_FMA_CHAIN)) return chain64_tc<Tin>(a, s);
    }
    const size_t smem = chain_factor_smem<T, NB>();
    auto kern = chain_factor_kernel<Tin, T, NB>;
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    const unsigned grid = a.seq ? 1u : (unsigned)a.Q;
    kern<<<grid, Tile<NB>::THREADS, smem, s>>>(a);
    count_launch();
    return cudaGetLastError();
}

template <class Tin, class T, bool TC>
static cudaError_t wide_chain_factor_tc(const ChainFactorArgs<Tin, T> &a, cudaStream_t s)
{
    const size_t smem = wide_factor_smem<T, TC>();
    auto kern = wide_chain_factor_kernel<Tin, T, TC>;
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    cudaFuncSetAttribute(kern, cudaFuncAttributePreferredSharedMemoryCarveout, 100);
    const unsigned grid = a.seq ? 1u : (unsigned)a.Q;
    kern<<<grid, WIDE_THREADS, smem, s>>>(a);
    count_launch();
    return cudaGetLastError();
}

// partitioned levels of 65..128-wide blocks with FP32 factors: the chain
// kernel that keeps a step on chip (bss_chain128_tc.cuh), unless the
// L2-staged wide kernel is chosen
template <class Tin>
static bool use_chain128(const ChainFactorArgs<Tin, float> &a)
{
    return !a.seq && a.n <= 128 && !(a.variant & FACTOR_WIDE_L2);
}

// tensor map of a level's B blocks for chain128_tc_kernel: a 2D FP64 tensor
// of n rows x (N - 1) n columns (column stride n * 8 bytes), boxes of 16 rows
// x 128 columns, 128-byte swizzle, zero fill outside; L2 fills of 128 bytes
// (a box row is 128 bytes: a wider fill would fetch rows the next chunk
// reads only later).  False (the kernel then
// reads B with plain loads) when the layout does not qualify or the driver
// entry point is missing.
template <class Tin>
bool chain128_tmap_b(const ChainFactorArgs<Tin, float> &a, CUtensorMap *map)
{
    std::memset(map, 0, sizeof(*map));
    if (sizeof(Tin) != 8 || a.n % 2 != 0 || a.N < 2 || ((uintptr_t)a.B_in % 16u) != 0) return false;
    using Encode = CUresult (*)(CUtensorMap *, CUtensorMapDataType, cuuint32_t, void *, const cuuint64_t *,
                                const cuuint64_t *, const cuuint32_t *, const cuuint32_t *, CUtensorMapInterleave,
                                CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);
    static Encode encode = []() -> Encode {
        void *fn = nullptr;
        cudaDriverEntryPointQueryResult q{};
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &fn, 12000, cudaEnableDefault, &q) !=
                cudaSuccess ||
            q != cudaDriverEntryPointSuccess)
            return nullptr;
        return reinterpret_cast<Encode>(fn);
    }();
    if (!encode) return false;
    const cuuint64_t dims[2] = {(cuuint64_t)a.n, (cuuint64_t)(a.N - 1) * (cuuint64_t)a.n};
    const cuuint64_t strides[1] = {(cuuint64_t)a.n * sizeof(Tin)};
    const cuuint32_t box[2] = {16u, 128u};
    const cuuint32_t estr[2] = {1u, 1u};
    return encode(map, CU_TENSOR_MAP_DATA_TYPE_FLOAT64, 2, const_cast<Tin *>(a.B_in), dims, strides, box, estr,
                  CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
                  CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

template <class Tin>
static cudaError_t chain128_tc(const ChainFactorArgs<Tin, float> &a, cudaStream_t s)
{
    const size_t smem = chain128_tc_smem();
    CUtensorMap tmB;
    const int tma_b = chain128_tmap_b<Tin>(a, &tmB) ? 1 : 0;
    auto kern = chain128_tc_kernel<Tin>;
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    cudaFuncSetAttribute(kern, cudaFuncAttributePreferredSharedMemoryCarveout, 100);
    int dev = 0, sms = 1;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    const unsigned grid = (unsigned)(a.Q < sms ? a.Q : sms);  // one CTA per SM walks several partitions
    kern<<<grid, C128_THREADS, smem, s>>>(a, tmB, tma_b);
    count_launch();
    return cudaGetLastError();
}

template <class Tin, class T>
static cudaError_t wide_chain_factor(const ChainFactorArgs<Tin, T> &a, cudaStream_t s)
{
    if constexpr (std::is_same<T, float>::value) {
        if (use_chain128<Tin>(a)) return chain128_tc<Tin>(a, s);
        if (wide_uses_tc<T>(a.n)) return wide_chain_factor_tc<Tin, T, true>(a, s);
    }
    return wide_chain_factor_tc<Tin, T, false>(a, s);
}

template <class Tin, class T>
cudaError_t launch_chain_factor(const ChainFactorArgs<Tin, T> &a, cudaStream_t s)
{
    switch (tile_for(a.n)) {
    case 16: return chain_factor_nb<Tin, T, 16>(a, s);
    case 32: return chain_factor_nb<Tin, T, 32>(a, s);
    case 64: return chain_factor_nb<Tin, T, 64>(a, s);
    case WIDE_CLASS: return wide_chain_factor<Tin, T>(a, s);
    default: return cudaErrorInvalidValue;
    }
}

template <class Tin, class T, int NB>
static int ctas_nb(int variant)
{
    if constexpr (std::is_same<T, float>::value && NB == 64) {
        if (!(variant & FACTOR_FMA_CHAIN)) {
            const size_t smem = chain64_tc_smem();
            auto kern = chain64_tc_kernel<Tin>;
            if (cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) != cudaSuccess)
                return 1;
            cudaFuncSetAttribute(kern, cudaFuncAttributePreferredSharedMemoryCarveout, 100);
            return ctas_per_sm(kern, C64_THREADS, smem);
        }
    }
    const size_t smem = chain_factor_smem<T, NB>();
    auto kern = chain_factor_kernel<Tin, T, NB>;
    if (cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) != cudaSuccess) return 1;
    int nblk = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nblk, kern, Tile<NB>::THREADS, smem) != cudaSuccess) return 1;
    return nblk > 0 ? nblk : 1;
}

template <class Tin, class T, bool TC>
static int wide_ctas_tc()
{
    const size_t smem = wide_factor_smem<T, TC>();
    auto kern = wide_chain_factor_kernel<Tin, T, TC>;
    if (cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) != cudaSuccess) return 1;
    // ask for the whole unified L1/shared array as shared memory
    cudaFuncSetAttribute(kern, cudaFuncAttributePreferredSharedMemoryCarveout, 100);
    return ctas_per_sm(kern, WIDE_THREADS, smem);
}

template <class Tin, class T>
int chain_factor_ctas_per_sm(int n, int variant)
{
    switch (tile_for(n)) {
    case 16: return ctas_nb<Tin, T, 16>(variant);
    case 32: return ctas_nb<Tin, T, 32>(variant);
    case 64: return ctas_nb<Tin, T, 64>(variant);
    case WIDE_CLASS:
        if constexpr (std::is_same<T, float>::value) {
            // the on-chip kernel runs one CTA per SM over several partitions
            // each; the partitions are sized for the level's solve sweeps,
            // which run two CTAs per SM
            if (n <= 128 && !(variant & FACTOR_WIDE_L2)) return 2;
            if (wide_uses_tc<T>(n)) return wide_ctas_tc<Tin, T, true>();
        }
        return wide_ctas_tc<Tin, T, false>();
    default: return 1;
    }
}

template <class Tsrc, class T, class Tdst>
cudaError_t launch_assemble_schur(const Tsrc *A_src, const T *C, Tdst *A_next, Tdst *B_next, long long N,
                                  long long Q, int n, cudaStream_t s)
{
    const long long work = (2 * Q + 1) * (long long)n * n;
    assemble_schur_kernel<Tsrc, T, Tdst><<<grid_for(work, 256), 256, 0, s>>>(A_src, C, A_next, B_next, N, Q, n);
    count_launch();
    return cudaGetLastError();
}

template <class T>
static cudaError_t set_solve_smem(const void *kern, size_t smem)
{
    return cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
}

// the streamed sweeps need 16-byte aligned blocks and right-hand sides
template <class T>
static bool stream_aligned(const SolveArgs<T> &a)
{
    const uintptr_t m = (uintptr_t)a.Af | (uintptr_t)a.Bf | (uintptr_t)a.Y | (uintptr_t)a.d;
    return (m & 15u) == 0 && ((size_t)a.n * sizeof(T)) % 16 == 0;
}

template <class T>
cudaError_t launch_chain_fwd(const SolveArgs<T> &a, cudaStream_t s)
{
    if (!a.seq && solve_streamed<T>(a.n, a.kc) && stream_aligned(a)) {
        const size_t smem = stream_smem_bytes<T>(a.n, a.kc);
        auto kern = chain_fwd_stream_kernel<T>;
        cudaError_t e = set_solve_smem<T>((const void *)kern, smem);
        if (e != cudaSuccess) return e;
        kern<<<(unsigned)a.Q, SOLVE_THREADS, smem, s>>>(a);
        count_launch();
        return cudaGetLastError();
    }
    const bool staged = solve_staged<T>(a.n, a.kc);
    const size_t smem = solve_smem_bytes<T>(a.n, a.kc, staged);
    auto kern = staged ? chain_fwd_kernel<T, true> : chain_fwd_kernel<T, false>;
    cudaError_t e = set_solve_smem<T>((const void *)kern, smem);
    if (e != cudaSuccess) return e;
    const unsigned grid = a.seq ? 1u : (unsigned)a.Q;
    kern<<<grid, SOLVE_THREADS, smem, s>>>(a);
    count_launch();
    return cudaGetLastError();
}

template <class T, class Tsep>
cudaError_t launch_chain_bwd(const SolveArgs<T> &a, cudaStream_t s)
{
    if (solve_streamed<T>(a.n, a.kc) && stream_aligned(a)) {
        const size_t smem = stream_smem_bytes<T>(a.n, a.kc);
        auto kern = chain_bwd_stream_kernel<T, Tsep>;
        cudaError_t e = set_solve_smem<T>((const void *)kern, smem);
        if (e != cudaSuccess) return e;
        kern<<<(unsigned)a.Q, SOLVE_THREADS, smem, s>>>(a);
        count_launch();
        return cudaGetLastError();
    }
    const bool staged = solve_staged<T>(a.n, a.kc);
    const size_t smem = solve_smem_bytes<T>(a.n, a.kc, staged);
    auto kern = staged ? chain_bwd_kernel<T, Tsep, true> : chain_bwd_kernel<T, Tsep, false>;
    cudaError_t e = set_solve_smem<T>((const void *)kern, smem);
    if (e != cudaSuccess) return e;
    kern<<<(unsigned)a.Q, SOLVE_THREADS, smem, s>>>(a);
    count_launch();
    return cudaGetLastError();
}

template <class T, class Tn>
cudaError_t launch_assemble_rhs(const T *d, const T *bvec, Tn *dn, long long N, long long Q, int n, int k, int j0,
                                int kc, cudaStream_t s)
{
    const long long work = (Q + 1) * (long long)n * kc;
    assemble_rhs_kernel<T, Tn><<<grid_for(work, 256), 256, 0, s>>>(d, bvec, dn, N, Q, n, k, j0, kc);
    count_launch();
    return cudaGetLastError();
}

template <class T>
cudaError_t launch_opnorm(const T *A, const T *B, long long N, int n, DevStatus *st, cudaStream_t s)
{
    opnorm_kernel<T><<<grid_for(N * n, 256), 256, 0, s>>>(A, B, N, n, st);
    count_launch();
    return cudaGetLastError();
}

template <class T>
cudaError_t launch_absmax(const T *v, long long count, unsigned long long *dst, cudaStream_t s)
{
    absmax_kernel<T><<<grid_for(count, 256), 256, 0, s>>>(v, count, dst);
    count_launch();
    return cudaGetLastError();
}

template <class T, class Tr>
cudaError_t launch_residual(const T *A, const T *B, const T *x, const T *d, Tr *r, long long N, int n, int k,
                            int with_norm, DevStatus *st, cudaStream_t s)
{
    auto kern = residual_kernel<T, Tr>;
    int kc = k;
    while (kc > 1 && residual_smem_bytes<T>(n, kc) > (size_t)200 * 1024) kc = (kc + 1) / 2;
    const size_t smem = residual_smem_bytes<T>(n, kc);
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    int dev = 0, sms = 1, per_sm = 1;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, RES_THREADS, smem);
    long long grid = (long long)sms * (per_sm > 0 ? per_sm : 1);
    if (grid > N) grid = N;
    const long long per_cta = (N + grid - 1) / grid;
    grid = (N + per_cta - 1) / per_cta;
    for (int j0 = 0; j0 < k; j0 += kc) {
        const int kk = (k - j0 < kc) ? k - j0 : kc;
        kern<<<(unsigned)grid, RES_THREADS, smem, s>>>(A, B, x, d, r, N, n, k, j0, kk, per_cta,
                                                       (with_norm && j0 == 0) ? 1 : 0, st);
        count_launch();
        e = cudaGetLastError();
        if (e != cudaSuccess) return e;
    }
    return cudaSuccess;
}

template <class Tr, int THREADS>
cudaError_t launch_residual_df_t(const double *A, const double *B, const double *x, const double *d, Tr *r,
                                 long long N, int n, int k, int with_norm, DevStatus *st, cudaStream_t s)
{
    int kc = k;  // every column in one pass when the partials fit: A and B are read once
    while (kc > 1 && residual_df_smem_bytes<THREADS>(n, kc) > residual_df_smem_cap<THREADS>()) kc = (kc + 1) / 2;
    // blocks through bulk copies into shared memory when all columns go in one
    // pass and two CTAs still fit an SM (256-thread CTAs; even n, aligned A, B)
    const bool raw = THREADS == 256 && kc == k && n % 2 == 0 && ((uintptr_t)A % 16u) == 0 &&
                     ((uintptr_t)B % 16u) == 0 && residual_df_smem_bytes<THREADS, true>(n, k) <= (size_t)113 * 1024;
    auto kern = raw ? residual_df_kernel<Tr, THREADS, true> : residual_df_kernel<Tr, THREADS, false>;
    const size_t smem = raw ? residual_df_smem_bytes<THREADS, true>(n, kc) : residual_df_smem_bytes<THREADS>(n, kc);
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    e = cudaFuncSetAttribute(kern, cudaFuncAttributePreferredSharedMemoryCarveout, 100);
    if (e != cudaSuccess) return e;
    const int per_sm = ctas_per_sm(kern, THREADS, smem);
    int dev = 0, sms = 1;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    long long grid = (long long)sms * (per_sm > 0 ? per_sm : 1);
    if (grid > N) grid = N;
    const long long per_cta = (N + grid - 1) / grid;
    grid = (N + per_cta - 1) / per_cta;
    for (int j0 = 0; j0 < k; j0 += kc) {
        const int kk = (k - j0 < kc) ? k - j0 : kc;
        kern<<<(unsigned)grid, THREADS, smem, s>>>(A, B, x, d, r, N, n, k, j0, kk, per_cta,
                                                   (with_norm && j0 == 0) ? with_norm : 0, st);
        count_launch();
        e = cudaGetLastError();
        if (e != cudaSuccess) return e;
    }
    return cudaSuccess;
}

template <class Tr>
cudaError_t launch_residual_df(const double *A, const double *B, const double *x, const double *d, Tr *r,
                               long long N, int n, int k, int with_norm, DevStatus *st, cudaStream_t s)
{
    if (res_df_threads(n) == 512)
        return launch_residual_df_t<Tr, 512>(A, B, x, d, r, N, n, k, with_norm, st, s);
    return launch_residual_df_t<Tr, 256>(A, B, x, d, r, N, n, k, with_norm, st, s);
}

template <class Tc>
cudaError_t launch_update(double *x, const Tc *c, long long count, int assign, cudaStream_t s)
{
    update_kernel<Tc><<<grid_for(count, 256), 256, 0, s>>>(x, c, count, assign);
    count_launch();
    return cudaGetLastError();
}

template <class Ts, class Td>
cudaError_t launch_convert(Td *dst, const Ts *src, long long count, cudaStream_t s)
{
    convert_kernel<Ts, Td><<<grid_for(count, 256), 256, 0, s>>>(dst, src, count);
    count_launch();
    return cudaGetLastError();
}

template <class T>
cudaError_t launch_init_identity(T *A, long long first_blk, long long last_blk, int n, cudaStream_t s)
{
    if (last_blk <= first_blk) return cudaSuccess;
    init_identity_kernel<T><<<grid_for((last_blk - first_blk) * (long long)n * n, 256), 256, 0, s>>>(
        A, first_blk, last_blk, n);
    count_launch();
    return cudaGetLastError();
}

}  // namespace bss
