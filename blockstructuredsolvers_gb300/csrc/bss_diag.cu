// Diagnostic: one tensor-core product C = X^T Y (the wide kernel's
// tcgen05 3xTF32 path) against an FP64 product of the same FP32 inputs.
// No counterpart in the reference; used by the tests.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <vector>

#include "bss_internal.h"

using namespace bss;

namespace {

__global__ void diag_fill_kernel(float *X, float *Y, int n)
{
    for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < n * n; e += gridDim.x * blockDim.x) {
        unsigned x = (unsigned)e * 2654435761u + 12345u;
        x ^= x >> 13;
        x *= 0x5bd1e995u;
        x ^= x >> 15;
        X[e] = (float)((int)(x & 0xFFFF) - 32768) / 32768.0f;
        unsigned y = (unsigned)e * 40503u + 977u;
        y ^= y >> 11;
        y *= 0x27d4eb2du;
        y ^= y >> 15;
        Y[e] = (float)((int)(y & 0xFFFF) - 32768) / 65536.0f + (e % (n + 1) == 0 ? 1.0f : 0.0f);
    }
}

__global__ void diag_ref_kernel(const float *X, const float *Y, double *R, int n)
{
    for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < n * n; e += gridDim.x * blockDim.x) {
        const int i = e % n, j = e / n;
        double s = 0.0;
        for (int k = 0; k < n; ++k) s += (double)X[k + i * n] * (double)Y[k + j * n];
        R[e] = s;
    }
}

__global__ void __launch_bounds__(256) diag_tc_kernel(const float *X, const float *Y, float *C, int n, int *abort_out)
{
    extern __shared__ __align__(128) unsigned char smem_wide[];
    unsigned char *tail = smem_wide + TC_NSTAGE * TC_STAGE_BYTES;
    TcCtx tcc{};
    tc_setup(tcc, reinterpret_cast<uint32_t *>(tail + 16), reinterpret_cast<uint64_t *>(tail), smem_wide,
             reinterpret_cast<int *>(tail + 32));
    tc_tn<float>(tcc, X, Y, n, smem_wide);
    tc_store<float>(tcc, C, n, 1.f, (const float *)nullptr);
    if (threadIdx.x == 0) *abort_out = *tcc.abort;
    tc_teardown(tcc);
}

}  // namespace

extern "C" int bss_tc_selftest(int64_t n, double *max_rel_err)
{
    if (n < 1 || n > 128 || !max_rel_err) return fail(BSS_ERR_ARG, "bss_tc_selftest: 1 <= n <= 128");
    float *X = nullptr, *Y = nullptr, *C = nullptr;
    double *R = nullptr;
    int *ab = nullptr;
    const size_t nn = (size_t)n * n;
    BSS_CUDA(cudaMalloc((void **)&X, nn * 4));
    BSS_CUDA(cudaMalloc((void **)&Y, nn * 4));
    BSS_CUDA(cudaMalloc((void **)&C, nn * 4));
    BSS_CUDA(cudaMalloc((void **)&R, nn * 8));
    BSS_CUDA(cudaMalloc((void **)&ab, 4));
    diag_fill_kernel<<<64, 256>>>(X, Y, (int)n);
    diag_ref_kernel<<<64, 256>>>(X, Y, R, (int)n);
    const int smem = TC_NSTAGE * TC_STAGE_BYTES + 128;
    cudaError_t e = cudaFuncSetAttribute(diag_tc_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
    if (e == cudaSuccess) {
        diag_tc_kernel<<<1, 256, smem>>>(X, Y, C, (int)n, ab);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaDeviceSynchronize();
    std::vector<float> hc(nn);
    std::vector<double> hr(nn);
    int abort_flag = 0;
    if (e == cudaSuccess) e = cudaMemcpy(hc.data(), C, nn * 4, cudaMemcpyDeviceToHost);
    if (e == cudaSuccess) e = cudaMemcpy(hr.data(), R, nn * 8, cudaMemcpyDeviceToHost);
    if (e == cudaSuccess) e = cudaMemcpy(&abort_flag, ab, 4, cudaMemcpyDeviceToHost);
    cudaFree(X);
    cudaFree(Y);
    cudaFree(C);
    cudaFree(R);
    cudaFree(ab);
    if (e != cudaSuccess) return cuda_fail(e, "bss_tc_selftest");
    if (abort_flag) return fail(BSS_ERR_TIMEOUT, "tensor-core wait expired");
    double mx = 0.0, md = 0.0;
    for (size_t q = 0; q < nn; ++q) {
        mx = std::max(mx, std::abs(hr[q]));
        md = std::max(md, std::abs((double)hc[q] - hr[q]));
    }
    *max_rel_err = mx > 0 ? md / mx : md;
    return BSS_OK;
}

// Diagnostic: the occupancy query the planner makes for the FP32-factor
// wide kernel (tensor-core form): out[0..2] = error codes of the two
// attribute calls and the query, out[3] = blocks per SM, out[4] = registers
// per thread, out[5] = dynamic shared memory bytes
extern "C" int bss_diag_wide_occupancy(int64_t *out)
{
    if (!out) return fail(BSS_ERR_ARG, "out is NULL");
    auto kern = wide_chain_factor_kernel<double, float, true>;
    const size_t smem = wide_factor_smem<float, true>();
    out[0] = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    out[1] = cudaFuncSetAttribute(kern, cudaFuncAttributePreferredSharedMemoryCarveout, 100);
    int nblk = -1;
    out[2] = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nblk, kern, WIDE_THREADS, smem);
    out[3] = nblk;
    cudaFuncAttributes fa{};
    cudaFuncGetAttributes(&fa, kern);
    out[4] = fa.numRegs;
    out[5] = (int64_t)smem;
    return BSS_OK;
}

// Diagnostic: the residual r = d - T x of an FP64 system by the exact FP64
// kernel (method 0) or by the refinement's double-float kernel (method 1),
// written to r (device, n x k per block); synchronises.
extern "C" int bss_diag_residual(int64_t N, int64_t n, int64_t k, int32_t method, const double *A, const double *B,
                                 const double *x, const double *d, double *r, void *stream)
{
    if (N < 1 || n < 1 || k < 1 || !A || (N > 1 && !B) || !x || !d || !r || (method != 0 && method != 1))
        return fail(BSS_ERR_ARG, "bss_diag_residual: bad argument");
    if (residual_smem_bytes<double>((int)n, 1) > (size_t)200 * 1024)
        return fail(BSS_ERR_ARG, "bss_diag_residual: block size too large for the residual kernel");
    cudaStream_t s = (cudaStream_t)stream;
    DevStatus *st = nullptr;
    BSS_CUDA(cudaMallocAsync((void **)&st, sizeof(DevStatus), s));
    BSS_CUDA(cudaMemsetAsync(st, 0, sizeof(DevStatus), s));
    cudaError_t e = method == 0
                        ? launch_residual<double, double>(A, B, x, d, r, N, (int)n, (int)k, 1, st, s)
                        : launch_residual_df<double>(A, B, x, d, r, N, (int)n, (int)k, 1, st, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    cudaFreeAsync(st, s);
    if (e != cudaSuccess) return cuda_fail(e, "bss_diag_residual");
    return BSS_OK;
}

namespace {
// an mbarrier that expects one arrival and never gets it: the bounded wait of
// the tensor-core kernels (mbar_wait) must give up after `polls` polls and
// say so; out[0] = 1 when it expired, out[1] = clock cycles it took
__global__ void diag_wait_kernel(unsigned polls, long long *out)
{
    __shared__ __align__(8) uint64_t mbar;
    if (threadIdx.x == 0) {
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(&mbar)) : "memory");
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        const long long t0 = clock64();
        const bool ok = mbar_wait(smem_u32(&mbar), 0u, polls);
        out[1] = clock64() - t0;
        out[0] = ok ? 0 : 1;
    }
}
}  // namespace

// Diagnostic: the bounded mbarrier wait on a barrier nothing arrives on.
extern "C" int bss_diag_wait_timeout(int64_t polls, int64_t *timed_out, int64_t *cycles)
{
    if (polls < 1 || polls > (int64_t)TC_WAIT_LIMIT || !timed_out || !cycles)
        return fail(BSS_ERR_ARG, "bss_diag_wait_timeout: bad argument");
    long long *d = nullptr;
    BSS_CUDA(cudaMalloc((void **)&d, 2 * sizeof(long long)));
    diag_wait_kernel<<<1, 32>>>((unsigned)polls, d);
    count_launch();
    long long h[2] = {0, 0};
    cudaError_t e = cudaGetLastError();
    if (e == cudaSuccess) e = cudaMemcpy(h, d, sizeof(h), cudaMemcpyDeviceToHost);
    cudaFree(d);
    if (e != cudaSuccess) return cuda_fail(e, "bss_diag_wait_timeout");
    *timed_out = h[0];
    *cycles = h[1];
    return BSS_OK;
}

// ---------------------------------------------------------------------------
// FMA-pipe peak microbenchmark: every thread runs 8 independent FMA chains
// (enough to cover the pipe latency with 8 warps per scheduler) for `iters`
// iterations; one FMA = 2 flops.  The result is written only when the
// impossible flag is set, which keeps the compiler from removing the chains.
// ---------------------------------------------------------------------------
namespace {
template <class T>
__global__ void __launch_bounds__(256) fma_peak_kernel(T a, T b, int iters, int flag, T *out)
{
    T x0 = (T)threadIdx.x, x1 = x0 + T(1), x2 = x0 + T(2), x3 = x0 + T(3);
    T x4 = x0 + T(4), x5 = x0 + T(5), x6 = x0 + T(6), x7 = x0 + T(7);
#pragma unroll 4
    for (int i = 0; i < iters; ++i) {
        x0 = fma(x0, a, b);
        x1 = fma(x1, a, b);
        x2 = fma(x2, a, b);
        x3 = fma(x3, a, b);
        x4 = fma(x4, a, b);
        x5 = fma(x5, a, b);
        x6 = fma(x6, a, b);
        x7 = fma(x7, a, b);
    }
    if (flag) out[blockIdx.x * blockDim.x + threadIdx.x] = x0 + x1 + x2 + x3 + x4 + x5 + x6 + x7;
}

template <class T>
int fma_peak(double *tflops)
{
    int dev = 0, sms = 0;
    BSS_CUDA(cudaGetDevice(&dev));
    BSS_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    const int blocks = sms * 8, threads = 256;  // 8 CTAs of 256 threads per SM: 64 warps
    const int iters = sizeof(T) == 8 ? 1 << 12 : 1 << 16;
    cudaEvent_t e0, e1;
    BSS_CUDA(cudaEventCreate(&e0));
    BSS_CUDA(cudaEventCreate(&e1));
    float best = 1e30f;
    for (int r = 0; r < 4; ++r) {  // first launch warms up; best of the rest
        cudaEventRecord(e0, 0);
        fma_peak_kernel<T><<<blocks, threads>>>(T(0.999), T(1e-3), iters, 0, (T *)nullptr);
        count_launch();
        cudaEventRecord(e1, 0);
        cudaError_t e = cudaEventSynchronize(e1);
        if (e != cudaSuccess) {
            cudaEventDestroy(e0);
            cudaEventDestroy(e1);
            return cuda_fail(e, "fma_peak_kernel");
        }
        float ms = 0.f;
        cudaEventElapsedTime(&ms, e0, e1);
        if (r > 0) best = std::min(best, ms);
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    const double flops = 2.0 * 8.0 * (double)iters * (double)blocks * (double)threads;
    *tflops = flops / (best * 1e-3) / 1e12;
    return BSS_OK;
}
}  // namespace

extern "C" int bss_diag_fma_peak(int32_t dtype, double *tflops)
{
    if (!tflops) return fail(BSS_ERR_ARG, "bss_diag_fma_peak: tflops is NULL");
    if (dtype == BSS_F64) return fma_peak<double>(tflops);
    if (dtype == BSS_F32) return fma_peak<float>(tflops);
    return fail(BSS_ERR_ARG, "bss_diag_fma_peak: dtype must be BSS_F32 or BSS_F64");
}

extern "C" int bss_diag_set_factor_variant(int32_t variant)
{
    if (variant < 0 || (variant & ~FACTOR_VARIANTS) != 0)
        return fail(BSS_ERR_ARG, "bss_diag_set_factor_variant: a combination of BSS_FACTOR_FMA_CHAIN, BSS_FACTOR_WIDE_L2");
    set_default_factor_variant(variant);
    return BSS_OK;
}

extern "C" int32_t bss_diag_get_factor_variant(void) { return default_factor_variant(); }
