// Host <-> handle copies: bss_upload (a system from host memory into the
// handle's A/B/d tensors) and bss_download (the solution out of d_tensor).
//
// The reference's factorization reads only the upper triangle of each
// diagonal block: potrf with CUBLAS_FILL_MODE_UPPER in the batched and
// sequential GPU paths (src/backbone_cuda.jl:21-33, 77-99) and potrf!('U')
// on the CPU (src/backbone_cpu.jl:7, 12); the lower triangle of an A_i never
// changes its result.  BSS_UPLOAD_UPPER gives the upload the same meaning:
// after the copy a kernel mirrors each upper triangle into the lower one on
// the device, so every kernel of the library (they read whole blocks, e.g.
// the FP64 refinement residual) sees the symmetric matrix the reference
// factors, whatever the host's lower triangles hold.
//
// Every tensor crosses the host link as one contiguous copy.  The copy
// engines' rate from page-locked host memory bounds an upload (about 210
// GB/s on GB300, the same for one large copy, several copies on several
// streams, or SM loads of mapped host memory).  Moving only the upper
// triangles measured slower: as strided 3D copies (column bands, depth N
// blocks) the driver spends ~1.7 ms of host time per 16384-block upload, and
// as 2D copies with the block stride as pitch the copy engines ran at a
// fraction of their rate.
#include <cuda_runtime.h>

#include "bss_internal.h"

using namespace bss;

namespace {

constexpr int MT = 32;  // mirror tile edge

// lower(A_i) = upper(A_i)^T for blocks 0 .. N-1: work item = (block, lower
// tile (I, J), J <= I); the upper tile (J, I) goes through shared memory
// (column reads and column writes both coalesced).  Reads touch only the
// upper triangle and writes only the strict lower one, so work items never
// race.
template <class T>
__global__ void __launch_bounds__(256) mirror_upper_kernel(T *A, long long N, int n, int tiles)
{
    __shared__ T s[MT][MT + 1];
    const int pairs = tiles * (tiles + 1) / 2;
    const long long total = N * pairs;
    const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;
    const long long nn = (long long)n * n;
    for (long long w = blockIdx.x; w < total; w += gridDim.x) {
        const long long blk = w / pairs;
        int p = (int)(w - blk * pairs), I = 0;
        while (p > I) {
            p -= I + 1;
            ++I;
        }
        const int J = p;
        T *M = A + blk * nn;
        // s[cc][tx] = upper element (row J*32 + tx, column I*32 + cc)
        for (int cc = ty; cc < MT; cc += 8) {
            const int c = I * MT + cc, r = J * MT + tx;
            if (c < n && r <= c) s[cc][tx] = M[(long long)c * n + r];
        }
        __syncthreads();
        // lower element (row I*32 + tx, column J*32 + cc) = upper (column, row)
        for (int cc = ty; cc < MT; cc += 8) {
            const int c = J * MT + cc, r = I * MT + tx;
            if (r < n && r > c) M[(long long)c * n + r] = s[tx][cc];
        }
        __syncthreads();
    }
}

template <class T>
cudaError_t launch_mirror_upper(T *A, long long N, int n, cudaStream_t s)
{
    if (N <= 0 || n < 2) return cudaSuccess;
    const int tiles = (n + MT - 1) / MT;
    const long long total = N * (long long)(tiles * (tiles + 1) / 2);
    int dev = 0, sms = 152;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    const long long cap = (long long)sms * 8;
    mirror_upper_kernel<T><<<(unsigned)(total < cap ? total : cap), 256, 0, s>>>(A, N, n, tiles);
    count_launch();
    return cudaGetLastError();
}

}  // namespace

extern "C" int bss_upload(bss_handle *h, const void *A, const void *B, const void *d, int32_t flags,
                          int64_t *host_bytes)
{
    if (!h) return fail(BSS_ERR_ARG, "handle is NULL");
    if (flags != BSS_UPLOAD_FULL && flags != BSS_UPLOAD_UPPER) return fail(BSS_ERR_ARG, "unknown upload flags");
    if (h->external_arena) return fail(BSS_ERR_STATE, "the handle belongs to a batch: upload through its tensors");
    const long long N = h->N_user;
    const int n = (int)h->n;
    const size_t es = tsize(h->dtype), nn = (size_t)n * n;
    long long moved = 0;
    if (A) {
        BSS_CUDA(cudaMemcpyAsync(h->A, A, N * nn * es, cudaMemcpyHostToDevice, h->stream));
        moved += (long long)(N * nn * es);
        if (flags == BSS_UPLOAD_UPPER) {
            const cudaError_t e = h->dtype == F64 ? launch_mirror_upper<double>((double *)h->A, N, n, h->stream)
                                                  : launch_mirror_upper<float>((float *)h->A, N, n, h->stream);
            if (e != cudaSuccess) return cuda_fail(e, "mirror_upper");
        }
    }
    if (B && N > 1) {
        BSS_CUDA(cudaMemcpyAsync(h->B, B, (N - 1) * nn * es, cudaMemcpyHostToDevice, h->stream));
        moved += (long long)((N - 1) * nn * es);
    }
    if (d) {
        const size_t bytes = (size_t)N * n * h->k * es;
        BSS_CUDA(cudaMemcpyAsync(h->d, d, bytes, cudaMemcpyHostToDevice, h->stream));
        moved += (long long)bytes;
    }
    if (host_bytes) *host_bytes = moved;
    return BSS_OK;
}

extern "C" int bss_download(bss_handle *h, void *x)
{
    if (!h) return fail(BSS_ERR_ARG, "handle is NULL");
    if (!x) return fail(BSS_ERR_ARG, "x is NULL");
    const size_t bytes = (size_t)h->N_user * h->n * h->k * tsize(h->dtype);
    BSS_CUDA(cudaMemcpyAsync(x, h->d, bytes, cudaMemcpyDeviceToHost, h->stream));
    return BSS_OK;
}
