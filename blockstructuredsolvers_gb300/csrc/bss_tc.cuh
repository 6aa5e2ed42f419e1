// Tensor-core (tcgen05) products C = X^T Y of n x n FP32 blocks, n <= 128,
// for the wide chain kernel.  sm_100-family only (built for sm_103a).
//
// Accuracy: the mixed-precision factorization needs FP32-level products, so
// each operand is split into two TF32 parts, x = hi + lo (hi = tf32(x),
// lo = tf32(x - hi)), and C = Xh^T Yh + Xh^T Yl + Xl^T Yh is accumulated in
// FP32 in tensor memory (the 3xTF32 scheme; relative error ~2^-21).
//
// Layout: one MMA is M = 128 (rows i of C = columns of X), N = 128 (columns
// j of C = columns of Y), K = 8.  Both operands are "K-major": for each i
// (resp. j) the K values are contiguous, which is exactly a column of the
// column-major block.  In shared memory each operand chunk of K = 32 is
// stored in the canonical no-swizzle layout: core matrices of 8 rows x 16
// bytes (4 values of K), the 8 core matrices of one 8-row group adjacent
// along K (leading byte offset 128) and the 16 row groups 1024 bytes apart
// (stride byte offset 1024), so element (i, k) of the chunk sits at byte
// (i / 8) * 1024 + (k / 4) * 128 + (i % 8) * 16 + (k % 4) * 4; a thread
// writing 16 bytes at e * 16 (e = 0 .. 1023) covers the chunk linearly.
// TC_NSTAGE stages of four 16 KB arrays (X hi/lo, Y hi/lo), each guarded by
// an mbarrier (tcgen05.commit arrives when the stage's MMAs are done).
//
// The accumulator is 128 lanes x 128 columns of FP32 in TMEM (lane = row i,
// column = j).  Warp w reads lanes 32 (w % 4) .. +31 and columns
// 64 (w / 4) .. +63 (256-thread CTAs).  Every wait on an mbarrier is
// bounded; on expiry the CTA sets an abort flag, the caller records a
// timeout in the status and stops.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

namespace bss {

constexpr int TC_K_CHUNK = 32;
constexpr int TC_OPERAND_BYTES = 128 * TC_K_CHUNK * 4;  // one operand part of one chunk: 16 KB
constexpr int TC_STAGE_BYTES = 4 * TC_OPERAND_BYTES;    // X hi, X lo, Y hi, Y lo
constexpr int TC_NSTAGE = 1;  // stage buffers (one: two CTAs fit per SM)
constexpr int TC_TMEM_COLS = 128;
// try_wait polls before a stage counts as lost: a poll on an unfinished
// mbarrier suspends ~7.8K SM cycles (measured), so 2^18 polls give up after
// about one second; a stage of MMAs completes within a few polls
constexpr unsigned TC_WAIT_LIMIT = 1u << 18;

struct TcCtx {
    uint32_t taddr;      // TMEM accumulator (lane 0, first column)
    uint32_t stage;      // shared address of stage 0
    uint32_t mbar;       // shared address of mbarrier 0 (8 bytes each)
    uint32_t phase[2];   // parity to wait for next, per stage
    uint32_t pending[2]; // a commit on this stage not yet waited for
    int *abort;          // shared flag: a wait expired
};

__device__ __forceinline__ uint32_t smem_u32(const void *p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ uint32_t to_tf32(float x)
{
    uint32_t r;
    asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(r) : "f"(x));
    return r;
}

// ---- FP64 -> FP32 conversion on the integer pipes ----
// GB300's cvt.rn.f32.f64 runs on the FP64 pipe (measured ~2 conversions per
// clock per SM against ~7.5 for this integer form).  The 128-wide chain
// kernel, which converts 32K FP64 values per step with registers to spare,
// uses the bit operations of IEEE round-to-nearest-even (bit-identical to
// cvt.rn on 268M values spanning the FP32 normal range, ties and carries);
// in the register-bound 64-wide kernels the longer form measured slower:
// rebias the exponent (1023 -> 127), keep the top 23 of the 52 fraction bits
// and round on the other 29 (a carry out of the fraction raises the
// exponent, as rounding does).  Magnitudes below 2^-126 become signed zero
// (no FP32 subnormals), above the FP32 range infinity; NaN becomes infinity.
__device__ __forceinline__ float f64_to_f32(double a)
{
    const unsigned hi = (unsigned)__double2hiint(a), lo = (unsigned)__double2loint(a);
    const unsigned mag = hi & 0x7FFFFFFFu;
    const int e = (int)(mag >> 20) - 896;
    unsigned bits = ((unsigned)e << 23) + (((mag & 0xFFFFFu) << 3) | (lo >> 29));
    const unsigned rest = lo & 0x1FFFFFFFu;
    bits += (rest > 0x10000000u || (rest == 0x10000000u && (bits & 1u))) ? 1u : 0u;
    bits = e <= 0 ? 0u : (e >= 255 || bits >= 0x7F800000u ? 0x7F800000u : bits);
    return __uint_as_float(bits | (hi & 0x80000000u));
}
__device__ __forceinline__ float f64_to_f32(float a) { return a; }

// instruction descriptor: kind::tf32, D = F32, A = B = TF32, both K-major,
// M = 128, N = 128, dense, no negation
__host__ __device__ constexpr uint32_t tc_idesc_128x128()
{
    return (1u << 4)              // D format F32
           | (2u << 7)            // A format TF32
           | (2u << 10)           // B format TF32
           | ((128u >> 3) << 17)  // N / 8
           | ((128u >> 4) << 24); // M / 16
}

// shared memory descriptor of a canonical no-swizzle K-major operand
__device__ __forceinline__ uint64_t tc_smem_desc(uint32_t saddr)
{
    uint64_t d = (uint64_t)((saddr & 0x3FFFFu) >> 4);
    d |= (uint64_t)(128u >> 4) << 16;   // leading byte offset: next core matrix along K
    d |= (uint64_t)(1024u >> 4) << 32;  // stride byte offset: next 8-row group
    d |= (uint64_t)1 << 46;             // descriptor version of the sm_100 family
    return d;                            // base offset 0, no swizzle
}

__device__ __forceinline__ void tc_mma(uint32_t taddr, uint64_t da, uint64_t db, uint32_t idesc, uint32_t acc)
{
    asm volatile(
        "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
        " tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n}\n" ::"r"(taddr),
        "l"(da), "l"(db), "r"(idesc), "r"(acc)
        : "memory");
}

__device__ __forceinline__ void tc_commit(uint32_t mbar)
{
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(mbar)
                 : "memory");
}

__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void fence_async_smem() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }

// bounded wait for the given parity of an mbarrier (at most `limit`
// try_wait polls); false when it expired
__device__ __forceinline__ bool mbar_wait(uint32_t mbar, uint32_t parity, unsigned limit = TC_WAIT_LIMIT)
{
    for (unsigned it = 0; it < limit; ++it) {
        uint32_t ok;
        asm volatile(
            "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n"
            " selp.u32 %0, 1, 0, p;\n}\n"
            : "=r"(ok)
            : "r"(mbar), "r"(parity)
            : "memory");
        if (ok) return true;
    }
    return false;
}

// CTA set-up: warp 0 allocates the TMEM accumulator, thread 0 initialises
// the two mbarriers.  `slot` is a 4-byte shared word for the TMEM address.
__device__ __forceinline__ void tc_setup(TcCtx &c, uint32_t *slot, uint64_t *mbars, unsigned char *stage, int *abort)
{
    if (threadIdx.x < 32) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(slot)),
                     "r"((uint32_t)TC_TMEM_COLS)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    if (threadIdx.x == 0) {
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(&mbars[0])) : "memory");
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(&mbars[1])) : "memory");
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        *abort = 0;
    }
    fence_async_smem();
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    c.taddr = *slot;
    c.stage = smem_u32(stage);
    c.mbar = smem_u32(mbars);
    c.phase[0] = c.phase[1] = 0;
    c.pending[0] = c.pending[1] = 0;
    c.abort = abort;
}

// CTA tear-down: every thread is past its last TMEM access
__device__ __forceinline__ void tc_teardown(const TcCtx &c)
{
    tc_fence_before();
    __syncthreads();
    if (threadIdx.x < 32) {
        tc_fence_after();
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(c.taddr),
                     "r"((uint32_t)TC_TMEM_COLS)
                     : "memory");
    }
}

// wait for a stage's last commit (uniform over the CTA); on expiry set abort
__device__ __forceinline__ void tc_wait_stage(TcCtx &c, int s)
{
    if (!c.pending[s]) return;
    if (!mbar_wait(c.mbar + 8u * s, c.phase[s])) *c.abort = 1;
    c.phase[s] ^= 1u;
    c.pending[s] = 0;
}

template <class Tg>
__device__ __forceinline__ float ld_cg_f(const Tg *p)
{
    return (float)__ldcg(p);
}

// load this thread's 16 values of chunk k0 .. k0+31 of an operand (column i
// of the n x n column-major matrix G, zero beyond n): all loads are issued
// before any use, so the chunk costs one memory latency
template <class Tg>
__device__ __forceinline__ void tc_load_chunk(const Tg *G, int n, int k0, float (&v)[4][4])
{
#pragma unroll
    for (int q = 0; q < 4; ++q) {
        const int e = threadIdx.x + 256 * q;
        const int i = 8 * (e >> 6) + (e & 7);
        const int k = k0 + 4 * ((e >> 3) & 7);
#pragma unroll
        for (int u = 0; u < 4; ++u) v[q][u] = (i < n && k + u < n) ? ld_cg_f<Tg>(G + (size_t)i * n + k + u) : 0.f;
    }
}

// split into hi / lo TF32 parts and store in the canonical layout
__device__ __forceinline__ void tc_store_chunk(const float (&v)[4][4], uint4 *hi, uint4 *lo)
{
#pragma unroll
    for (int q = 0; q < 4; ++q) {
        const int e = threadIdx.x + 256 * q;
        uint32_t h[4], l[4];
#pragma unroll
        for (int u = 0; u < 4; ++u) {
            h[u] = to_tf32(v[q][u]);
            l[u] = to_tf32(v[q][u] - __uint_as_float(h[u]));
        }
        hi[e] = make_uint4(h[0], h[1], h[2], h[3]);
        lo[e] = make_uint4(l[0], l[1], l[2], l[3]);
    }
}

// TMEM <- X^T Y for n x n column-major X (FP32) and Y (FP32 or FP64), n <= 128.
// All 256 threads of the CTA call it; on return the product is complete in
// TMEM (or *c.abort is set) and the operands may be overwritten.  When Y is
// X, the chunk is staged once and serves both operands.  The loads of a
// chunk are issued before waiting for the MMAs still reading the stage, so
// memory latency overlaps the tensor-core work.
template <class Ty>
__device__ __noinline__ void tc_tn(TcCtx &c, const float *X, const Ty *Y, int n, unsigned char *stage_base)
{
    const int nch = (n + TC_K_CHUNK - 1) / TC_K_CHUNK;
    constexpr uint32_t idesc = tc_idesc_128x128();
    const bool same = (const void *)X == (const void *)Y;
    for (int ch = 0; ch < nch; ++ch) {
        const int s = ch % TC_NSTAGE;
        float vx[4][4], vy[4][4];
        tc_load_chunk<float>(X, n, ch * TC_K_CHUNK, vx);
        if (!same) tc_load_chunk<Ty>(Y, n, ch * TC_K_CHUNK, vy);
        tc_wait_stage(c, s);  // the MMAs that last read this stage are done
        unsigned char *st = stage_base + s * TC_STAGE_BYTES;
        tc_store_chunk(vx, reinterpret_cast<uint4 *>(st), reinterpret_cast<uint4 *>(st + TC_OPERAND_BYTES));
        if (!same)
            tc_store_chunk(vy, reinterpret_cast<uint4 *>(st + 2 * TC_OPERAND_BYTES),
                           reinterpret_cast<uint4 *>(st + 3 * TC_OPERAND_BYTES));
        fence_async_smem();  // generic-proxy stores -> visible to the tensor core
        __syncthreads();
        if (threadIdx.x == 0) {
            tc_fence_after();
            const uint32_t sb = c.stage + (uint32_t)(s * TC_STAGE_BYTES);
            const uint32_t yb = same ? sb : sb + 2 * TC_OPERAND_BYTES;
#pragma unroll
            for (int kk = 0; kk < TC_K_CHUNK / 8; ++kk) {
                const uint32_t off = (uint32_t)kk * 256u;  // K = 8: two core matrices along K
                const uint64_t xh = tc_smem_desc(sb + off), xl = tc_smem_desc(sb + TC_OPERAND_BYTES + off);
                const uint64_t yh = tc_smem_desc(yb + off), yl = tc_smem_desc(yb + TC_OPERAND_BYTES + off);
                tc_mma(c.taddr, xh, yh, idesc, (ch | kk) != 0 ? 1u : 0u);
                tc_mma(c.taddr, xh, yl, idesc, 1u);
                tc_mma(c.taddr, xl, yh, idesc, 1u);
            }
            tc_commit(c.mbar + 8u * s);
        }
        c.pending[s] = 1;
    }
    // drain (the later commit covers every MMA issued before it)
    for (int q = 0; q < TC_NSTAGE; ++q) tc_wait_stage(c, (nch + q) % TC_NSTAGE);
    tc_fence_after();
}

// 32 accumulator columns of this thread's row: row 32 (w % 4) + lane,
// columns 64 (w / 4) + 32 half + 0 .. 31
__device__ __forceinline__ void tc_load_row32(const TcCtx &c, int half, float (&v)[32])
{
    const int w = threadIdx.x >> 5;
    const uint32_t a = c.taddr + ((uint32_t)(32 * (w & 3)) << 16) + (uint32_t)(64 * (w >> 2));
    uint32_t r[32];
    {
        asm volatile(
            "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,"
            "%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];"
            : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
              "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]),
              "=r"(r[15]), "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]),
              "=r"(r[22]), "=r"(r[23]), "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]),
              "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
            : "r"(a + 32u * (uint32_t)half));
        asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
        for (int q = 0; q < 32; ++q) v[q] = __uint_as_float(r[q]);
    }
}

// dst(i, j) = scale * C(i, j) + (base ? base(i, j) : 0) for i, j < n; then
// every thread is past its TMEM reads (the next product may overwrite).
// The 32 base values of a half row are loaded together (one memory latency)
// before the accumulator half is read.
template <class Tb>
__device__ __forceinline__ void tc_store(const TcCtx &c, float *dst, int n, float scale, const Tb *base)
{
    const int w = threadIdx.x >> 5;
    const int i = 32 * (w & 3) + (threadIdx.x & 31);
#pragma unroll 1
    for (int half = 0; half < 2; ++half) {
        const int j0 = 64 * (w >> 2) + 32 * half;
        float b[32];
#pragma unroll
        for (int q = 0; q < 32; ++q) {
            const int j = j0 + q;
            b[q] = (base && i < n && j < n) ? (float)__ldcg(base + (size_t)i + (size_t)j * n) : 0.f;
        }
        float v[32];
        tc_load_row32(c, half, v);
        if (i < n) {
#pragma unroll
            for (int q = 0; q < 32; ++q) {
                const int j = j0 + q;
                if (j < n) dst[(size_t)i + (size_t)j * n] = scale * v[q] + b[q];
            }
        }
    }
    tc_fence_before();
    __syncthreads();
}

// ---- bulk copies and the bounded mbarrier waits of the copy-fed kernels ----
constexpr long long C64_WAIT_CYCLES = 2000000000LL;  // ~1 s of SM clock

__device__ __forceinline__ void mbar_expect_tx(uint32_t mbar, uint32_t bytes)
{
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(mbar), "r"(bytes) : "memory");
}

// one bulk copy global -> shared (16-byte aligned, size a multiple of 16),
// completing `bytes` of transaction count on the mbarrier
__device__ __forceinline__ void bulk_g2s(uint32_t dst, const void *src, uint32_t bytes, uint32_t mbar)
{
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(dst),
                 "l"(src), "r"(bytes), "r"(mbar)
                 : "memory");
}

__device__ __forceinline__ void bulk_prefetch_l2(const void *src, uint32_t bytes)
{
    asm volatile("cp.async.bulk.prefetch.L2.global [%0], %1;" ::"l"(src), "r"(bytes) : "memory");
}

// an mbarrier and the parity of its outstanding phase (thread 0's view)
struct C64Bar {
    uint32_t addr;
    uint32_t phase;
    bool pending;
};

__device__ __forceinline__ bool mbar_test(uint32_t mbar, uint32_t parity)
{
    uint32_t ok;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.test_wait.parity.shared::cta.b64 p, [%1], %2;\n"
        " selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(ok)
        : "r"(mbar), "r"(parity)
        : "memory");
    return ok != 0;
}

// thread 0 only: wait for the outstanding phase, at most C64_WAIT_CYCLES; on
// expiry set the abort flag and leave the phase outstanding (drained before
// exit).  The other threads learn the outcome at the next CTA barrier.
__device__ __forceinline__ void c64_wait1(C64Bar &b, int *abort)
{
    if (!b.pending) return;
    const long long t0 = clock64();
    for (;;) {
        if (mbar_test(b.addr, b.phase)) {
            b.phase ^= 1u;
            b.pending = false;
            return;
        }
        if (clock64() - t0 > C64_WAIT_CYCLES) {
            *abort = 1;
            return;
        }
    }
}

}  // namespace bss
