// Chain factor kernel for wide blocks (n in 65..128) with FP32 factors on the
// 5th-generation tensor cores, one CTA per SM: one CTA walks one partition's
// chain like chain_factor_body (same recursion, same outputs V_i, W_i, Y_i
// and S_LL / S_RR / S_LR), holding the whole step on chip.  Reference: the
// potrf/trsm/gemm sequence of cholesky_factorize_batched! and the Schur
// products of compute_schur_complement! (src/backbone_cuda.jl:70-101,
// 143-157).
//
// Products (3xTF32: x = hi + lo, C = Xh Yh + Xh Yl + Xl Yh in the FP32 TMEM
// accumulator, relative error ~2^-21 like FP32 FMA products), each an
// M = 128, N = 128 MMA sequence D(m, j) = sum_k A(m, k) B(j, k) over K = 128
// in chunks of 16.  "op(X)" is the operand whose row m is column m of X:
//   phase 1 (from the carried W_{i-1}, Y_{i-1}):
//     D1 = op(W) op(W)^T = W^T W          -> Ahat_i = A_i - W^T W
//     D2 = op(Y) op(W)^T = Y^T W = -Z_i^T  (row m of D2 is -column m of Z_i)
//     S_LL += op(Y) op(Y)^T = Y^T Y        (accumulated in TMEM over the chain)
//   phase 2 (after U^T U = Ahat_i, V_i = U^-1 on the CUDA cores):
//     D1 = op(Z) op(V)^T = Z^T V = Y_i^T   (row m of D1 is column m of Y_i)
//     DW = op(B) op(V)^T = B^T V = W_i^T
// and at the chain end phase 1 on the last W, Y gives S_RR = W^T W (D1),
// S_LR = Y^T W (D2) and the last S_LL term.  A row of a Y_i^T / W_i^T
// accumulator is a row of the next step's operand, so the factors never
// leave the chip between the step that makes them and the step that uses
// them; they are written to HBM once, for the solve.
//
// Tensor memory (512 columns, 128 lanes): S_LL | D1 | D2 | DW, 128 columns each.
//
// Shared memory (~217 KB), by phase of a step:
//   [0, 66 KB)      the carried Y_{i-1} as op(Y) rows (FP32, row stride 132
//                   floats) in phase 1; A_i column chunks 1-4 for the Ahat
//                   readout; then V (sV, the Cholesky's column-major tile,
//                   leading dimension 132)
//   [66, 132 KB)    the carried W_{i-1} rows in phase 1; then Ahat / U
//                   (sS); then, with the next 30 KB, the two phase-2 stages
//   [132, 196 KB)   the two phase-1 stages; A_i chunks 5-7; the B_i chunks
//   [196, 216 KB)   A_i chunk 0 (lands during phase 1); the third B_i chunk
//   control words   pivot reciprocals, pivot-row buffer, flags, TMEM
//                   address, mbarriers (two stages, eight A chunks, three
//                   B chunks)
// A stage holds one K = 16 chunk of each operand it feeds, split into hi and
// lo TF32 parts, each part 128 rows x 16 K in the canonical no-swizzle
// K-major layout: 8-row x 16-byte core matrices, the four of a row group
// adjacent along K (leading byte offset 128), row groups 512 bytes apart
// (stride byte offset 512).  Converter threads take consecutive rows, so
// each quarter-warp reads and writes 128 contiguous bytes: no bank
// conflicts.  The chunk after the one being multiplied is split while the
// tensor core works on the current one.  tcgen05.mma blocks the issuing
// thread for the MMA's duration (measured: issue time equals execution
// time, 104 cycles per M = N = 128, K = 8 TF32 MMA), so phase 1, whose 18
// MMAs per chunk outweigh its split, is warp-specialised: warp 0 issues
// chunk c while warps 1-7 split chunk c + 1 (`c128_pipeline`); phase 2,
// whose split (three operands) outweighs its 12 MMAs, splits on all eight
// warps and thread 0 issues between barriers.
//
// Block loads are bulk copies (cp.async.bulk) completing on mbarriers (L2
// prefetch hints a step ahead measured no gain in time or DRAM bytes):
// A_i in column chunks of 16 (contiguous in the column-major block), chunk 0
// issued at the step's start into a buffer of its own, the others as soon
// as phase 1 has released their buffers; B_i in row chunks of 16 (the K
// chunks of op(B)): one 2D tensor copy per chunk (cp.async.bulk.tensor, box
// of 16 rows x 128 columns of the level's B, out-of-range rows and columns
// filled with zeros) with the 128-byte swizzle, so that the converters'
// reads of eight consecutive columns hit eight different bank groups; three
// chunks in flight: the first three land during the Cholesky, each later
// one is issued when the chunk three before it has been split (FP64 input,
// the first level of the mixed path; FP32 levels read B_i with plain loads).
// Blocks whose columns do not start on 16 bytes (odd n; FP32 input with n
// not a multiple of 4) are read with plain loads.
//
// Thread 0 issues every MMA and waits on the stage barriers at the end of a
// phase, on the A copies and (phase 2) on the stages and B copies; in phase 1
// thread 32 waits on the stage barriers for the converter warps.  Every wait
// is a spin on mbarrier.test_wait bounded by ~1 s of SM clock; the other
// threads meet the waiting thread at the next barrier.  An expired wait sets
// an abort flag, the CTA stops its chain, waits (bounded) for its copies and
// gives its MMAs time to finish, frees its TMEM, and the timeout is recorded
// in the status.
#pragma once

namespace bss {

constexpr int C128_THREADS = 256;
constexpr int C128_LD = Geo<float, 128>::LD;              // 132
constexpr int C128_RLD = 132;                             // row stride of the carried operands (floats)
constexpr int C128_MAT = 128 * C128_LD * 4;               // 67584: one padded 128 x 128 FP32 matrix
constexpr int C128_PART = 128 * 16 * 4;                   // 8192: one split part of a K = 16 chunk
constexpr int C128_STAGE1 = 4 * C128_PART;                // W hi, W lo, Y hi, Y lo
constexpr int C128_STAGE2 = 6 * C128_PART;                // Z hi, Z lo, B hi, B lo, V hi, V lo
constexpr int C128_OFF_Y = 0;                             // carried Y / sV
constexpr int C128_OFF_X = C128_MAT;                      // carried W / sS / phase-2 stages
constexpr int C128_OFF_S1 = 2 * C128_MAT;                 // phase-1 stages
constexpr int C128_ACH = 16 * 128 * 8;                   // one A_i column chunk (16 FP64 columns)
constexpr int C128_BCH = 16 * 128 * 8;                   // one B_i row chunk: 128 columns x 16 rows (FP64)
constexpr int C128_NBBUF = 3;                             // B_i chunks in flight
constexpr int C128_OFF_B = C128_OFF_X + 2 * C128_STAGE2;  // B_i chunk buffers (Cholesky, phase 2)
constexpr int C128_OFF_A0 = C128_OFF_S1 + 2 * C128_STAGE1;  // A_i chunk 0 (phase 1)
constexpr int C128_OFF_CTL = C128_OFF_B + C128_NBBUF * C128_BCH > C128_OFF_A0 + C128_ACH
                                 ? C128_OFF_B + C128_NBBUF * C128_BCH
                                 : C128_OFF_A0 + C128_ACH;
constexpr int C128_NCHUNK = 8;                            // K = 128 in chunks of 16
constexpr uint32_t C128_T_SLL = 0, C128_T_D1 = 128, C128_T_D2 = 256, C128_T_DW = 384;  // TMEM columns
static_assert(C128_OFF_A0 + C128_ACH <= C128_OFF_CTL, "A chunk 0 below the control words");
static_assert(C128_OFF_B % 1024 == 0 && C128_BCH % 1024 == 0, "128-byte-swizzled TMA boxes start on 1024 bytes");

// byte offset of logical byte `off` of a box that the tensor copy wrote with
// the 128-byte swizzle: the 16-byte unit index (bits 4-6) XOR the 128-byte
// row index (bits 7-9)
__device__ __forceinline__ uint32_t c128_swz(uint32_t off) { return off ^ (((off >> 7) & 7u) << 4); }

// one 2D tensor copy (box of the tensor map at element coordinates x = row,
// y = column) into shared memory, completing on the mbarrier
__device__ __forceinline__ void tma_load_2d(uint32_t dst, const CUtensorMap *map, int x, int y, uint32_t mbar)
{
    asm volatile(
        "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], [%4];" ::"r"(dst),
        "l"(reinterpret_cast<uint64_t>(map)), "r"(x), "r"(y), "r"(mbar)
        : "memory");
}
static_assert(4 * C128_ACH <= C128_MAT && C128_OFF_S1 + 3 * C128_ACH <= C128_OFF_S1 + 2 * C128_STAGE1,
              "A chunks 1-7 fit the carried-Y region and the phase-1 stages");

// shared-memory offset of A_i column chunk j: chunk 0 has a buffer of its
// own (it lands while phase 1 still holds the other regions), chunks 1-4
// take the carried-Y region and 5-7 the phase-1 stages once phase 1 is done
__host__ __device__ constexpr int c128_achunk(int j)
{
    return j == 0 ? C128_OFF_A0 : (j <= 4 ? C128_OFF_Y + (j - 1) * C128_ACH : C128_OFF_S1 + (j - 5) * C128_ACH);
}

// thread 0: bounded wait on the mbarrier at `addr` whose outstanding parity
// is bit j of `phase` when bit j of `pending` is set; sets *abort on expiry
__device__ __forceinline__ void c128_waitbit(uint32_t addr, int j, uint32_t &phase, uint32_t &pending, int *abort)
{
    if (!((pending >> j) & 1u)) return;
    const long long t0 = clock64();
    for (;;) {
        if (mbar_test(addr, (phase >> j) & 1u)) {
            phase ^= 1u << j;
            pending &= ~(1u << j);
            return;
        }
        if (clock64() - t0 > C64_WAIT_CYCLES) {
            *abort = 1;
            return;
        }
    }
}

constexpr size_t chain128_tc_smem() { return (size_t)C128_OFF_CTL + 1024; }

// byte offset of (row m, K group k4 .. k4+3) in one part of a stage
__device__ __forceinline__ uint32_t c128_off(int m, int k4)
{
    return (uint32_t)((m >> 3) * 512 + (k4 >> 2) * 128 + (m & 7) * 16);
}

__device__ __forceinline__ uint64_t c128_desc(uint32_t saddr)
{
    uint64_t d = (uint64_t)((saddr & 0x3FFFFu) >> 4);
    d |= (uint64_t)(128u >> 4) << 16;  // leading byte offset: next core matrix along K
    d |= (uint64_t)(512u >> 4) << 32;  // stride byte offset: next 8-row group
    d |= (uint64_t)1 << 46;            // descriptor version of the sm_100 family
    return d;
}

// TMEM cols at tm (+)= A x B^T over one K = 16 chunk in 3xTF32 (parts at
// shared addresses ah/al, bh/bl); issued by one thread
__device__ __forceinline__ void c128_mma16(uint32_t tm, uint32_t ah, uint32_t al, uint32_t bh, uint32_t bl,
                                           bool accumulate)
{
    constexpr uint32_t id = tc_idesc_128x128();
#pragma unroll
    for (int kk = 0; kk < 2; ++kk) {
        const uint32_t o = (uint32_t)kk * 256u;  // K = 8: two core matrices along K
        tc_mma(tm, c128_desc(ah + o), c128_desc(bh + o), id, (accumulate || kk) ? 1u : 0u);
        tc_mma(tm, c128_desc(ah + o), c128_desc(bl + o), id, 1u);
        tc_mma(tm, c128_desc(al + o), c128_desc(bh + o), id, 1u);
    }
}

// four values split into hi / lo TF32 parts, stored at part offset o
__device__ __forceinline__ void c128_put4(unsigned char *hi, unsigned char *lo, uint32_t o, float a, float b, float c,
                                          float d)
{
    const uint32_t h0 = to_tf32(a), h1 = to_tf32(b), h2 = to_tf32(c), h3 = to_tf32(d);
    *reinterpret_cast<uint4 *>(hi + o) = make_uint4(h0, h1, h2, h3);
    *reinterpret_cast<uint4 *>(lo + o) =
        make_uint4(to_tf32(a - __uint_as_float(h0)), to_tf32(b - __uint_as_float(h1)),
                   to_tf32(c - __uint_as_float(h2)), to_tf32(d - __uint_as_float(h3)));
}

// 8 consecutive accumulator columns of this thread's TMEM lane
__device__ __forceinline__ void c128_ld8(uint32_t addr, float (&v)[8])
{
    uint32_t r[8];
    asm volatile("tcgen05.ld.sync.aligned.32x32b.x8.b32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%8];"
                 : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7])
                 : "r"(addr));
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
    for (int q = 0; q < 8; ++q) v[q] = __uint_as_float(r[q]);
}

// column-major n x n block from the carried rows (row m = column m)
__device__ __forceinline__ void c128_store_block(float *dst, const float *raw, int n, int tid)
{
    if (n == 128) {
        for (int e = tid; e < 128 * 32; e += C128_THREADS) {
            const int m = e >> 5, k4 = (e & 31) * 4;
            *reinterpret_cast<float4 *>(dst + m * 128 + k4) = *reinterpret_cast<const float4 *>(raw + m * C128_RLD + k4);
        }
    } else {
        for (int e = tid; e < n * n; e += C128_THREADS) {
            const int m = e / n, k = e - m * n;
            dst[e] = raw[m * C128_RLD + k];
        }
    }
}

// bounded wait for the mbarrier phase of the given parity; sets *abort on expiry
__device__ __forceinline__ void c128_wait_parity(uint32_t mb, uint32_t parity, int *abort)
{
    const long long t0 = clock64();
    while (!mbar_test(mb, parity))
        if (clock64() - t0 > C64_WAIT_CYCLES) {
            *abort = 1;
            return;
        }
}

__device__ __forceinline__ void c128_converters_sync() { asm volatile("bar.sync 2, 224;" ::: "memory"); }

// One product phase (C128_NCHUNK chunks through two stages) with the MMA issue
// apart from the operand split: warp 0 only issues (tcgen05.mma blocks the
// issuing thread for the MMA's duration), warps 1-7 split chunk c + 1 into
// the other stage while the tensor core works on chunk c.  Before that split,
// thread 32 waits for the MMAs of chunk c - 1 (they read that stage) and, with
// `ready`, for anything else the split needs; a named barrier then joins the
// 224 converter threads.  Every phase has 8 chunks, so the commit of chunk c
// on stage c & 1 completes the mbarrier phase of parity (c >> 1) & 1, and each
// stage's waits run in order (none waits two phases ahead).  conv(c) runs on
// the converter threads, issue(c) on thread 0 (its commit follows), after(c)
// on every thread once chunk c + 1 is split (after(-1): chunk 0).  Returns false (in every thread)
// when a wait expired; on return every MMA of the phase is complete.
template <class Ready, class Conv, class Issue, class After>
__device__ __forceinline__ bool c128_pipeline(const uint32_t (&mb)[2], int *abort, int tid, Ready ready, Conv conv,
                                              Issue issue, After after)
{
    const int w = tid >> 5;
    // iteration c issues chunk c (c >= 0) and splits chunk c + 1; one call site
    // each, so the heavy split code is inlined once
#pragma unroll 1
    for (int c = -1; c < C128_NCHUNK; ++c) {
        if (c >= 0 && tid == 0) {
            tc_fence_after();
            issue(c);
            tc_commit(mb[c & 1]);
        }
        if (w != 0 && c + 1 < C128_NCHUNK) {
            if (tid == 32) {
                if (c >= 1) c128_wait_parity(mb[(c + 1) & 1], (uint32_t)(((c - 1) >> 1) & 1), abort);
                ready(c + 1);
            }
            c128_converters_sync();
            conv(c + 1);
            fence_async_smem();  // generic-proxy stores -> visible to the tensor core
        }
        tc_fence_before();
        __syncthreads();
        if (*abort) return false;
        after(c);
    }
    if (tid == 0) {  // the last commits on both stages: chunks 6 and 7
        c128_wait_parity(mb[0], (uint32_t)(((C128_NCHUNK - 2) >> 1) & 1), abort);
        c128_wait_parity(mb[1], (uint32_t)(((C128_NCHUNK - 1) >> 1) & 1), abort);
    }
    __syncthreads();
    tc_fence_after();
    return *abort == 0;
}

// phase 1 on the carried rows: D1 = W^T W, D2 = Y^T W, S_LL (+)= Y^T Y.
// Thread 0 calls rows_read() once the last chunk is split (the carried rows
// are free; the stages are not, until the phase ends).  Returns false (in
// every thread) when a wait expired; on return the products are complete in TMEM.
template <class F>
__device__ __forceinline__ bool c128_phase1(uint32_t tm, const float *rawW, const float *rawY, unsigned char *stages,
                                            uint32_t stages_addr, const uint32_t (&mb)[2], int *abort, bool sll,
                                            int tid, F rows_read)
{
    return c128_pipeline(
        mb, abort, tid, [](int) {},
        [&](int c) {
            unsigned char *st = stages + (c & 1) * C128_STAGE1;
            for (int e = tid - 32; e < 512; e += C128_THREADS - 32) {
                const int m = e & 127, q = e >> 7;
                const uint32_t o = c128_off(m, 4 * q);
                const float4 wv = *reinterpret_cast<const float4 *>(rawW + m * C128_RLD + 16 * c + 4 * q);
                const float4 yv = *reinterpret_cast<const float4 *>(rawY + m * C128_RLD + 16 * c + 4 * q);
                c128_put4(st, st + C128_PART, o, wv.x, wv.y, wv.z, wv.w);
                c128_put4(st + 2 * C128_PART, st + 3 * C128_PART, o, yv.x, yv.y, yv.z, yv.w);
            }
        },
        [&](int c) {
            const uint32_t a = stages_addr + (uint32_t)((c & 1) * C128_STAGE1);
            const uint32_t wh = a, wl = a + C128_PART, yh = a + 2 * C128_PART, yl = a + 3 * C128_PART;
            c128_mma16(tm + C128_T_D1, wh, wl, wh, wl, c > 0);
            c128_mma16(tm + C128_T_D2, yh, yl, wh, wl, c > 0);
            c128_mma16(tm + C128_T_SLL, yh, yl, yh, yl, sll || c > 0);
        },
        [&](int c) {
            if (c == C128_NCHUNK - 2 && tid == 0) rows_read();  // the last chunk is split: the rows are free
        });
}

template <class Tin>
__global__ void __launch_bounds__(C128_THREADS, 1)
    chain128_tc_kernel(ChainFactorArgs<Tin, float> g, const __grid_constant__ CUtensorMap tmB, int tma_b)
{
    constexpr int LD = C128_LD;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    float *rawY = reinterpret_cast<float *>(smem_raw + C128_OFF_Y);
    float *sV = rawY;
    float *rawW = reinterpret_cast<float *>(smem_raw + C128_OFF_X);
    float *sS = rawW;
    unsigned char *ctl = smem_raw + C128_OFF_CTL;
    float *dinv = reinterpret_cast<float *>(ctl);  // 128 pivot reciprocals
    float *prow = dinv + 128;                      // 64 floats: the Cholesky's pivot-row buffer
    int *sflag = reinterpret_cast<int *>(ctl + 768);
    uint32_t *tslot = reinterpret_cast<uint32_t *>(ctl + 772);
    int *abort = reinterpret_cast<int *>(ctl + 776);
    uint64_t *mbars = reinterpret_cast<uint64_t *>(ctl + 784);  // stages 0-1, A chunks 2-9, B chunks 10-12

    const int tid = threadIdx.x, w = tid >> 5, lane = tid & 31;
    const int L = 32 * (w & 3) + lane;  // this thread's TMEM lane (accumulator row)
    const int cb = 64 * (w >> 2);       // its first accumulator column
    const uint32_t lane_base = (uint32_t)(32 * (w & 3)) << 16;
    const int n = g.n;
    const long long nn = (long long)n * n;
    const bool aligned = ((uintptr_t)g.A_in % 16u) == 0 && ((uintptr_t)g.B_in % 16u) == 0;
    // bulk copies of column chunks (A) and the tensor copies of row chunks (B)
    // start on 16 bytes; the latter also need the 1024-byte-aligned buffers
    const bool bulk = aligned && (sizeof(Tin) == 8 ? n % 2 == 0 : n % 4 == 0);
    const bool tmab = sizeof(Tin) == 8 && bulk && tma_b != 0 && ((smem_u32(smem_raw) + C128_OFF_B) & 1023u) == 0;

    if (w == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(tslot)),
                     "r"(512u)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    if (tid == 0) {
        for (int q = 0; q < 2 + C128_NCHUNK + C128_NBBUF; ++q)
            asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(&mbars[q])) : "memory");
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        *abort = 0;
    }
    fence_async_smem();
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tm = *tslot;
    const uint32_t base_addr = smem_u32(smem_raw);
    const uint32_t mbA = smem_u32(&mbars[2]), mbB = smem_u32(&mbars[2 + C128_NCHUNK]);
    const uint32_t mbs[2] = {smem_u32(&mbars[0]), smem_u32(&mbars[1])};  // stage barriers (MMA commits)
    // thread 0's view of the stage barriers in phase 2 (phase 1 leaves each
    // with an even number of completed phases, so the parities agree) and of
    // the copy mbarriers
    C64Bar bar[2] = {{mbs[0], 0u, false}, {mbs[1], 0u, false}};
    uint32_t a_phase = 0, a_pend = 0, b_phase = 0, b_pend = 0;
    const int rm = tid & 127, rq = tid >> 7;  // phase-2 converter mapping: operand row, K group

    // thread 0: A_i column chunk j (16 columns, contiguous) into its buffer
    auto issue_a = [&](const Tin *Ag, int j) {
        const int cols = min(16, n - 16 * j);
        if (cols <= 0) return;
        const uint32_t bytes = (uint32_t)(cols * n) * (uint32_t)sizeof(Tin);
        const uint32_t mb = mbA + 8u * (uint32_t)j;
        mbar_expect_tx(mb, bytes);
        bulk_g2s(base_addr + (uint32_t)c128_achunk(j), Ag + (long long)16 * j * n, bytes, mb);
        a_pend |= 1u << j;
    };
    // thread 64: B_i row chunk c (rows 16 c .. +15 of the block's 128 columns)
    // into buffer c % 3 with one tensor copy; thread 0 marks it outstanding
    auto issue_b = [&](long long blk, int c) {
        if (16 * c >= n) return;
        const int b = c % C128_NBBUF;
        const uint32_t mb = mbB + 8u * (uint32_t)b;
        if (tid == 64) {
            fence_async_smem();
            mbar_expect_tx(mb, (uint32_t)(16 * 128 * sizeof(Tin)));  // the whole box, zero-filled parts included
            tma_load_2d(base_addr + (uint32_t)(C128_OFF_B + b * C128_BCH), &tmB, 16 * c, (int)(blk * n), mb);
        }
        if (tid == 0) b_pend |= 1u << b;
    };

    // partitions p = blockIdx.x, + gridDim.x, ... (the grid is at most one CTA per SM)
    for (long long p = blockIdx.x; p < g.Q && !*abort; p += gridDim.x) {
    const long long sL = (p * (g.N - 1)) / g.Q;
    const long long sR = ((p + 1) * (g.N - 1)) / g.Q;
    const long long first = sL + 1, last = sR - 1;
    bool sll = false;
    for (long long i = first; i <= last; ++i) {
        const long long t = i - first;
        const Tin *Ag = g.A_in + i * nn;
        const Tin *Bg = g.B_in + i * nn;
        // A_i's first chunk has a buffer of its own; at a chain's first step
        // (no phase 1) every chunk's buffer is free
        if (tid == 0 && bulk) {
            fence_async_smem();
            issue_a(Ag, 0);
            if (t == 0)
                for (int j = 1; j < C128_NCHUNK; ++j) issue_a(Ag, j);
        }
        // ---- phase 1: D1 = W^T W, D2 = Y^T W, S_LL += Y^T Y on the carried rows
        if (t > 0) {
            auto rows_read = [&]() {  // thread 0: the carried-Y region takes A chunks 1-4
                if (bulk) {
                    fence_async_smem();
                    for (int j = 1; j <= 4; ++j) issue_a(Ag, j);
                }
            };
            if (!c128_phase1(tm, rawW, rawY, smem_raw + C128_OFF_S1, base_addr + C128_OFF_S1, mbs, abort, sll, tid,
                             rows_read))
                break;
            sll = true;
            if (tid == 0 && bulk)  // the drained phase-1 stages take A chunks 5-7
                for (int j = 5; j < C128_NCHUNK; ++j) issue_a(Ag, j);
        }
        // ---- Ahat_i = A_i - D1 into sS (identity outside n x n); sS overlays the carried W, read by now
        if (bulk) {
            // chunk by chunk as the copies land: this thread's row L, 8 columns of the chunk
            const int h = w >> 2;
#pragma unroll 1
            for (int j = 0; j < C128_NCHUNK; ++j) {
                if (tid == 0) c128_waitbit(mbA + 8u * (uint32_t)j, j, a_phase, a_pend, abort);
                __syncthreads();
                if (*abort) break;
                const int c0 = 16 * j + 8 * h;
                float d[8];
                if (t > 0) {
                    c128_ld8(tm + lane_base + C128_T_D1 + (uint32_t)c0, d);
                } else {
#pragma unroll
                    for (int u = 0; u < 8; ++u) d[u] = 0.f;
                }
                const Tin *ach = reinterpret_cast<const Tin *>(smem_raw + c128_achunk(j));
#pragma unroll
                for (int u = 0; u < 8; ++u) {
                    const int c = c0 + u;
                    sS[L + c * LD] = (L < n && c < n) ? f64_to_f32(ach[(c - 16 * j) * n + L]) - d[u] : (L == c ? 1.f : 0.f);
                }
            }
            if (*abort) break;
        } else {
#pragma unroll 1
            for (int hf = 0; hf < 2; ++hf) {
                const int c0 = cb + 32 * hf;
                // every load is issued (clamped to a valid address) before any is used
                Tin ga[32];
#pragma unroll
                for (int q = 0; q < 32; ++q) {
                    const int c = c0 + q;
                    ga[q] = __ldcg(Ag + ((L < n && c < n) ? L + (long long)c * n : 0));
                }
                float d[32];
                if (t > 0) {
                    c64_ld32(tm + lane_base + C128_T_D1 + (uint32_t)c0, d);
                } else {
#pragma unroll
                    for (int q = 0; q < 32; ++q) d[q] = 0.f;
                }
#pragma unroll
                for (int q = 0; q < 32; ++q) {
                    const int c = c0 + q;
                    sS[L + c * LD] = (L < n && c < n) ? f64_to_f32(ga[q]) - d[q] : (L == c ? 1.f : 0.f);
                }
            }
        }
        __syncthreads();
        // B_i's first chunks land during the Cholesky (the A chunk buffers are read)
        if (tmab)
            for (int c = 0; c < C128_NBBUF; ++c) issue_b(i, c);
        // ---- U^T U = Ahat, V = U^-1 (CUDA cores; ends with a CTA barrier)
        const int bad = chol_inv_blocked<float, 128, C128_THREADS, true, true>(sS, sV, dinv, sflag, tid, prow);
        if (bad && tid == 0) record_bad_pivot(g.st, g.level, i);
        // ---- phase 2: D1 = Z^T V = Y_i^T, DW = B^T V = W_i^T
        {
            const Tin *Bs = g.B_in + sL * nn;  // Z_first = B_sL^T
#pragma unroll 1
            for (int c = 0; c < C128_NCHUNK; ++c) {
                const int s = c & 1, bb = c % C128_NBBUF;
                if (tid == 0) {
                    c64_wait1(bar[s], abort);
                    if (tmab) c128_waitbit(mbB + 8u * (uint32_t)bb, bb, b_phase, b_pend, abort);
                }
                tc_fence_before();
                __syncthreads();
                if (*abort) break;
                unsigned char *st = smem_raw + C128_OFF_X + s * C128_STAGE2;
                // V: op(V) row m = column m of V (zero below the diagonal tiles)
#pragma unroll
                for (int hq = 0; hq < 2; ++hq) {
                    const int q = rq + 2 * hq, k = 16 * c + 4 * q;
                    float4 v = *reinterpret_cast<const float4 *>(sV + k + rm * LD);
                    if ((k >> 4) > (rm >> 4)) v = make_float4(0.f, 0.f, 0.f, 0.f);
                    c128_put4(st + 4 * C128_PART, st + 5 * C128_PART, c128_off(rm, 4 * q), v.x, v.y, v.z, v.w);
                }
                // B: op(B) row m = column m of B_i, rows 16 c + 8 rq .. +7
                {
                    float bv[8];
                    if (tmab) {
                        // column rm of the box, values 8 rq .. 8 rq + 7 (zero-filled outside the block)
                        const unsigned char *buf = smem_raw + C128_OFF_B + bb * C128_BCH;
#pragma unroll
                        for (int u = 0; u < 8; u += 16 / (int)sizeof(Tin)) {
                            const uint32_t off = (uint32_t)((rm * 16 + 8 * rq + u) * (int)sizeof(Tin));
                            const uint4 raw = *reinterpret_cast<const uint4 *>(buf + c128_swz(off));
                            if constexpr (sizeof(Tin) == 8) {
                                bv[u] = f64_to_f32(__hiloint2double((int)raw.y, (int)raw.x));
                                bv[u + 1] = f64_to_f32(__hiloint2double((int)raw.w, (int)raw.z));
                            } else {
                                bv[u] = __uint_as_float(raw.x);
                                bv[u + 1] = __uint_as_float(raw.y);
                                bv[u + 2] = __uint_as_float(raw.z);
                                bv[u + 3] = __uint_as_float(raw.w);
                            }
                        }
#pragma unroll
                        for (int u = 0; u < 8; ++u)
                            if (rm >= n || 16 * c + 8 * rq + u >= n) bv[u] = 0.f;
                    } else {
                        Tin gb[8];
#pragma unroll
                        for (int u = 0; u < 8; ++u) {
                            const int k = 16 * c + 8 * rq + u;
                            gb[u] = __ldg(Bg + ((rm < n && k < n) ? k + (long long)rm * n : 0));
                        }
#pragma unroll
                        for (int u = 0; u < 8; ++u) {
                            const int k = 16 * c + 8 * rq + u;
                            bv[u] = (rm < n && k < n) ? f64_to_f32(gb[u]) : 0.f;
                        }
                    }
#pragma unroll
                    for (int hq = 0; hq < 2; ++hq)
                        c128_put4(st + 2 * C128_PART, st + 3 * C128_PART, c128_off(rm, 8 * rq + 4 * hq), bv[4 * hq],
                                  bv[4 * hq + 1], bv[4 * hq + 2], bv[4 * hq + 3]);
                }
                // Z: op(Z) row m = column m of Z_i = -(row m of D2); Z_first = B_sL^T
                {
                    const int kz = 8 * (w >> 2);
                    float z[8];
                    if (t > 0) {
                        c128_ld8(tm + lane_base + C128_T_D2 + (uint32_t)(16 * c + kz), z);
#pragma unroll
                        for (int u = 0; u < 8; ++u) z[u] = -z[u];
                    } else {
#pragma unroll
                        for (int u = 0; u < 8; ++u) {
                            const int k = 16 * c + kz + u;
                            z[u] = (L < n && k < n) ? f64_to_f32(__ldcg(Bs + L + (long long)k * n)) : 0.f;
                        }
                    }
                    c128_put4(st, st + C128_PART, c128_off(L, kz), z[0], z[1], z[2], z[3]);
                    c128_put4(st, st + C128_PART, c128_off(L, kz + 4), z[4], z[5], z[6], z[7]);
                }
                fence_async_smem();
                __syncthreads();
                if (tid == 0) {
                    tc_fence_after();
                    const uint32_t a = base_addr + C128_OFF_X + (uint32_t)(s * C128_STAGE2);
                    const uint32_t zh = a, zl = a + C128_PART, bh = a + 2 * C128_PART, bl = a + 3 * C128_PART;
                    const uint32_t vh = a + 4 * C128_PART, vl = a + 5 * C128_PART;
                    c128_mma16(tm + C128_T_D1, zh, zl, vh, vl, c > 0);
                    c128_mma16(tm + C128_T_DW, bh, bl, vh, vl, c > 0);
                    tc_commit(bar[s].addr);
                    bar[s].pending = true;
                }
                // the B buffer just split takes the chunk three ahead
                if (tmab && c + C128_NBBUF < C128_NCHUNK) issue_b(i, c + C128_NBBUF);
            }
        }
        if (tid == 0) {
            c64_wait1(bar[0], abort);
            c64_wait1(bar[1], abort);
        }
        __syncthreads();
        if (*abort) break;
        tc_fence_after();
        // ---- V_i to HBM in whole lines (column m of V is column m of sV; zero below the diagonal tiles)
        {
            float *Vg = g.A_f + i * nn;
            if (n == 128) {
                for (int e = tid; e < 128 * 32; e += C128_THREADS) {
                    const int m = e >> 5, k4 = (e & 31) * 4;
                    float4 v = *reinterpret_cast<const float4 *>(sV + k4 + m * LD);
                    if ((k4 >> 4) > (m >> 4)) v = make_float4(0.f, 0.f, 0.f, 0.f);
                    *reinterpret_cast<float4 *>(Vg + m * 128 + k4) = v;
                }
            } else {
                for (int e = tid; e < n * n; e += C128_THREADS) {
                    const int m = e / n, k = e - m * n;
                    Vg[e] = ((k >> 4) > (m >> 4)) ? 0.f : sV[k + m * LD];
                }
            }
        }
        __syncthreads();  // sV is read: the carried Y rows take its place
        // ---- Y_i, W_i: TMEM rows -> carried rows (next step's operands) -> HBM
#pragma unroll 1
        for (int hf = 0; hf < 2; ++hf) {
            const int c0 = cb + 32 * hf;
            float d[32];
            c64_ld32(tm + lane_base + C128_T_D1 + (uint32_t)c0, d);
#pragma unroll
            for (int q = 0; q < 32; q += 4)
                *reinterpret_cast<float4 *>(rawY + L * C128_RLD + c0 + q) = make_float4(d[q], d[q + 1], d[q + 2], d[q + 3]);
            c64_ld32(tm + lane_base + C128_T_DW + (uint32_t)c0, d);
#pragma unroll
            for (int q = 0; q < 32; q += 4)
                *reinterpret_cast<float4 *>(rawW + L * C128_RLD + c0 + q) = make_float4(d[q], d[q + 1], d[q + 2], d[q + 3]);
        }
        __syncthreads();
        c128_store_block(g.Y + i * nn, rawY, n, tid);
        c128_store_block(g.B_f + i * nn, rawW, n, tid);
    }

    // ---- chain end: S_RR = W^T W (D1), S_LR = Y^T W (D2), S_LL += Y^T Y
    if (!*abort && first <= last) {
        if (c128_phase1(tm, rawW, rawY, smem_raw + C128_OFF_S1, base_addr + C128_OFF_S1, mbs, abort, sll, tid,
                        []() {})) {
            float *Cp = g.C + p * 3 * nn;
#pragma unroll 1
            for (int hf = 0; hf < 2; ++hf) {
                const int c0 = cb + 32 * hf;
#pragma unroll 1
                for (int r = 0; r < 3; ++r) {  // S_LL, S_RR, S_LR
                    const uint32_t col = r == 0 ? C128_T_SLL : (r == 1 ? C128_T_D1 : C128_T_D2);
                    float d[32];
                    c64_ld32(tm + lane_base + col + (uint32_t)c0, d);
                    float *dst = Cp + r * nn;
                    if (L < n) {
#pragma unroll
                        for (int q = 0; q < 32; ++q)
                            if (c0 + q < n) dst[L + (long long)(c0 + q) * n] = d[q];
                    }
                }
            }
        }
    }
    __syncthreads();
    }  // partitions
    __syncthreads();
    if (*abort && tid == 0) {
        // a wait gave up: wait (bounded) for this CTA's copies in flight and
        // give its MMAs time to finish before shared memory and TMEM are released
        int ignored = 0;
        for (int j = 0; j < C128_NCHUNK; ++j) c128_waitbit(mbA + 8u * (uint32_t)j, j, a_phase, a_pend, &ignored);
        for (int b = 0; b < C128_NBBUF; ++b) c128_waitbit(mbB + 8u * (uint32_t)b, b, b_phase, b_pend, &ignored);
        const long long t0 = clock64();
        while (clock64() - t0 < C64_WAIT_CYCLES / 8) {
        }
        if (g.st) atomicExch(&g.st->tc_timeout, 1);
    }

    tc_fence_before();
    __syncthreads();
    if (w == 0) {
        tc_fence_after();
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tm), "r"(512u) : "memory");
    }
}

}  // namespace bss
