// Chain factor kernel for 64-wide blocks (n in 33..64) with FP32 factors on
// the 5th-generation tensor cores: one CTA walks one partition's chain like
// chain_factor_body (same recursion, same outputs V_i, W_i, Y_i and
// S_LL / S_RR / S_LR), with every product of a chain step on tcgen05.mma and
// the block loads on the bulk-copy (TMA) engine.
//
// Products (K = 64, 3xTF32: x = hi + lo, C = Xh Yh + Xh Yl + Xl Yh in the FP32
// TMEM accumulator, relative error ~2^-21 like FP32 FMA products).  The A
// operand of each stacks two 64-row operands (M = 128):
//   P1 = [W_{i-1} | Y_{i-1}]^T [W_{i-1} | Y_{i-1}]   (N = 128)
//        columns 0-63,   rows 0-63:   W^T W  -> Ahat_i = A_i - W^T W
//        columns 0-63,   rows 64-127: Y^T W  -> Z_i = -(Y^T W)^T
//        columns 64-127, rows 64-127: Y^T Y, accumulated in TMEM over the
//        chain (S_LL); rows 0-63 unused
//   P2 = [Z_i | B_i]^T V_i                   (N = 64)
//        rows 0-63:   Z^T V = Y_i^T
//        rows 64-127: B^T V = W_i^T
// and at the chain end P1 on [W_last | Y_last] gives S_RR = W^T W and
// S_LR = Y^T W with the last S_LL term.  P1 accumulates onto all 128
// columns (one MMA sequence cannot overwrite some columns and accumulate
// others), so the readout of P2 stores zeros into columns 0-63 behind it.  Reference: the potrf/trsm/gemm sequence of
// cholesky_factorize_batched! and the Schur products of
// compute_schur_complement! (src/backbone_cuda.jl:70-101, 143-157).
//
// Shared memory (108.6 KB: two CTAs per SM):
//   R   72 KB  the stacked A operand in the no-swizzle K-major layout of
//              8-row x 16-byte core matrices, with the hi and lo parts
//              interleaved per 8-row group: element (row, k) of part h at
//              (row/8)*4608 + h*2304 + (k/4)*144 + (row%8)*16 + (k%4)*4
//              (leading byte offset 144, stride byte offset 4608).  The core
//              matrices of a row group sit 144 bytes apart instead of 128, so
//              eight threads writing the same row at eight consecutive k
//              groups hit eight different bank groups (with 128 they would
//              all hit one).  Rows 64-127 (hi and lo) are the contiguous upper
//              36 KB, where B_i lands raw from HBM before conversion
//   VR  36 KB  the Cholesky tiles sS, sV (padded column-major, as
//              chol_inv_blocked wants them); after the Cholesky the V operand
//              (same layout); between steps the raw A_{i+1}
// TMEM: 128 columns: 0-63 the P1/P2 accumulator, 64-127 S_LL (P1's second half).
//
// Block loads: A_{i+1} (into VR, issued once P2 of step i has read V) and
// B_i (into R's upper half, issued once P1 of step i has read R) are single
// cp.async.bulk copies completing on mbarriers; both blocks are prefetched
// into L2 (cp.async.bulk.prefetch.L2) a whole step ahead.  Blocks whose byte
// size is not a multiple of 16 (odd n) are read with plain loads instead.
// Their FP64 -> FP32 conversions run where warps 1-7 would otherwise wait:
// A_i into the Cholesky tile sS while thread 0 issues P1, and B_i into
// its operand rows while warp 0 factors the first diagonal tile of the
// Cholesky (both in place: every raw value is read into registers before the
// named barrier 2 lets the first converted one be written).
//
// Thread 0 issues every MMA and is the only thread that waits on the MMA
// mbarrier; thread 32 issues the bulk copies and is the only thread that
// waits on theirs (each a spin on mbarrier.test_wait, bounded by ~1 s of SM
// clock); the other threads meet them at the next CTA or named barrier
// instead of polling.  An expired wait sets an abort flag, the CTA stops its
// chain, threads 0 and 32 wait (bounded) for the MMAs and copies still in
// flight, the CTA frees its TMEM and the timeout is recorded in the status.
#pragma once

namespace bss {

constexpr int C64_LBO = 144;                    // next core matrix along K
constexpr int C64_PART = 16 * C64_LBO;          // the lo part of a row group: 2304
constexpr int C64_SBO = 2 * C64_PART;           // next 8-row group: 4608
constexpr int C64_UPPER = 8 * C64_SBO;          // rows 64-127: 36864
constexpr int C64_R_BYTES = 16 * C64_SBO;       // 73728
constexpr int C64_VR_BYTES = 8 * C64_SBO;       // 36864 >= sS + sV (34816), >= a raw FP64 block (32768)
constexpr int C64_THREADS = 256;

constexpr size_t chain64_tc_smem() { return (size_t)C64_R_BYTES + C64_VR_BYTES + 512 + 64; }

__device__ __forceinline__ uint32_t c64_off(int row, int k, int part)
{
    return (uint32_t)((row >> 3) * C64_SBO + part * C64_PART + (k >> 2) * C64_LBO + (row & 7) * 16 + (k & 3) * 4);
}

__device__ __forceinline__ uint64_t c64_desc(uint32_t saddr)
{
    uint64_t d = (uint64_t)((saddr & 0x3FFFFu) >> 4);
    d |= (uint64_t)(C64_LBO >> 4) << 16;  // leading byte offset: next core matrix along K
    d |= (uint64_t)(C64_SBO >> 4) << 32;  // stride byte offset: next 8-row group
    d |= (uint64_t)1 << 46;               // descriptor version of the sm_100 family
    return d;
}

// kind::tf32, D = F32, A = B = TF32, both K-major, M = 128, N = 64
__host__ __device__ constexpr uint32_t c64_idesc()
{
    return (1u << 4) | (2u << 7) | (2u << 10) | ((64u >> 3) << 17) | ((128u >> 4) << 24);
}

// kind::tf32, D = F32, A = B = TF32, both K-major, M = 128, N = 128
__host__ __device__ constexpr uint32_t c64_idesc_n128()
{
    return (1u << 4) | (2u << 7) | (2u << 10) | ((128u >> 3) << 17) | ((128u >> 4) << 24);
}

// TMEM cols at tm (+)= Aop(128 rows at shared address a) x Bop(64 rows at b)^T
// over K = 64 in 3xTF32; issued by one thread
__device__ __forceinline__ void c64_mma(uint32_t tm, uint32_t a, uint32_t b, bool accumulate)
{
    constexpr uint32_t id = c64_idesc();
#pragma unroll
    for (int kk = 0; kk < 8; ++kk) {
        const uint32_t o = (uint32_t)kk * (2u * C64_LBO);  // K = 8: two core matrices along K
        const uint64_t ah = c64_desc(a + o), al = c64_desc(a + C64_PART + o);
        const uint64_t bh = c64_desc(b + o), bl = c64_desc(b + C64_PART + o);
        tc_mma(tm, ah, bh, id, (accumulate || kk) ? 1u : 0u);
        tc_mma(tm, ah, bl, id, 1u);
        tc_mma(tm, al, bh, id, 1u);
    }
}

// TMEM cols tm .. tm+127 (+)= R x R^T over K = 64 in 3xTF32 (R: the 128 stacked
// operand rows at shared address r, as both A and B); issued by one thread
__device__ __forceinline__ void c64_mma_rr(uint32_t tm, uint32_t r, bool accumulate)
{
    constexpr uint32_t id = c64_idesc_n128();
#pragma unroll
    for (int kk = 0; kk < 8; ++kk) {
        const uint32_t o = (uint32_t)kk * (2u * C64_LBO);
        const uint64_t h = c64_desc(r + o), l = c64_desc(r + C64_PART + o);
        tc_mma(tm, h, h, id, (accumulate || kk) ? 1u : 0u);
        tc_mma(tm, h, l, id, 1u);
        tc_mma(tm, l, h, id, 1u);
    }
}

// zeros into 32 consecutive accumulator columns of this thread's TMEM lane
__device__ __forceinline__ void c64_zero32(uint32_t addr)
{
    asm volatile(
        "tcgen05.st.sync.aligned.32x32b.x32.b32 [%0], {%1,%1,%1,%1,%1,%1,%1,%1,%1,%1,%1,%1,%1,%1,%1,%1,"
        "%1,%1,%1,%1,%1,%1,%1,%1,%1,%1,%1,%1,%1,%1,%1,%1};" ::"r"(addr), "r"(0u)
        : "memory");
    asm volatile("tcgen05.wait::st.sync.aligned;" ::: "memory");
}

// four consecutive K values (k4 .. k4+3) of one operand row, split hi / lo
__device__ __forceinline__ void c64_put4(unsigned char *base, int row, int k4, float a, float b, float c, float d)
{
    const uint32_t h0 = to_tf32(a), h1 = to_tf32(b), h2 = to_tf32(c), h3 = to_tf32(d);
    const uint32_t l0 = to_tf32(a - __uint_as_float(h0)), l1 = to_tf32(b - __uint_as_float(h1));
    const uint32_t l2 = to_tf32(c - __uint_as_float(h2)), l3 = to_tf32(d - __uint_as_float(h3));
    *reinterpret_cast<uint4 *>(base + c64_off(row, k4, 0)) = make_uint4(h0, h1, h2, h3);
    *reinterpret_cast<uint4 *>(base + c64_off(row, k4, 1)) = make_uint4(l0, l1, l2, l3);
}

// 32 consecutive accumulator columns of this thread's TMEM lane
__device__ __forceinline__ void c64_ld32(uint32_t addr, float (&v)[32])
{
    uint32_t r[32];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,"
        "%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
          "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]),
          "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]),
          "=r"(r[23]), "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]),
          "=r"(r[30]), "=r"(r[31])
        : "r"(addr));
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
    for (int q = 0; q < 32; ++q) v[q] = __uint_as_float(r[q]);
}

// warps 1-7 (the converters) meet here; warp 0 never takes part
__device__ __forceinline__ void c64_workers_sync() { asm volatile("bar.sync 2, 224;" ::: "memory"); }

constexpr int C64_AREG = (64 * 64 + 223) / 224;  // A_i elements per converter thread: 19
constexpr int C64_BREG = (16 * 64 + 223) / 224;  // B_i 4-element groups per converter thread: 5

template <class Tin>
__global__ void __launch_bounds__(C64_THREADS, 2) chain64_tc_kernel(ChainFactorArgs<Tin, float> g)
{
    constexpr int LD = Geo<float, 64>::LD;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    unsigned char *R = smem_raw;
    unsigned char *VR = smem_raw + C64_R_BYTES;
    float *sS = reinterpret_cast<float *>(VR);
    float *sV = sS + Geo<float, 64>::SLOT;
    float *dinv = reinterpret_cast<float *>(VR + C64_VR_BYTES);
    float *prow = dinv + 64;  // 64 floats: the Cholesky's pivot-row buffer
    unsigned char *tail = VR + C64_VR_BYTES + 512;
    int *sflag = reinterpret_cast<int *>(tail);
    uint32_t *tslot = reinterpret_cast<uint32_t *>(tail + 4);
    int *abort = reinterpret_cast<int *>(tail + 8);
    uint64_t *mbars = reinterpret_cast<uint64_t *>(tail + 16);  // MMA, A copy, B copy
    const Tin *rawA = reinterpret_cast<const Tin *>(VR);
    const Tin *rawB = reinterpret_cast<const Tin *>(R + C64_UPPER);

    const int tid = threadIdx.x, w = tid >> 5, lane = tid & 31;
    const int L = 32 * (w & 3) + lane;  // this thread's TMEM lane (accumulator row)
    const int c0 = 32 * (w >> 2);       // its first accumulator column
    const uint32_t lane_base = (uint32_t)(32 * (w & 3)) << 16;
    const int n = g.n;
    const long long nn = (long long)n * n;
    const long long p = blockIdx.x;
    const long long sL = (p * (g.N - 1)) / g.Q;
    const long long sR = ((p + 1) * (g.N - 1)) / g.Q;
    const long long first = sL + 1, last = sR - 1;
    const uint32_t blk_bytes = (uint32_t)(nn * (long long)sizeof(Tin));
    const bool bulk = (blk_bytes % 16u) == 0 && ((uintptr_t)g.A_in % 16u) == 0 && ((uintptr_t)g.B_in % 16u) == 0;

    if (w == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(tslot)),
                     "r"(128u)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    if (tid == 0) {
        for (int q = 0; q < 3; ++q)
            asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(&mbars[q])) : "memory");
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        *abort = 0;
    }
    fence_async_smem();
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tm = *tslot;
    const uint32_t sRa = smem_u32(R), sVa = smem_u32(VR);
    C64Bar bM{smem_u32(&mbars[0]), 0u, false}, bA{smem_u32(&mbars[1]), 0u, false}, bB{smem_u32(&mbars[2]), 0u, false};

    if (first <= last && bulk && tid == 32) {
        mbar_expect_tx(bA.addr, blk_bytes);
        bulk_g2s(sVa, g.A_in + first * nn, blk_bytes, bA.addr);
        bA.pending = true;
        bulk_prefetch_l2(g.B_in + first * nn, blk_bytes);
    }
    bool sll_started = false;
    for (long long i = first; i <= last; ++i) {
        const long long t = i - first;
        if (tid == 0) {
            // ---- P1 on [W_{i-1} | Y_{i-1}] (written and fenced by the previous step)
            if (t > 0) {
                tc_fence_after();
                c64_mma_rr(tm, sRa, sll_started);
                tc_commit(bM.addr);
                bM.pending = true;
                sll_started = true;
            }
            c64_wait1(bM, abort);
        } else if (w > 0) {
            // ---- meanwhile warps 1-7: A_i (identity outside n x n) to FP32 in sS, in place
            if (tid == 32) {
                c64_wait1(bA, abort);
                if (bulk && i < last) {  // the next step's blocks into L2
                    bulk_prefetch_l2(g.A_in + (i + 1) * nn, blk_bytes);
                    bulk_prefetch_l2(g.B_in + (i + 1) * nn, blk_bytes);
                }
            }
            c64_workers_sync();
            const Tin *Ag = bulk ? rawA : g.A_in + i * nn;
            float av[C64_AREG];
#pragma unroll
            for (int u = 0; u < C64_AREG; ++u) {
                const int e = (tid - 32) + 224 * u, r = e & 63, c = e >> 6;
                av[u] = (e < 4096 && r < n && c < n) ? (float)Ag[r + c * n] : (r == c ? 1.f : 0.f);
            }
            c64_workers_sync();  // every raw A_i value is read before sS (same bytes) is written
#pragma unroll
            for (int u = 0; u < C64_AREG; ++u) {
                const int e = (tid - 32) + 224 * u;
                if (e < 4096) sS[(e & 63) + (e >> 6) * LD] = av[u];
            }
        }
        __syncthreads();
        if (*abort) break;
        // R has been read by P1: B_i raw into its upper half (it lands during the Cholesky)
        if (tid == 32 && bulk) {
            fence_async_smem();
            mbar_expect_tx(bB.addr, blk_bytes);
            bulk_g2s(sRa + (uint32_t)C64_UPPER, g.B_in + i * nn, blk_bytes, bB.addr);
            bB.pending = true;
        }
        tc_fence_after();
        // ---- Ahat_i = A_i - W^T W (rows L < 64) and Z_i (rows L >= 64) from the P1 accumulator
        if (t > 0) {
            float dv[32];
            c64_ld32(tm + lane_base + (uint32_t)c0, dv);
            if (L < 64) {
                if (L < n) {
#pragma unroll
                    for (int q = 0; q < 32; ++q)
                        if (c0 + q < n) sS[L + (c0 + q) * LD] -= dv[q];
                }
            } else {
                const int cz = L - 64;  // column cz of Z = row cz of the P2 operand
#pragma unroll
                for (int q = 0; q < 32; q += 4) {
                    float z[4];
#pragma unroll
                    for (int u = 0; u < 4; ++u) z[u] = (cz < n && c0 + q + u < n) ? -dv[q + u] : 0.f;
                    c64_put4(R, cz, c0 + q, z[0], z[1], z[2], z[3]);
                }
            }
        } else {
            // Z_first = B_sL^T: row r of the operand (column r of Z) is row r of B_sL
            const int row = tid >> 2, k0 = (tid & 3) * 16;
            const Tin *Bs = g.B_in + sL * nn;
#pragma unroll
            for (int q = 0; q < 16; q += 4) {
                float z[4];
#pragma unroll
                for (int u = 0; u < 4; ++u) {
                    const int k = k0 + q + u;
                    z[u] = (row < n && k < n) ? (float)Bs[row + (long long)k * n] : 0.f;
                }
                c64_put4(R, row, k0 + q, z[0], z[1], z[2], z[3]);
            }
        }
        tc_fence_before();
        __syncthreads();
        // ---- U^T U = Ahat, V = U^-1 (CUDA cores; ends with a CTA barrier).  While
        // warp 0 factors the first diagonal tile, warps 1-7 turn the raw B_i in R's
        // upper half into its operand rows 64-127 (row 64 + j = column j of B_i),
        // in place: all raw values are read into registers first
        auto convert_b = [&](int K) {
            if (K != 0 || !bulk) return;
            if (tid == 32) c64_wait1(bB, abort);
            c64_workers_sync();
            if (*abort) return;
            float bv[C64_BREG][4];
#pragma unroll
            for (int u = 0; u < C64_BREG; ++u) {
                const int gi = (tid - 32) + 224 * u, j = gi >> 4, k4 = (gi & 15) * 4;
                if (gi < 1024 && n == 64) {
                    if constexpr (sizeof(Tin) == 8) {
                        const double2 b0 = *reinterpret_cast<const double2 *>(rawB + k4 + j * 64);
                        const double2 b1 = *reinterpret_cast<const double2 *>(rawB + k4 + 2 + j * 64);
                        bv[u][0] = (float)b0.x;
                        bv[u][1] = (float)b0.y;
                        bv[u][2] = (float)b1.x;
                        bv[u][3] = (float)b1.y;
                    } else {
                        const float4 b4 = *reinterpret_cast<const float4 *>(rawB + k4 + j * 64);
                        bv[u][0] = b4.x;
                        bv[u][1] = b4.y;
                        bv[u][2] = b4.z;
                        bv[u][3] = b4.w;
                    }
                } else {
#pragma unroll
                    for (int q = 0; q < 4; ++q) {
                        const int k = k4 + q;
                        bv[u][q] = (gi < 1024 && j < n && k < n) ? (float)rawB[k + j * n] : 0.f;
                    }
                }
            }
            c64_workers_sync();  // every raw B_i value is read before its bytes become operand rows
#pragma unroll
            for (int u = 0; u < C64_BREG; ++u) {
                const int gi = (tid - 32) + 224 * u;
                if (gi < 1024) c64_put4(R, 64 + (gi >> 4), (gi & 15) * 4, bv[u][0], bv[u][1], bv[u][2], bv[u][3]);
            }
        };
        const int bad =
            chol_inv_blocked<float, 64, C64_THREADS, true, true>(sS, sV, dinv, sflag, tid, prow, convert_b);
        if (bad && tid == 0) record_bad_pivot(g.st, g.level, i);
        if (*abort) break;
        // ---- V_i to HBM and the V_i operand (and, read with plain loads when the
        // blocks are not bulk-copied, the B_i operand).  Thread (jr + 16 m, k4):
        // 16 threads walk one column's 64 rows in float4 steps (conflict-free
        // reads of the padded sV, coalesced V stores), and their operand writes
        // land in distinct bank groups (leading byte offset 144)
        {
            const int jr = tid >> 4, k4 = (tid & 15) * 4;
            float vv[4][4];
#pragma unroll
            for (int m = 0; m < 4; ++m) {
                const int j = jr + 16 * m;
                const float4 v4 = *reinterpret_cast<const float4 *>(sV + k4 + j * LD);
                const bool lower = (k4 >> 4) > (j >> 4);  // V's lower tiles are zero
                vv[m][0] = lower ? 0.f : v4.x;
                vv[m][1] = lower ? 0.f : v4.y;
                vv[m][2] = lower ? 0.f : v4.z;
                vv[m][3] = lower ? 0.f : v4.w;
            }
            float *Vg = g.A_f + i * nn;
#pragma unroll
            for (int m = 0; m < 4; ++m) {
                const int j = jr + 16 * m;
                if (n == 64) {
                    *reinterpret_cast<float4 *>(Vg + j * 64 + k4) = make_float4(vv[m][0], vv[m][1], vv[m][2], vv[m][3]);
                } else if (j < n) {
#pragma unroll
                    for (int u = 0; u < 4; ++u)
                        if (k4 + u < n) Vg[(long long)j * n + k4 + u] = vv[m][u];
                }
            }
            __syncthreads();  // sV is read: its bytes become the V operand
#pragma unroll
            for (int m = 0; m < 4; ++m) {
                const int j = jr + 16 * m;
                c64_put4(VR, j, k4, vv[m][0], vv[m][1], vv[m][2], vv[m][3]);
                if (!bulk) {
                    const Tin *Bg = g.B_in + i * nn;
                    float b[4];
#pragma unroll
                    for (int u = 0; u < 4; ++u) {
                        const int k = k4 + u;
                        b[u] = (j < n && k < n) ? (float)Bg[k + (long long)j * n] : 0.f;
                    }
                    c64_put4(R, 64 + j, k4, b[0], b[1], b[2], b[3]);
                }
            }
        }
        fence_async_smem();
        __syncthreads();
        // ---- P2 = [Z_i | B_i]^T V_i
        if (tid == 0) {
            tc_fence_after();
            c64_mma(tm, sRa, sVa, false);
            tc_commit(bM.addr);
            bM.pending = true;
            c64_wait1(bM, abort);
        }
        __syncthreads();
        if (*abort) break;
        if (tid == 32 && bulk && i < last) {  // P2 has read V: the next A block into VR
            fence_async_smem();
            mbar_expect_tx(bA.addr, blk_bytes);
            bulk_g2s(sVa, g.A_in + (i + 1) * nn, blk_bytes, bA.addr);
            bA.pending = true;
        }
        tc_fence_after();
        // ---- Y_i (rows L < 64) and W_i (rows L >= 64): to HBM and into R as [W_i | Y_i]
        float dv[32];
        c64_ld32(tm + lane_base + (uint32_t)c0, dv);
        c64_zero32(tm + lane_base + (uint32_t)c0);  // the next P1 accumulates onto these columns
        {
            const bool isY = L < 64;
            const int col = isY ? L : L - 64;
            float *dst = (isY ? g.Y : g.B_f) + i * nn;
            if (n == 64) {
#pragma unroll
                for (int q = 0; q < 32; q += 4)
                    *reinterpret_cast<float4 *>(dst + col * 64 + c0 + q) = make_float4(dv[q], dv[q + 1], dv[q + 2], dv[q + 3]);
            } else if (col < n) {
#pragma unroll
                for (int q = 0; q < 32; ++q)
                    if (c0 + q < n) dst[(long long)col * n + c0 + q] = dv[q];
            }
            const int row = isY ? 64 + col : col;
#pragma unroll
            for (int q = 0; q < 32; q += 4) c64_put4(R, row, c0 + q, dv[q], dv[q + 1], dv[q + 2], dv[q + 3]);
        }
        fence_async_smem();
        tc_fence_before();
        __syncthreads();
    }

    // ---- chain end: S_RR = W^T W, S_LR = Y^T W and the last S_LL term (P1)
    if (!*abort && first <= last) {
        if (tid == 0) {
            tc_fence_after();
            c64_mma_rr(tm, sRa, sll_started);
            tc_commit(bM.addr);
            bM.pending = true;
            c64_wait1(bM, abort);
        }
        __syncthreads();
        tc_fence_after();
        float dv[32];
        float *Cp = g.C + p * 3 * nn;
        c64_ld32(tm + lane_base + (uint32_t)c0, dv);
        {
            const int r = L < 64 ? L : L - 64;
            float *dst = Cp + (L < 64 ? nn : 2 * nn);  // S_RR rows, S_LR rows
            if (r < n) {
#pragma unroll
                for (int q = 0; q < 32; ++q)
                    if (c0 + q < n) dst[r + (long long)(c0 + q) * n] = dv[q];
            }
        }
        c64_ld32(tm + lane_base + 64u + (uint32_t)c0, dv);
        if (L >= 64 && L - 64 < n) {
            const int r = L - 64;
#pragma unroll
            for (int q = 0; q < 32; ++q)
                if (c0 + q < n) Cp[r + (long long)(c0 + q) * n] = dv[q];
        }
    }
    __syncthreads();
    if (*abort) {
        // a wait gave up: wait (bounded) for this CTA's MMAs (thread 0) and
        // copies (thread 32) still in flight before its shared memory and
        // TMEM are released
        int ignored = 0;
        if (tid == 0) {
            c64_wait1(bM, &ignored);
            if (g.st) atomicExch(&g.st->tc_timeout, 1);
        } else if (tid == 32) {
            c64_wait1(bA, &ignored);
            c64_wait1(bB, &ignored);
        }
    }
    tc_fence_before();
    __syncthreads();
    if (w == 0) {
        tc_fence_after();
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tm), "r"(128u) : "memory");
    }
}

}  // namespace bss
