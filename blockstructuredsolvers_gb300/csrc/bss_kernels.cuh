// Device kernels of the GB300 batched block-tridiagonal SPD solver.
//
// Algorithm (one recursion level; reference src/gpu_batched.jl:184-258 and
// src/backbone_cuda.jl:70-184 compute the same separator system with batched
// cuBLAS/cuSOLVER calls):
//
//   A level has N blocks.  Separators sit at s_p = floor(p*(N-1)/Q),
//   p = 0..Q; partition p owns the interior chain s_p+1 .. s_{p+1}-1.
//   One CTA walks one partition's chain ("chain kernel").  For interior
//   block i (t-th of the chain) it keeps W_{i-1} and Y_{i-1} in shared memory
//   and computes
//       Ahat  = A_i - W_{i-1}^T W_{i-1}                 (t > 0)
//       U^T U = Ahat,  V = U^{-1}                        (register Cholesky + inverse)
//       Z     = B_{s_p}^T (t = 0)  or  -W_{i-1}^T Y_{i-1}
//       Y_i   = V^T Z          left-separator fill  (R^{-T} G_left)
//       W_i   = V^T B_i        block-bidiagonal factor (U^{-T} B)
//       S_LL += Y_i^T Y_i
//   and at the chain end S_RR = W_last^T W_last, S_LR = Y_last^T W_last.
//   The reference's F = T^{-1} G (n x 2n per block) and M_2n = sum G^T F
//   (m gemms, mostly on zero blocks) are replaced by the left fill Y
//   (n x n per block) and three symmetric products: the separator system is
//       A'_p = A_{s_p} - S_LL(p) - S_RR(p-1),     B'_p = -S_LR(p).
//   The coarsest level runs the same kernel with no separators (sequential
//   block Cholesky, reference src/backbone_cuda.jl:14-37 / backbone_cpu.jl:5-15).
//
//   After factorization the A slot of interior block i holds V_i = U_i^{-1}
//   (upper triangular), the B slot holds W_i, and Y_i lives in workspace.
//   Solve (reference solve!, gpu_batched.jl:229-258):
//       forward   y_i = V_i^T (d_i - W_{i-1}^T y_{i-1});  bL = sum Y_i^T y_i;
//                 bR = W_last^T y_last;  d'_p = d_{s_p} - bL(p) - bR(p-1)
//       recurse on the separator system -> x_sep
//       backward  x_i = V_i (y_i - Y_i x_L - W_i x_{i+1})   (x_{last+1} = x_R)
//
// Shared-memory matrix tiles are column-major NB x NB with leading dimension
// LD = NB + 16/sizeof(T) (16 B pad: conflict-free 128-bit column reads).
// Each thread owns the RA x RB elements (ti + TI*a, tj + TJ*b) of a tile.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

namespace bss {

// ---------------------------------------------------------------------------
// status shared by all kernels of a handle
// ---------------------------------------------------------------------------
struct DevStatus {
    unsigned long long bad_key;  // min over ((level << 40) | block) of failed pivots
    unsigned long long rnorm;    // FP64 bits of max |r| (non-negative doubles order as ints)
    unsigned long long xnorm;    // FP64 bits of max |x|
    unsigned long long dnorm;    // FP64 bits of max |d|
    unsigned long long anorm;    // FP64 bits of ||T||_inf
    double relres;
    int done;
    int pad;
};

__device__ __forceinline__ void record_bad_pivot(DevStatus *st, int level, long long block)
{
    if (st) {
        unsigned long long key = ((unsigned long long)level << 40) | (unsigned long long)block;
        atomicMin(&st->bad_key, key);
    }
}

__device__ __forceinline__ void atomic_max_nonneg(unsigned long long *addr, double v)
{
    atomicMax(addr, (unsigned long long)__double_as_longlong(v));
}

// ---------------------------------------------------------------------------
// tile configuration per block size NB
// ---------------------------------------------------------------------------
template <int NB>
struct Tile;
template <>
struct Tile<64> {
    static constexpr int TI = 16, TJ = 16, RA = 4, RB = 4, THREADS = 256;
};
template <>
struct Tile<32> {
    static constexpr int TI = 16, TJ = 8, RA = 2, RB = 4, THREADS = 128;
};
template <>
struct Tile<16> {
    static constexpr int TI = 16, TJ = 4, RA = 1, RB = 4, THREADS = 64;
};

template <class T>
struct Vec;
template <>
struct Vec<float> {
    using type = float4;
    static constexpr int W = 4;
};
template <>
struct Vec<double> {
    using type = double2;
    static constexpr int W = 2;
};

template <class T, int NB>
struct Geo {
    static constexpr int LD = NB + 16 / (int)sizeof(T);
    static constexpr int SLOT = NB * LD;  // elements per smem matrix slot
};

__device__ __forceinline__ void fma_vec(float &acc, const float4 &x, const float4 &y)
{
    acc = fmaf(x.x, y.x, acc);
    acc = fmaf(x.y, y.y, acc);
    acc = fmaf(x.z, y.z, acc);
    acc = fmaf(x.w, y.w, acc);
}
__device__ __forceinline__ void fma_vec(double &acc, const double2 &x, const double2 &y)
{
    acc = fma(x.x, y.x, acc);
    acc = fma(x.y, y.y, acc);
}

// acc[a][b] += sum_k X(k, ti+TI*a) * Y(k, tj+TJ*b)     (C += X^T Y)
template <class T, int NB>
__device__ __forceinline__ void tn_acc(T (&acc)[Tile<NB>::RA][Tile<NB>::RB], const T *X, const T *Y,
                                       int ti, int tj)
{
    using TL = Tile<NB>;
    using V = typename Vec<T>::type;
    constexpr int LD = Geo<T, NB>::LD;
    constexpr int W = Vec<T>::W;
#pragma unroll 4
    for (int k = 0; k < NB; k += W) {
        V xa[TL::RA], yb[TL::RB];
#pragma unroll
        for (int a = 0; a < TL::RA; ++a) xa[a] = *reinterpret_cast<const V *>(X + k + (ti + TL::TI * a) * LD);
#pragma unroll
        for (int b = 0; b < TL::RB; ++b) yb[b] = *reinterpret_cast<const V *>(Y + k + (tj + TL::TJ * b) * LD);
#pragma unroll
        for (int a = 0; a < TL::RA; ++a)
#pragma unroll
            for (int b = 0; b < TL::RB; ++b) fma_vec(acc[a][b], xa[a], yb[b]);
    }
}

// acc1 += X^T Y1, acc2 += X^T Y2 (shared X reads)
template <class T, int NB>
__device__ __forceinline__ void tn_acc2(T (&acc1)[Tile<NB>::RA][Tile<NB>::RB],
                                        T (&acc2)[Tile<NB>::RA][Tile<NB>::RB], const T *X, const T *Y1,
                                        const T *Y2, int ti, int tj)
{
    using TL = Tile<NB>;
    using V = typename Vec<T>::type;
    constexpr int LD = Geo<T, NB>::LD;
    constexpr int W = Vec<T>::W;
#pragma unroll 2
    for (int k = 0; k < NB; k += W) {
        V xa[TL::RA], yb[TL::RB], zb[TL::RB];
#pragma unroll
        for (int a = 0; a < TL::RA; ++a) xa[a] = *reinterpret_cast<const V *>(X + k + (ti + TL::TI * a) * LD);
#pragma unroll
        for (int b = 0; b < TL::RB; ++b) {
            yb[b] = *reinterpret_cast<const V *>(Y1 + k + (tj + TL::TJ * b) * LD);
            zb[b] = *reinterpret_cast<const V *>(Y2 + k + (tj + TL::TJ * b) * LD);
        }
#pragma unroll
        for (int a = 0; a < TL::RA; ++a)
#pragma unroll
            for (int b = 0; b < TL::RB; ++b) {
                fma_vec(acc1[a][b], xa[a], yb[b]);
                fma_vec(acc2[a][b], xa[a], zb[b]);
            }
    }
}

template <class T, int NB>
__device__ __forceinline__ void zero_tile(T (&acc)[Tile<NB>::RA][Tile<NB>::RB])
{
#pragma unroll
    for (int a = 0; a < Tile<NB>::RA; ++a)
#pragma unroll
        for (int b = 0; b < Tile<NB>::RB; ++b) acc[a][b] = T(0);
}

// load block (column-major n x n, leading dim n) into the thread's tile;
// outside n x n: identity (diag_pad) or zero.  transpose: tile(r,c) = G(c,r).
template <class Tin, class T, int NB>
__device__ __forceinline__ void load_tile(T (&dst)[Tile<NB>::RA][Tile<NB>::RB], const Tin *__restrict__ g,
                                          int n, int ti, int tj, bool diag_pad, bool transpose)
{
    using TL = Tile<NB>;
#pragma unroll
    for (int a = 0; a < TL::RA; ++a)
#pragma unroll
        for (int b = 0; b < TL::RB; ++b) {
            const int r = ti + TL::TI * a, c = tj + TL::TJ * b;
            T v;
            if (r < n && c < n)
                v = (T)(transpose ? g[c + (size_t)r * n] : g[r + (size_t)c * n]);
            else
                v = (diag_pad && r == c) ? T(1) : T(0);
            dst[a][b] = v;
        }
}

template <class T, int NB>
__device__ __forceinline__ void store_tile_global(T *__restrict__ g, const T (&src)[Tile<NB>::RA][Tile<NB>::RB],
                                                  int n, int ti, int tj, T scale)
{
    using TL = Tile<NB>;
#pragma unroll
    for (int a = 0; a < TL::RA; ++a)
#pragma unroll
        for (int b = 0; b < TL::RB; ++b) {
            const int r = ti + TL::TI * a, c = tj + TL::TJ * b;
            if (r < n && c < n) g[r + (size_t)c * n] = scale * src[a][b];
        }
}

template <class T, int NB>
__device__ __forceinline__ void store_tile_smem(T *s, const T (&src)[Tile<NB>::RA][Tile<NB>::RB], int ti,
                                                int tj, T scale)
{
    using TL = Tile<NB>;
    constexpr int LD = Geo<T, NB>::LD;
#pragma unroll
    for (int a = 0; a < TL::RA; ++a)
#pragma unroll
        for (int b = 0; b < TL::RB; ++b) s[(ti + TL::TI * a) + (tj + TL::TJ * b) * LD] = scale * src[a][b];
}

template <class T>
__device__ __forceinline__ T safe_pivot(T p)
{
    return (p > T(0) && p < T(INFINITY)) ? p : T(1);
}

// ---------------------------------------------------------------------------
// Blocked upper Cholesky + inverse of an NB x NB SPD tile in shared memory.
// On entry sS holds S; only its upper triangle is read (as LAPACK potrf 'U'
// in the reference's backbone_cpu.jl:7,13 / cusolverDnXpotrf(Batched) 'U').
// On exit sS's upper triangle holds U (U^T U = S), its lower triangle is
// scratch, and sV holds V = U^{-1} (upper, zeros below the diagonal -- the
// caller zeroes sV's strictly lower 16x16 tiles once).
// Panels are PB = 16 wide: one warp factors each 16x16 diagonal tile with
// shuffles (lane r owns column r), another warp inverts it by per-lane back
// substitution while the rest of the CTA solves the row panel; the trailing
// matrix update and the NB/16-1 block stages of V are spread over the CTA.
// ---------------------------------------------------------------------------
constexpr int PB = 16;

template <class T, int LD>
__device__ __forceinline__ int warp_chol16(T *sS, T *dinv, int o, int lane)
{
    const int r = lane & (PB - 1);
    T u[PB];
#pragma unroll
    for (int c = 0; c < PB; ++c) u[c] = sS[(o + c) + (o + r) * LD];  // S(o+c, o+r), valid for c <= r
    int bad = 0;
    T udiag = T(1);
#pragma unroll
    for (int j = 0; j < PB; ++j) {
        T piv = __shfl_sync(0xffffffffu, u[j], j);
        if (!(piv > T(0) && piv < T(INFINITY))) {
            bad = 1;
            piv = T(1);
        }
        const T ujr = u[j] * (T(1) / sqrt(piv));  // U(j, r), r >= j
        u[j] = ujr;
        if (j == r) udiag = ujr;
#pragma unroll
        for (int c = j + 1; c < PB; ++c) {
            const T ujc = __shfl_sync(0xffffffffu, ujr, c);  // U(j, c) from lane c
            u[c] = fma(-ujc, ujr, u[c]);                      // S(c, r) -= U(j,c) U(j,r)
        }
    }
    if (lane < PB) {
#pragma unroll
        for (int c = 0; c < PB; ++c)
            if (c <= r) sS[(o + c) + (o + r) * LD] = u[c];
        dinv[o + r] = T(1) / udiag;
    }
    return bad;
}

// V_KK = U_KK^{-1}: lane r computes column r by back substitution.
template <class T, int LD>
__device__ __forceinline__ void warp_inv16(const T *sS, const T *dinv, T *sV, int o, int lane)
{
    const int r = lane & (PB - 1);
    T v[PB];
#pragma unroll
    for (int q = PB - 1; q >= 0; --q) {
        T s0 = (q == r) ? T(1) : T(0), s1 = T(0);
#pragma unroll
        for (int t = q + 1; t < PB; ++t) {
            if ((t & 1) == 0)
                s0 = fma(-sS[(o + q) + (o + t) * LD], v[t], s0);
            else
                s1 = fma(-sS[(o + q) + (o + t) * LD], v[t], s1);
        }
        v[q] = (s0 + s1) * dinv[o + q];
    }
    if (lane < PB) {
#pragma unroll
        for (int c = 0; c < PB; ++c) sV[(o + c) + (o + r) * LD] = v[c];
    }
}

// row panel right of diagonal tile o: U(o:o+16, c) = U_KK^{-T} S(o:o+16, c)
template <class T, int LD, int NB>
__device__ __forceinline__ void panel_trsm(T *sS, const T *dinv, int o, int t0, int nthr)
{
    for (int c = o + PB + t0; c < NB; c += nthr) {
        T x[PB];
#pragma unroll
        for (int p = 0; p < PB; ++p) x[p] = sS[(o + p) + c * LD];
#pragma unroll
        for (int p = 0; p < PB; ++p) {
            x[p] *= dinv[o + p];
#pragma unroll
            for (int q = p + 1; q < PB; ++q) x[q] = fma(-sS[(o + p) + (o + q) * LD], x[p], x[q]);
        }
#pragma unroll
        for (int p = 0; p < PB; ++p) sS[(o + p) + c * LD] = x[p];
    }
}

// S(a, b) -= sum_p U(o+p, a) U(o+p, b)   for o+16 <= a <= b < NB
template <class T, int LD, int NB>
__device__ __forceinline__ void trailing_update(T *sS, int o, int tid, int nthr)
{
    using V = typename Vec<T>::type;
    constexpr int W = Vec<T>::W;
    const int m = NB - o - PB;
    for (int e = tid; e < m * m; e += nthr) {
        const int b = e / m;
        const int a = e - b * m;
        if (a > b) continue;
        const int ca = o + PB + a, cb = o + PB + b;
        T acc = T(0);
#pragma unroll
        for (int p = 0; p < PB; p += W) {
            const V x = *reinterpret_cast<const V *>(sS + (o + p) + ca * LD);
            const V y = *reinterpret_cast<const V *>(sS + (o + p) + cb * LD);
            fma_vec(acc, x, y);
        }
        sS[ca + cb * LD] -= acc;
    }
}

// off-diagonal tiles of V = U^{-1}:  V_IJ = -V_II sum_{P=I+1..J} U_IP V_PJ,
// one super-diagonal stage at a time (s = J - I).  T_IJ is kept in the
// (scratch) lower tile (J, I) of sS.
template <class T, int LD, int NB>
__device__ __forceinline__ void inverse_stages(T *sS, T *sV, int tid, int nthr)
{
    constexpr int KP = NB / PB;
#pragma unroll 1
    for (int s = 1; s < KP; ++s) {
        const int ntile = KP - s;
        for (int e = tid; e < ntile * PB * PB; e += nthr) {
            const int tile = e / (PB * PB), w = e - tile * PB * PB;
            const int a = w % PB, b = w / PB;
            const int I = tile, J = tile + s;
            T acc = T(0);
            for (int P = I + 1; P <= J; ++P)
#pragma unroll
                for (int q = 0; q < PB; ++q)
                    acc = fma(sS[(PB * I + a) + (PB * P + q) * LD], sV[(PB * P + q) + (PB * J + b) * LD], acc);
            sS[(PB * J + a) + (PB * I + b) * LD] = acc;
        }
        __syncthreads();
        for (int e = tid; e < ntile * PB * PB; e += nthr) {
            const int tile = e / (PB * PB), w = e - tile * PB * PB;
            const int a = w % PB, b = w / PB;
            const int I = tile, J = tile + s;
            T acc = T(0);
#pragma unroll
            for (int c = 0; c < PB; ++c)
                if (c >= a) acc = fma(sV[(PB * I + a) + (PB * I + c) * LD], sS[(PB * J + c) + (PB * I + b) * LD], acc);
            sV[(PB * I + a) + (PB * J + b) * LD] = -acc;
        }
        __syncthreads();
    }
}

// Factor the tile in sS into sV = U^{-1}.  Returns nonzero (in every thread)
// if a pivot failed.  Ends with a __syncthreads.
template <class T, int NB, int THREADS>
__device__ __forceinline__ int chol_inv_blocked(T *sS, T *sV, T *dinv, int *sflag, int tid)
{
    constexpr int LD = Geo<T, NB>::LD;
    constexpr int KP = NB / PB;
    const int warp = tid >> 5, lane = tid & 31;
    if (tid == 0) *sflag = 0;
#pragma unroll 1
    for (int K = 0; K < KP; ++K) {
        const int o = PB * K;
        if (warp == 0) {
            const int bad = warp_chol16<T, LD>(sS, dinv, o, lane);
            if (bad && lane == 0) *sflag = 1;
        }
        __syncthreads();
        if (warp == (THREADS > 32 ? 1 : 0)) warp_inv16<T, LD>(sS, dinv, sV, o, lane);
        if (K + 1 < KP) {
            if (THREADS > 32) {
                const int t0 = warp == 0 ? lane : tid - 32;
                if (warp != 1) panel_trsm<T, LD, NB>(sS, dinv, o, t0, THREADS - 32);
            } else {
                panel_trsm<T, LD, NB>(sS, dinv, o, tid, THREADS);
            }
            __syncthreads();
            trailing_update<T, LD, NB>(sS, o, tid, THREADS);
        }
        __syncthreads();
    }
    inverse_stages<T, LD, NB>(sS, sV, tid, THREADS);
    return *sflag;
}

// ---------------------------------------------------------------------------
// chain factor kernel
// ---------------------------------------------------------------------------
template <class Tin, class T>
struct ChainFactorArgs {
    const Tin *A_in;  // level A (N blocks)
    const Tin *B_in;  // level B (N-1 blocks)
    T *A_f;           // factor V_i per block (may alias A_in when Tin == T)
    T *B_f;           // factor W_i per block (may alias B_in)
    T *Y;             // left fill per block (N blocks, interior used); null when seq
    T *C;             // Q x [S_LL | S_RR | S_LR] (n x n each); null when seq
    long long N;
    long long Q;      // partitions (ignored when seq)
    int n;
    int seq;          // 1: one chain over all blocks, no separators
    int level;
    DevStatus *st;
};

template <class T, int NB>
constexpr size_t chain_factor_smem()
{
    return (size_t)(6 * Geo<T, NB>::SLOT + NB) * sizeof(T) + 16;
}

template <class Tin, class T, int NB>
__global__ void __launch_bounds__(Tile<NB>::THREADS, sizeof(T) == 4 ? 2 : 1) chain_factor_kernel(ChainFactorArgs<Tin, T> g)
{
    using TL = Tile<NB>;
    constexpr int LD = Geo<T, NB>::LD;
    constexpr int SLOT = Geo<T, NB>::SLOT;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    T *sV = reinterpret_cast<T *>(smem_raw);
    T *sW = sV + SLOT;
    T *sY = sW + SLOT;
    T *sZ = sY + SLOT;
    T *sB = sZ + SLOT;
    T *sS = sB + SLOT;
    T *dinv = sS + SLOT;                              // NB
    int *sflag = reinterpret_cast<int *>(dinv + NB);

    const int tid = threadIdx.x;
    const int ti = tid % TL::TI, tj = tid / TL::TI;
    const int n = g.n;
    const long long nn = (long long)n * n;
    const bool seq = g.seq != 0;
    const long long p = blockIdx.x;

    long long first, last, sL = 0;
    if (seq) {
        first = 0;
        last = g.N - 1;
    } else {
        sL = (p * (g.N - 1)) / g.Q;
        const long long sR = ((p + 1) * (g.N - 1)) / g.Q;
        first = sL + 1;
        last = sR - 1;
    }

    T accLL[TL::RA][TL::RB];
    zero_tile<T, NB>(accLL);
    for (int e = tid; e < SLOT; e += TL::THREADS) sV[e] = T(0);  // V's strictly lower tiles stay zero
    __syncthreads();

    for (long long i = first; i <= last; ++i) {
        const long long t = i - first;
        const bool has_next = !seq || (i < g.N - 1);
        T S[TL::RA][TL::RB];
        load_tile<Tin, T, NB>(S, g.A_in + i * nn, n, ti, tj, true, false);
        if (t > 0) {
            T accS[TL::RA][TL::RB];
            zero_tile<T, NB>(accS);
            if (!seq) {
                T accZ[TL::RA][TL::RB];
                zero_tile<T, NB>(accZ);
                tn_acc2<T, NB>(accS, accZ, sW, sW, sY, ti, tj);
                store_tile_smem<T, NB>(sZ, accZ, ti, tj, T(-1));
            } else {
                tn_acc<T, NB>(accS, sW, sW, ti, tj);
            }
#pragma unroll
            for (int a = 0; a < TL::RA; ++a)
#pragma unroll
                for (int b = 0; b < TL::RB; ++b) S[a][b] -= accS[a][b];
        } else if (!seq) {
            T Zt[TL::RA][TL::RB];
            load_tile<Tin, T, NB>(Zt, g.B_in + sL * nn, n, ti, tj, false, true);  // Z = B_{sL}^T
            store_tile_smem<T, NB>(sZ, Zt, ti, tj, T(1));
        }
        T Bi[TL::RA][TL::RB];
        if (has_next) load_tile<Tin, T, NB>(Bi, g.B_in + i * nn, n, ti, tj, false, false);

        store_tile_smem<T, NB>(sS, S, ti, tj, T(1));
        if (has_next) store_tile_smem<T, NB>(sB, Bi, ti, tj, T(1));
        __syncthreads();
        const int bad = chol_inv_blocked<T, NB, TL::THREADS>(sS, sV, dinv, sflag, tid);
        if (bad && tid == 0) record_bad_pivot(g.st, g.level, i);

        T accY[TL::RA][TL::RB], accW[TL::RA][TL::RB];
        zero_tile<T, NB>(accY);
        zero_tile<T, NB>(accW);
        if (!seq)
            tn_acc2<T, NB>(accY, accW, sV, sZ, sB, ti, tj);
        else if (has_next)
            tn_acc<T, NB>(accW, sV, sB, ti, tj);

        // V -> global (coalesced copy from sV)
        {
            T *dst = g.A_f + i * nn;
            const int nn32 = n * n;
            for (int e = tid; e < nn32; e += TL::THREADS) {
                const int c = e / n, r = e - c * n;
                dst[e] = sV[r + c * LD];
            }
        }
        if (has_next) {
            store_tile_global<T, NB>(g.B_f + i * nn, accW, n, ti, tj, T(1));
            store_tile_smem<T, NB>(sW, accW, ti, tj, T(1));
        }
        if (!seq) {
            store_tile_global<T, NB>(g.Y + i * nn, accY, n, ti, tj, T(1));
            store_tile_smem<T, NB>(sY, accY, ti, tj, T(1));
        }
        __syncthreads();
        if (!seq) tn_acc<T, NB>(accLL, sY, sY, ti, tj);
    }

    if (!seq) {
        T accRR[TL::RA][TL::RB], accLR[TL::RA][TL::RB];
        zero_tile<T, NB>(accRR);
        zero_tile<T, NB>(accLR);
        tn_acc<T, NB>(accRR, sW, sW, ti, tj);
        tn_acc<T, NB>(accLR, sY, sW, ti, tj);
        T *Cp = g.C + p * 3 * nn;
        store_tile_global<T, NB>(Cp, accLL, n, ti, tj, T(1));
        store_tile_global<T, NB>(Cp + nn, accRR, n, ti, tj, T(1));
        store_tile_global<T, NB>(Cp + 2 * nn, accLR, n, ti, tj, T(1));
    }
}

// ---------------------------------------------------------------------------
// separator system assembly: A'_s = A_{sep s} - S_LL(s) - S_RR(s-1),
// B'_s = -S_LR(s)     (reference compute_schur_complement!, backbone_cuda.jl:143-157)
// ---------------------------------------------------------------------------
template <class Tsrc, class T, class Tdst>
__global__ void assemble_schur_kernel(const Tsrc *__restrict__ A_src, const T *__restrict__ C,
                                      Tdst *__restrict__ A_next, Tdst *__restrict__ B_next, long long N,
                                      long long Q, int n)
{
    const long long nn = (long long)n * n;
    const long long totalA = (Q + 1) * nn;
    const long long totalB = Q * nn;
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < totalA + totalB;
         e += (long long)gridDim.x * blockDim.x) {
        if (e < totalA) {
            const long long s = e / nn, w = e % nn;
            const long long blk = (s * (N - 1)) / Q;
            double v = (double)A_src[blk * nn + w];
            if (s < Q) v -= (double)C[s * 3 * nn + w];
            if (s > 0) v -= (double)C[(s - 1) * 3 * nn + nn + w];
            A_next[e] = (Tdst)v;
        } else {
            const long long f = e - totalA;
            const long long s = f / nn, w = f % nn;
            B_next[f] = (Tdst)(-C[s * 3 * nn + 2 * nn + w]);
        }
    }
}

// ---------------------------------------------------------------------------
// solve kernels.  Per chain step the three factor blocks (V_i, W, Y_i) are
// staged unpadded (leading dimension n) in shared memory with cp.async, the
// next step's blocks streaming into the other half of a double buffer while
// the current step computes.  Transpose products (M^T v) use one warp per
// output column with the lanes along the contraction (conflict-free,
// shuffle reduction); normal products (M v) use one thread per output row,
// the contraction split over thread groups and reduced through smem.
// ---------------------------------------------------------------------------
constexpr int SOLVE_THREADS = 256;

__device__ __forceinline__ void cp_async16(void *smem, const void *gmem)
{
    const unsigned s = (unsigned)__cvta_generic_to_shared(smem);
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(s), "l"(gmem));
}
__device__ __forceinline__ void cp_async8(void *smem, const void *gmem)
{
    const unsigned s = (unsigned)__cvta_generic_to_shared(smem);
    asm volatile("cp.async.ca.shared.global [%0], [%1], 8;\n" ::"r"(s), "l"(gmem));
}
__device__ __forceinline__ void cp_async4(void *smem, const void *gmem)
{
    const unsigned s = (unsigned)__cvta_generic_to_shared(smem);
    asm volatile("cp.async.ca.shared.global [%0], [%1], 4;\n" ::"r"(s), "l"(gmem));
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::); }
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_all;\n" ::: "memory"); }

// async copy of `count` contiguous elements (both ends aligned to 16 B when
// count*sizeof(T) is a multiple of 16, which the caller's layout guarantees)
template <class T>
__device__ __forceinline__ void async_copy(T *s, const T *__restrict__ g, int count)
{
    if (((count * (int)sizeof(T)) & 15) == 0) {
        const int chunks = count * (int)sizeof(T) / 16;
        for (int e = threadIdx.x; e < chunks; e += blockDim.x)
            cp_async16(reinterpret_cast<char *>(s) + 16 * e, reinterpret_cast<const char *>(g) + 16 * e);
    } else {
        for (int e = threadIdx.x; e < count; e += blockDim.x) {
            if (sizeof(T) == 8)
                cp_async8(s + e, g + e);
            else
                cp_async4(s + e, g + e);
        }
    }
}

// out(c, j) (+)= sign * sum_r M(r, c) v(r, j); M n x n (ld n), v/out n x kc (ld n)
template <class T>
__device__ __forceinline__ void cta_tmul(const T *sM, const T *v, T *out, int n, int kc, T sign, bool accumulate)
{
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
    for (int c = warp; c < n; c += nw) {
        for (int j = 0; j < kc; ++j) {
            T s = T(0);
            for (int r = lane; r < n; r += 32) s = fma(sM[r + c * n], v[r + j * n], s);
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
            if (lane == 0) out[c + j * n] = accumulate ? out[c + j * n] + sign * s : sign * s;
        }
    }
}

// out(r, j) = base(r, j) + sign * (sum_c M1(r,c) v1(c,j) [+ sum_c M2(r,c) v2(c,j)])
// (base may be null).  `red` holds max(blockDim, n*kc) elements.  Ends
// without a barrier; callers sync before reading `out`.
template <class T>
__device__ __forceinline__ void cta_nmul(const T *M1, const T *v1, const T *M2, const T *v2, const T *base, T *out,
                                         T sign, int n, int kc, T *red)
{
    const int no = n * kc;
    int parts = (int)blockDim.x / no;
    parts = parts < 1 ? 1 : (parts > 8 ? 8 : parts);
    for (int w = threadIdx.x; w < parts * no; w += blockDim.x) {
        const int part = w / no, o = w - part * no;
        const int j = o / n, r = o - j * n;
        const int c0 = (part * n) / parts, c1 = ((part + 1) * n) / parts;
        T s = T(0);
        for (int c = c0; c < c1; ++c) s = fma(M1[r + c * n], v1[c + j * n], s);
        if (M2)
            for (int c = c0; c < c1; ++c) s = fma(M2[r + c * n], v2[c + j * n], s);
        red[w] = s;
    }
    __syncthreads();
    for (int o = threadIdx.x; o < no; o += blockDim.x) {
        T s = T(0);
        for (int q = 0; q < parts; ++q) s += red[q * no + o];
        out[o] = (base ? base[o] : T(0)) + sign * s;
    }
}

template <class T>
struct SolveArgs {
    const T *Af;   // V per block
    const T *Bf;   // W per block
    const T *Y;    // left fill per block (null when seq)
    T *d;          // level RHS (N blocks, n*k elements per block); y / x in place
    T *bvec;       // Q x [bL | bR] (n x kc each, per column chunk)
    const void *xsep;  // next-level solution (Q+1 blocks, n x k each), type Tsep
    long long N;
    long long Q;
    int n;
    int k;         // columns per block in d / xsep
    int j0;        // first column of this pass
    int kc;        // columns in this pass
    int seq;
};

// shared memory: 2 buffers x 3 blocks + 5 vectors + reduction scratch
template <class T>
__host__ __device__ constexpr size_t solve_smem_bytes(int n, int kc)
{
    return (size_t)(6 * n * n + 5 * n * kc + (n * kc > SOLVE_THREADS ? n * kc : SOLVE_THREADS)) * sizeof(T);
}

// load n x kc columns j0.. of block blk of a (n x k per block) tensor
template <class Tg, class T>
__device__ __forceinline__ void load_rhs(T *s, const Tg *__restrict__ g, long long blk, int n, int k, int j0, int kc)
{
    const Tg *b = g + blk * (long long)n * k + (long long)j0 * n;
    for (int e = threadIdx.x; e < n * kc; e += blockDim.x) s[e] = (T)b[e];
}
template <class Tg, class T>
__device__ __forceinline__ void store_rhs(Tg *__restrict__ g, const T *s, long long blk, int n, int k, int j0, int kc)
{
    Tg *b = g + blk * (long long)n * k + (long long)j0 * n;
    for (int e = threadIdx.x; e < n * kc; e += blockDim.x) b[e] = (Tg)s[e];
}

// forward sweep of one partition; for the sequential (coarsest) level the
// whole chain followed by its backward sweep.
template <class T>
__global__ void __launch_bounds__(SOLVE_THREADS) chain_fwd_kernel(SolveArgs<T> g)
{
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int n = g.n, kc = g.kc;
    const int nn = n * n;
    T *buf = reinterpret_cast<T *>(smem_raw);  // [2][3][nn]: V, W, Y
    T *sr = buf + 6 * nn;
    T *sy = sr + n * kc;
    T *sbL = sy + n * kc;
    T *sbR = sbL + n * kc;
    T *sx = sbR + n * kc;
    T *red = sx + n * kc;
    const bool seq = g.seq != 0;
    const long long p = blockIdx.x;
    long long first, last;
    if (seq) {
        first = 0;
        last = g.N - 1;
    } else {
        const long long sL = (p * (g.N - 1)) / g.Q;
        const long long sR = ((p + 1) * (g.N - 1)) / g.Q;
        first = sL + 1;
        last = sR - 1;
    }
    for (int e = threadIdx.x; e < n * kc; e += blockDim.x) sbL[e] = T(0);
    // step i uses V_i (slot 0), W_{i-1} (slot 1), Y_i (slot 2) in buffer (i - first) & 1
    async_copy(buf, g.Af + first * (long long)nn, nn);
    if (!seq) async_copy(buf + 2 * nn, g.Y + first * (long long)nn, nn);
    cp_async_commit();
    for (long long i = first; i <= last; ++i) {
        T *cur = buf + ((i - first) & 1) * 3 * nn;
        T *nxt = buf + (((i - first) & 1) ^ 1) * 3 * nn;
        load_rhs(sr, g.d, i, n, g.k, g.j0, kc);
        cp_async_wait_all();
        __syncthreads();
        // prefetch step i+1 (W_i is also what bR needs after the last step)
        if (i < last) async_copy(nxt, g.Af + (i + 1) * (long long)nn, nn);
        if (!seq || i < last) async_copy(nxt + nn, g.Bf + i * (long long)nn, nn);
        if (!seq && i < last) async_copy(nxt + 2 * nn, g.Y + (i + 1) * (long long)nn, nn);
        cp_async_commit();
        if (i > first) {
            cta_tmul(cur + nn, sy, sr, n, kc, T(-1), true);
            __syncthreads();
        }
        cta_tmul(cur, sr, sy, n, kc, T(1), false);
        __syncthreads();
        if (!seq) cta_tmul(cur + 2 * nn, sy, sbL, n, kc, T(1), true);
        store_rhs(g.d, sy, i, n, g.k, g.j0, kc);
    }
    cp_async_wait_all();
    __syncthreads();
    if (!seq) {
        const T *wl = buf + (((last + 1 - first) & 1) * 3 + 1) * nn;  // W_last, prefetched in the last step
        cta_tmul(wl, sy, sbR, n, kc, T(1), false);
        __syncthreads();
        T *bp = g.bvec + p * 2 * (long long)n * kc;
        for (int e = threadIdx.x; e < n * kc; e += blockDim.x) {
            bp[e] = sbL[e];
            bp[n * kc + e] = sbR[e];
        }
        return;
    }
    // sequential level, backward: x_i = V_i (y_i - W_i x_{i+1}); step i uses
    // V_i (slot 0) and W_i (slot 1)
    async_copy(buf, g.Af + last * (long long)nn, nn);
    cp_async_commit();
    for (long long i = last; i >= first; --i) {
        T *cur = buf + ((last - i) & 1) * 3 * nn;
        T *nxt = buf + (((last - i) & 1) ^ 1) * 3 * nn;
        load_rhs(sr, g.d, i, n, g.k, g.j0, kc);
        cp_async_wait_all();
        __syncthreads();
        if (i > first) {
            async_copy(nxt, g.Af + (i - 1) * (long long)nn, nn);
            async_copy(nxt + nn, g.Bf + (i - 1) * (long long)nn, nn);
        }
        cp_async_commit();
        if (i < last) {
            cta_nmul<T>(cur + nn, sx, nullptr, nullptr, sr, sr, T(-1), n, kc, red);
            __syncthreads();
        }
        cta_nmul<T>(cur, sr, nullptr, nullptr, nullptr, sx, T(1), n, kc, red);
        __syncthreads();
        store_rhs(g.d, sx, i, n, g.k, g.j0, kc);
    }
    cp_async_wait_all();
}

// separator RHS: d'_s = d_{sep s} - bL(s) - bR(s-1)   (reference compute_schur_RHS!,
// backbone_cuda.jl:159-171, and the gather gpu_batched.jl:251)
template <class T, class Tn>
__global__ void assemble_rhs_kernel(const T *__restrict__ d, const T *__restrict__ bvec, Tn *__restrict__ dn,
                                    long long N, long long Q, int n, int k, int j0, int kc)
{
    const long long per = (long long)n * kc;
    const long long total = (Q + 1) * per;
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < total;
         e += (long long)gridDim.x * blockDim.x) {
        const long long s = e / per, w = e % per;
        const long long blk = (s * (N - 1)) / Q;
        const long long off = (long long)j0 * n + w;
        double v = (double)d[blk * (long long)n * k + off];
        if (s < Q) v -= (double)bvec[s * 2 * per + w];
        if (s > 0) v -= (double)bvec[(s - 1) * 2 * per + per + w];
        dn[s * (long long)n * k + off] = (Tn)v;
    }
}

// backward sweep of one partition: x_i = V_i (y_i - Y_i x_L - W_i x_{i+1}),
// x_{last+1} = x_R; also writes x_L (and x_R for the last partition) into
// the level's separator slots (reference update_boundary! + the scatter
// gpu_batched.jl:253, and cholesky_solve_batched! :257).
template <class T, class Tsep>
__global__ void __launch_bounds__(SOLVE_THREADS) chain_bwd_kernel(SolveArgs<T> g)
{
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int n = g.n, kc = g.kc;
    const int nn = n * n;
    T *buf = reinterpret_cast<T *>(smem_raw);  // [2][3][nn]: V_i, W_i, Y_i
    T *sz = buf + 6 * nn;
    T *sxL = sz + n * kc;
    T *sxn = sxL + n * kc;
    T *sxt = sxn + n * kc;
    T *red = sxt + 2 * n * kc;
    const long long p = blockIdx.x;
    const long long sL = (p * (g.N - 1)) / g.Q;
    const long long sR = ((p + 1) * (g.N - 1)) / g.Q;
    const long long first = sL + 1, last = sR - 1;
    const Tsep *xs = reinterpret_cast<const Tsep *>(g.xsep);
    async_copy(buf, g.Af + last * (long long)nn, nn);
    async_copy(buf + nn, g.Bf + last * (long long)nn, nn);
    async_copy(buf + 2 * nn, g.Y + last * (long long)nn, nn);
    cp_async_commit();
    load_rhs(sxL, xs, p, n, g.k, g.j0, kc);
    load_rhs(sxn, xs, p + 1, n, g.k, g.j0, kc);
    __syncthreads();
    store_rhs(g.d, sxL, sL, n, g.k, g.j0, kc);
    if (p == g.Q - 1) store_rhs(g.d, sxn, sR, n, g.k, g.j0, kc);
    for (long long i = last; i >= first; --i) {
        T *cur = buf + ((last - i) & 1) * 3 * nn;
        T *nxt = buf + (((last - i) & 1) ^ 1) * 3 * nn;
        load_rhs(sz, g.d, i, n, g.k, g.j0, kc);
        cp_async_wait_all();
        __syncthreads();
        if (i > first) {
            async_copy(nxt, g.Af + (i - 1) * (long long)nn, nn);
            async_copy(nxt + nn, g.Bf + (i - 1) * (long long)nn, nn);
            async_copy(nxt + 2 * nn, g.Y + (i - 1) * (long long)nn, nn);
        }
        cp_async_commit();
        cta_nmul<T>(cur + 2 * nn, sxL, cur + nn, sxn, sz, sz, T(-1), n, kc, red);
        __syncthreads();
        cta_nmul<T>(cur, sz, nullptr, nullptr, nullptr, sxt, T(1), n, kc, red);
        __syncthreads();
        for (int e = threadIdx.x; e < n * kc; e += blockDim.x) sxn[e] = sxt[e];
        store_rhs(g.d, sxt, i, n, g.k, g.j0, kc);
        __syncthreads();
    }
    cp_async_wait_all();
}

// ---------------------------------------------------------------------------
// FP64 refinement helpers
// ---------------------------------------------------------------------------
// ||T||_inf: row sums of |A_i| + |B_i| (rows) + |B_{i-1}| (columns)
template <class T>
__global__ void opnorm_kernel(const T *__restrict__ A, const T *__restrict__ B, long long N, int n,
                              DevStatus *st)
{
    const long long nn = (long long)n * n;
    double best = 0.0;
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < N * n;
         e += (long long)gridDim.x * blockDim.x) {
        const long long i = e / n;
        const int r = (int)(e % n);
        double s = 0.0;
        for (int c = 0; c < n; ++c) s += fabs((double)A[i * nn + r + (long long)c * n]);
        if (i + 1 < N)
            for (int c = 0; c < n; ++c) s += fabs((double)B[i * nn + r + (long long)c * n]);
        if (i >= 1)
            for (int c = 0; c < n; ++c) s += fabs((double)B[(i - 1) * nn + c + (long long)r * n]);
        best = fmax(best, s);
    }
    for (int o = 16; o > 0; o >>= 1) best = fmax(best, __shfl_xor_sync(0xffffffffu, best, o));
    if ((threadIdx.x & 31) == 0) atomic_max_nonneg(&st->anorm, best);
}

template <class T>
__global__ void absmax_kernel(const T *__restrict__ v, long long count, unsigned long long *dst)
{
    double best = 0.0;
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < count;
         e += (long long)gridDim.x * blockDim.x)
        best = fmax(best, fabs((double)v[e]));
    for (int o = 16; o > 0; o >>= 1) best = fmax(best, __shfl_xor_sync(0xffffffffu, best, o));
    if ((threadIdx.x & 31) == 0) atomic_max_nonneg(dst, best);
}

// r = d - T x in FP64 for one block per CTA; writes r (as Tr) and folds
// max|r| and max|x| into the status.
template <class T, class Tr>
__global__ void residual_kernel(const T *__restrict__ A, const T *__restrict__ B, const T *__restrict__ x,
                                const T *__restrict__ d, Tr *__restrict__ r, long long N, int n, int k,
                                DevStatus *st)
{
    extern __shared__ __align__(16) unsigned char smem_raw[];
    double *sBt = reinterpret_cast<double *>(smem_raw);  // B_{i-1}, ld n+1
    double *sx = sBt + n * (n + 1);                       // x_{i-1}, x_i, x_{i+1}: 3 * n * k
    const long long i = blockIdx.x;
    const long long nn = (long long)n * n;
    const long long nk = (long long)n * k;
    for (int e = threadIdx.x; e < 3 * n * k; e += blockDim.x) {
        const int q = e / (n * k), w = e % (n * k);
        const long long blk = i - 1 + q;
        sx[e] = (blk >= 0 && blk < N) ? (double)x[blk * nk + w] : 0.0;
    }
    if (i >= 1)
        for (int e = threadIdx.x; e < n * n; e += blockDim.x) {
            const int rr = e % n, cc = e / n;
            sBt[rr + cc * (n + 1)] = (double)B[(i - 1) * nn + e];
        }
    __syncthreads();
    double rmax = 0.0, xmax = 0.0;
    for (int o = threadIdx.x; o < n * k; o += blockDim.x) {
        const int row = o % n, j = o / n;
        double s = (double)d[i * nk + o];
        const double *xm = sx + j * n;
        const double *x0 = sx + n * k + j * n;
        const double *xp = sx + 2 * n * k + j * n;
        for (int c = 0; c < n; ++c) s = fma(-(double)A[i * nn + row + (long long)c * n], x0[c], s);
        if (i + 1 < N)
            for (int c = 0; c < n; ++c) s = fma(-(double)B[i * nn + row + (long long)c * n], xp[c], s);
        if (i >= 1)
            for (int c = 0; c < n; ++c) s = fma(-sBt[c + row * (n + 1)], xm[c], s);
        if (r) r[i * nk + o] = (Tr)s;
        rmax = fmax(rmax, fabs(s));
        xmax = fmax(xmax, fabs(x0[row]));
    }
    for (int o = 16; o > 0; o >>= 1) {
        rmax = fmax(rmax, __shfl_xor_sync(0xffffffffu, rmax, o));
        xmax = fmax(xmax, __shfl_xor_sync(0xffffffffu, xmax, o));
    }
    if ((threadIdx.x & 31) == 0) {
        atomic_max_nonneg(&st->rnorm, rmax);
        atomic_max_nonneg(&st->xnorm, xmax);
    }
}

static __global__ void relres_kernel(DevStatus *st, double tol)
{
    if (threadIdx.x == 0 && blockIdx.x == 0) {
        const double rn = __longlong_as_double((long long)st->rnorm);
        const double xn = __longlong_as_double((long long)st->xnorm);
        const double dn = __longlong_as_double((long long)st->dnorm);
        const double an = __longlong_as_double((long long)st->anorm);
        const double den = an * xn + dn;
        const double rel = den > 0.0 ? rn / den : 0.0;
        st->relres = rel;
        st->done = (rel <= tol) ? 1 : 0;
    }
}

// x (+)= c  (FP64 accumulation of an FP32 correction)
template <class Tc>
__global__ void update_kernel(double *__restrict__ x, const Tc *__restrict__ c, long long count, int assign)
{
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < count;
         e += (long long)gridDim.x * blockDim.x)
        x[e] = assign ? (double)c[e] : x[e] + (double)c[e];
}

template <class Ts, class Td>
__global__ void convert_kernel(Td *__restrict__ dst, const Ts *__restrict__ src, long long count)
{
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < count;
         e += (long long)gridDim.x * blockDim.x)
        dst[e] = (Td)src[e];
}

template <class T>
__global__ void init_identity_kernel(T *A, long long first_blk, long long last_blk, int n)
{
    const long long nn = (long long)n * n;
    const long long total = (last_blk - first_blk) * nn;
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < total;
         e += (long long)gridDim.x * blockDim.x) {
        const long long w = e % nn;
        A[first_blk * nn + e] = ((w % n) == (w / n)) ? T(1) : T(0);
    }
}

}  // namespace bss
