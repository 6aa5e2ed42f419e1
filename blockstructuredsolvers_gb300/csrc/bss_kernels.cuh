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

#include <cuda.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include <type_traits>

#include "bss_tc.cuh"

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
    int iters;        // refinement corrections applied by the last solve
    int need_anorm;   // the next residual also accumulates ||T||_inf
    int active;       // batch refinement: this system takes the pending correction
    unsigned long long iters_total;  // corrections over all device-loop solves (never reset)
    int tc_timeout;   // a bounded tensor-core wait expired (the factorization is void)
    int pad_;
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
// Structure flags (all decided at compile time, per 16-row segment of k):
//   TRI : X is upper triangular, so X(k, i) = 0 for k > i; in k-segment s only
//         rows with a >= s contribute (row ti+16a < 16s otherwise).
//   SYM : only C's upper block pairs a <= b are needed (symmetric result).
enum { TN_FULL = 0, TN_TRI = 1, TN_SYM = 2 };

template <class T, int NB, int F1>
__device__ __forceinline__ void tn_acc(T (&acc)[Tile<NB>::RA][Tile<NB>::RB], const T *X, const T *Y, int ti, int tj)
{
    using TL = Tile<NB>;
    using V = typename Vec<T>::type;
    constexpr int LD = Geo<T, NB>::LD;
    constexpr int W = Vec<T>::W;
    static_assert(TL::TI == 16, "segments are 16 rows");
#pragma unroll
    for (int seg = 0; seg < NB / 16; ++seg) {
#pragma unroll 2
        for (int kk = 0; kk < 16; kk += W) {
            const int k = 16 * seg + kk;
            V xa[TL::RA], yb[TL::RB];
#pragma unroll
            for (int a = 0; a < TL::RA; ++a)
                if (!(F1 & TN_TRI) || a >= seg) xa[a] = *reinterpret_cast<const V *>(X + k + (ti + TL::TI * a) * LD);
#pragma unroll
            for (int b = 0; b < TL::RB; ++b) yb[b] = *reinterpret_cast<const V *>(Y + k + (tj + TL::TJ * b) * LD);
#pragma unroll
            for (int a = 0; a < TL::RA; ++a)
#pragma unroll
                for (int b = 0; b < TL::RB; ++b)
                    if ((!(F1 & TN_TRI) || a >= seg) && (!(F1 & TN_SYM) || (TL::TI * a <= TL::TJ * b + TL::TJ - 1)))
                        fma_vec(acc[a][b], xa[a], yb[b]);
        }
    }
}

// acc1 += X^T Y1 (flags F1), acc2 += X^T Y2 (flags F2), shared X reads.
// TRI applies to X and so must be given to both or neither.
template <class T, int NB, int F1, int F2>
__device__ __forceinline__ void tn_acc2(T (&acc1)[Tile<NB>::RA][Tile<NB>::RB],
                                        T (&acc2)[Tile<NB>::RA][Tile<NB>::RB], const T *X, const T *Y1,
                                        const T *Y2, int ti, int tj)
{
    using TL = Tile<NB>;
    using V = typename Vec<T>::type;
    constexpr int LD = Geo<T, NB>::LD;
    constexpr int W = Vec<T>::W;
    static_assert(TL::TI == 16, "segments are 16 rows");
    static_assert((F1 & TN_TRI) == (F2 & TN_TRI), "TRI describes X");
#pragma unroll
    for (int seg = 0; seg < NB / 16; ++seg) {
#pragma unroll 2
        for (int kk = 0; kk < 16; kk += W) {
            const int k = 16 * seg + kk;
            V xa[TL::RA], yb[TL::RB], zb[TL::RB];
#pragma unroll
            for (int a = 0; a < TL::RA; ++a)
                if (!(F1 & TN_TRI) || a >= seg) xa[a] = *reinterpret_cast<const V *>(X + k + (ti + TL::TI * a) * LD);
#pragma unroll
            for (int b = 0; b < TL::RB; ++b) {
                yb[b] = *reinterpret_cast<const V *>(Y1 + k + (tj + TL::TJ * b) * LD);
                zb[b] = *reinterpret_cast<const V *>(Y2 + k + (tj + TL::TJ * b) * LD);
            }
#pragma unroll
            for (int a = 0; a < TL::RA; ++a)
#pragma unroll
                for (int b = 0; b < TL::RB; ++b) {
                    if (!(F1 & TN_TRI) || a >= seg) {
                        if (!(F1 & TN_SYM) || (TL::TI * a <= TL::TJ * b + TL::TJ - 1)) fma_vec(acc1[a][b], xa[a], yb[b]);
                        if (!(F2 & TN_SYM) || (TL::TI * a <= TL::TJ * b + TL::TJ - 1)) fma_vec(acc2[a][b], xa[a], zb[b]);
                    }
                }
        }
    }
}

// store a symmetric result computed on its upper block pairs: element
// (r, c) of every computed pair, plus its mirror (c, r) when the whole pair
// lies above the diagonal
template <class T, int NB>
__device__ __forceinline__ void store_sym_global(T *__restrict__ g, const T (&src)[Tile<NB>::RA][Tile<NB>::RB], int n,
                                                 int ti, int tj)
{
    using TL = Tile<NB>;
#pragma unroll
    for (int a = 0; a < TL::RA; ++a)
#pragma unroll
        for (int b = 0; b < TL::RB; ++b) {
            const int r = ti + TL::TI * a, c = tj + TL::TJ * b;
            if (TL::TI * a > TL::TJ * b + TL::TJ - 1) continue;         // pair not computed
            const bool strictly_upper = (TL::TI * a + TL::TI - 1 < TL::TJ * b);  // every element r < c
            if (r < n && c < n) {
                g[r + (size_t)c * n] = src[a][b];
                if (strictly_upper) g[c + (size_t)r * n] = src[a][b];
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
// scratch, and sV holds V = U^{-1} (upper, zeros below the diagonal
// -- the caller zeroes sV's strictly lower tiles once).
// Panels are PB = 16 wide: one warp factors each
// PB x PB diagonal tile with shuffles (lane r owns column r; the diagonal is
// carried in its own register so the pivot chain is shuffle -> rsqrt -> fma),
// another warp inverts it by per-lane back substitution while the rest of
// the CTA solves the row panel; the trailing update is spread over the CTA,
// and V's off-diagonal block columns are formed by the other warps while
// warp 0 factors the next diagonal tile.  The helpers are kept out of line:
// inlined together into the chain kernel they push arrays to local memory.
// ---------------------------------------------------------------------------

// 1/sqrt of a pivot: the hardware approximation in FP32 (2 ulp; FP32
// factors are refined in FP64 or checked at 1e-4), IEEE sqrt and divide in FP64
__device__ __forceinline__ float rsqrt_pivot(float p) { return rsqrtf(p); }
__device__ __forceinline__ double rsqrt_pivot(double p) { return 1.0 / sqrt(p); }

// 16-wide panels measured faster than 32-wide ones on GB300 for NB = 64
// (24k vs 30k cycles per 64x64 factorization in one CTA): the warp
// factorization of a diagonal tile is bound by shuffle issue, which grows
// with the panel width, and the 32x32 inverse stage costs more than three
// 16x16 ones.
template <int NB>
struct Panel {
    static constexpr int PB = 16;
};

template <class T, int LD, int PB>
__device__ __forceinline__ int warp_chol_i(T *sS, T *dinv, int o, int lane)
{
    const int r = lane & (PB - 1);
    T u[PB];
#pragma unroll
    for (int c = 0; c < PB; ++c) u[c] = sS[(o + c) + (o + r) * LD];  // S(o+c, o+r), valid for c <= r
    T diag = sS[(o + r) + (o + r) * LD];
    int bad = 0;
    T udiag = T(1);
#pragma unroll
    for (int j = 0; j < PB; ++j) {
        T piv = __shfl_sync(0xffffffffu, diag, j);
        if (!(piv > T(0) && piv < T(INFINITY))) {
            bad = 1;
            piv = T(1);
        }
        const T rs = rsqrt_pivot(piv);
        const T ujr = (r == j ? diag : u[j]) * rs;  // U(j, r) for r >= j
        if (j == r) udiag = ujr;
        diag = fma(-ujr, ujr, diag);                // own column's diagonal: the pivot chain
        u[j] = ujr;
#pragma unroll
        for (int c = j + 1; c < PB; ++c) {
            const T ujc = __shfl_sync(0xffffffffu, ujr, c);  // U(j, c) from lane c
            u[c] = fma(-ujc, ujr, u[c]);                      // S(c, r) -= U(j,c) U(j,r)
        }
    }
    if (lane < PB) {
#pragma unroll
        for (int c = 0; c < PB; ++c)
            if (c <= r) sS[(o + c) + (o + r) * LD] = (c == r) ? udiag : u[c];
        dinv[o + r] = T(1) / udiag;
    }
    return bad;
}
template <class T, int LD, int PB>
__device__ __noinline__ int warp_chol(T *sS, T *dinv, int o, int lane)
{
    return warp_chol_i<T, LD, PB>(sS, dinv, o, lane);
}

// V_KK = U_KK^{-1}: lane r computes column r by back substitution.
template <class T, int LD, int PB>
__device__ __forceinline__ void warp_inv_i(const T *sS, const T *dinv, T *sV, int o, int lane)
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
template <class T, int LD, int PB>
__device__ __noinline__ void warp_inv(const T *sS, const T *dinv, T *sV, int o, int lane)
{
    warp_inv_i<T, LD, PB>(sS, dinv, sV, o, lane);
}

// row panel right of diagonal tile o: U(o:o+PB, c) = U_KK^{-T} S(o:o+PB, c)
template <class T, int LD, int NB, int PB>
__device__ __forceinline__ void panel_trsm_i(T *sS, const T *dinv, int o, int t0, int nthr)
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
template <class T, int LD, int NB, int PB>
__device__ __noinline__ void panel_trsm(T *sS, const T *dinv, int o, int t0, int nthr)
{
    panel_trsm_i<T, LD, NB, PB>(sS, dinv, o, t0, nthr);
}

// S(a, b) -= sum_p U(o+p, a) U(o+p, b)   for o+PB <= a <= b < NB
template <class T, int LD, int NB, int PB>
__device__ __forceinline__ void trailing_update_i(T *sS, int o, int tid, int nthr)
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
template <class T, int LD, int NB, int PB>
__device__ __noinline__ void trailing_update(T *sS, int o, int tid, int nthr)
{
    trailing_update_i<T, LD, NB, PB>(sS, o, tid, nthr);
}

// off-diagonal tiles of V = U^{-1} after the factorization (FP64 chains):
// V_IJ = -V_II sum_{P=I+1..J} U_IP V_PJ, one super-diagonal stage at a time
// (s = J - I), all threads on every stage; T_IJ is kept in the (scratch)
// lower tile (J, I) of sS.  On GB300's FP64 pipe a warp-instruction costs
// its full slot whatever lanes are active, so FP64 takes this form, whose
// element-parallel stages skip the zero halves of the triangular tiles.
template <class T, int LD, int NB, int PB>
__device__ __noinline__ void inverse_stages(T *sS, T *sV, int tid, int nthr)
{
    constexpr int KP = NB / PB;
#pragma unroll 1
    for (int s = 1; s < KP; ++s) {
        const int ntile = KP - s;
        for (int e = tid; e < ntile * PB * PB; e += nthr) {
            const int tile = e / (PB * PB), w = e - tile * PB * PB;
            const int a = w % PB, b = w / PB;
            const int I = tile, J = tile + s;
            T acc0 = T(0), acc1 = T(0);
            for (int P = I + 1; P <= J; ++P)
#pragma unroll
                for (int q = 0; q < PB; q += 2) {
                    acc0 = fma(sS[(PB * I + a) + (PB * P + q) * LD], sV[(PB * P + q) + (PB * J + b) * LD], acc0);
                    acc1 = fma(sS[(PB * I + a) + (PB * P + q + 1) * LD], sV[(PB * P + q + 1) + (PB * J + b) * LD],
                               acc1);
                }
            sS[(PB * J + a) + (PB * I + b) * LD] = acc0 + acc1;
        }
        __syncthreads();
        for (int e = tid; e < ntile * PB * PB; e += nthr) {
            const int tile = e / (PB * PB), w = e - tile * PB * PB;
            const int a = w % PB, b = w / PB;
            const int I = tile, J = tile + s;
            T acc0 = T(0), acc1 = T(0);
            for (int c = a; c < PB; c += 2) {
                acc0 = fma(sV[(PB * I + a) + (PB * I + c) * LD], sS[(PB * J + c) + (PB * I + b) * LD], acc0);
                if (c + 1 < PB)
                    acc1 = fma(sV[(PB * I + a) + (PB * I + c + 1) * LD], sS[(PB * J + c + 1) + (PB * I + b) * LD],
                               acc1);
            }
            sV[(PB * I + a) + (PB * J + b) * LD] = -(acc0 + acc1);
        }
        __syncthreads();
    }
}

// Off-diagonal block column J of V = U^{-1} (rows I < J), from V U = I:
//   V_IJ = -(sum_{P=I..J-1} V_IP U_PJ) V_JJ
// Needs U's block rows above J (final once their row panels are solved) and
// V's block columns left of J, so it runs while the next diagonal tile is
// being factored.  One thread per row (I, a): the 16 sums T(a, :) in
// registers, then the row of -T V_JJ.
template <class T, int LD, int PB>
__device__ __forceinline__ void inv_column_i(const T *sS, T *sV, int J, int t0, int nthr)
{
    for (int e = t0; e < J * PB; e += nthr) {
        const int I = e / PB, a = e - I * PB;
        T t[PB];
#pragma unroll
        for (int c = 0; c < PB; ++c) t[c] = T(0);
        for (int P = I; P < J; ++P)
#pragma unroll 4
            for (int q = 0; q < PB; ++q) {
                const T v = sV[(PB * I + a) + (PB * P + q) * LD];  // V_IP(a, q)
#pragma unroll
                for (int c = 0; c < PB; ++c) t[c] = fma(v, sS[(PB * P + q) + (PB * J + c) * LD], t[c]);  // U_PJ(q, c)
            }
#pragma unroll 4
        for (int b = 0; b < PB; ++b) {
            T acc0 = T(0), acc1 = T(0);
#pragma unroll
            for (int c = 0; c < PB; c += 2) {
                acc0 = fma(t[c], sV[(PB * J + c) + (PB * J + b) * LD], acc0);
                acc1 = fma(t[c + 1], sV[(PB * J + c + 1) + (PB * J + b) * LD], acc1);
            }
            sV[(PB * I + a) + (PB * J + b) * LD] = -(acc0 + acc1);
        }
    }
}
template <class T, int LD, int PB>
__device__ __noinline__ void inv_column(const T *sS, T *sV, int J, int t0, int nthr)
{
    inv_column_i<T, LD, PB>(sS, sV, J, t0, nthr);
}

// ---- FP32 forms of the panel steps for callers with registers to spare ------
// Measured on GB300 (one 64 x 64 tile, 256 threads, alone on an SM): the
// 16-wide pivot chain took ~3.1K cycles with one shuffle per broadcast
// element and ~2.5K with the pivot row broadcast through shared memory; the
// first panel's trailing update ~2.6K with one 16-term dot per loop trip and
// ~1.8K register-tiled; the last block column of V ~3.6K on 48 threads and
// ~2.3K element-parallel on 256.  The whole factorization + inverse: 25.0K
// -> 20.7K cycles.

// 16-wide panel Cholesky by one warp (as warp_chol_i), the pivot row U(j, :)
// broadcast through `row` (64 floats of shared memory, double-buffered): one
// 32-lane store and four 128-bit broadcast reads per pivot instead of up to
// 15 dependent shuffles; the one element the next pivot needs, U(j, j+1),
// comes by a shuffle, so the shared-memory round trip is off the pivot chain
template <int LD, int PB>
__device__ __forceinline__ int warp_chol_row(float *sS, float *dinv, float *row, int o, int lane)
{
    const int r = lane & (PB - 1);
    float u[PB];
#pragma unroll
    for (int c = 0; c < PB; ++c) u[c] = sS[(o + c) + (o + r) * LD];  // S(o+c, o+r), valid for c <= r
    float diag = sS[(o + r) + (o + r) * LD];
    int bad = 0;
    float udiag = 1.f;
#pragma unroll
    for (int j = 0; j < PB; ++j) {
        float piv = __shfl_sync(0xffffffffu, diag, j);
        if (!(piv > 0.f && piv < INFINITY)) {
            bad = 1;
            piv = 1.f;
        }
        const float rs = rsqrtf(piv);
        const float ujr = (r == j ? diag : u[j]) * rs;  // U(j, r) for r >= j
        if (j == r) udiag = ujr;
        diag = fmaf(-ujr, ujr, diag);  // own column's diagonal: the pivot chain
        u[j] = ujr;
        if (j + 1 < PB) {
            // the next pivot needs only U(j, j+1) of this row: one shuffle keeps
            // it off the shared-memory round trip; the rest of the row (needed
            // from pivot j + 2 on) goes through shared memory meanwhile
            const float ujn = __shfl_sync(0xffffffffu, ujr, j + 1);
            u[j + 1] = fmaf(-ujn, ujr, u[j + 1]);
            if (j + 2 < PB) {
                float *rj = row + 32 * (j & 1);
                if (lane < PB) rj[r] = ujr;
                __syncwarp();
#pragma unroll
                for (int c4 = ((j + 2) / 4) * 4; c4 < PB; c4 += 4) {
                    const float4 v = *reinterpret_cast<const float4 *>(rj + c4);
                    const float ua[4] = {v.x, v.y, v.z, v.w};
#pragma unroll
                    for (int t = 0; t < 4; ++t)
                        if (c4 + t > j + 1) u[c4 + t] = fmaf(-ua[t], ujr, u[c4 + t]);  // S(c, r) -= U(j,c) U(j,r)
                }
            }
        }
    }
    if (lane < PB) {
#pragma unroll
        for (int c = 0; c < PB; ++c)
            if (c <= r) sS[(o + c) + (o + r) * LD] = (c == r) ? udiag : u[c];
        dinv[o + r] = 1.f / udiag;
    }
    return bad;
}

// trailing update of panel o in FP32: S(a, b) -= sum_p U(o+p, a) U(o+p, b)
// for the trailing columns b >= bfirst (relative to the trailing block),
// over nw warps (this one is warp wi of them): lanes take rows a (a + 32,
// ... up to the tile), warps take columns b; a thread keeps its U columns in
// registers and reads each U(., b) as a broadcast, all in 128-bit steps
// (column reads conflict-free for LD = NB + 4).  The Cholesky reads only the
// upper triangle, so row groups wholly below the diagonal are skipped.
template <int LD, int NB, int PB>
__device__ __forceinline__ void trailing_update_f32(float *sS, int o, int bfirst, int wi, int nw, int lane)
{
    static_assert(PB == 16, "four float4 per column segment");
    constexpr int H = (NB - PB + 31) / 32;  // row groups of 32 per lane
    const int m = NB - o - PB, c0 = o + PB;
    float4 ua[H][4];
#pragma unroll
    for (int h = 0; h < H; ++h) {
        const int a = lane + 32 * h;
        if (a < m) {
#pragma unroll
            for (int q = 0; q < 4; ++q) ua[h][q] = *reinterpret_cast<const float4 *>(sS + o + 4 * q + (c0 + a) * LD);
        }
    }
    for (int b = bfirst + wi; b < m; b += nw) {
        float4 ub[4];
#pragma unroll
        for (int q = 0; q < 4; ++q) ub[q] = *reinterpret_cast<const float4 *>(sS + o + 4 * q + (c0 + b) * LD);
#pragma unroll
        for (int h = 0; h < H; ++h) {
            const int a = lane + 32 * h;
            if (a < m && 32 * h <= b) {
                float acc = 0.f;
#pragma unroll
                for (int q = 0; q < 4; ++q) fma_vec(acc, ua[h][q], ub[q]);
                sS[(c0 + a) + (c0 + b) * LD] -= acc;
            }
        }
    }
}

// the next diagonal tile of panel o (rows and columns o + PB .. o + 2 PB - 1)
// updated by one warp: lane l takes column b = l % 16 and rows 8 (l / 16) .. +7
template <int LD, int PB>
__device__ __forceinline__ void tile_update_f32(float *sS, int o, int lane)
{
    static_assert(PB == 16, "four float4 per column segment");
    const int c0 = o + PB, b = lane & 15, a0 = (lane >> 4) * 8;
    float4 ub[4];
#pragma unroll
    for (int q = 0; q < 4; ++q) ub[q] = *reinterpret_cast<const float4 *>(sS + o + 4 * q + (c0 + b) * LD);
#pragma unroll
    for (int r = 0; r < 8; ++r) {
        const int a = a0 + r;
        float acc = 0.f;
#pragma unroll
        for (int q = 0; q < 4; ++q) fma_vec(acc, *reinterpret_cast<const float4 *>(sS + o + 4 * q + (c0 + a) * LD), ub[q]);
        sS[(c0 + a) + (c0 + b) * LD] -= acc;
    }
}

// Off-diagonal block column J of V = U^{-1} in FP32, element-parallel over
// `nthr` threads from t0 in two stages (`bar` = the barrier joining exactly
// those threads: 0 for the whole CTA, else a named barrier):
//   T_IJ = sum_{P=I..J-1} V_IP U_PJ      kept in the scratch lower tile (J, I) of sS
//   V_IJ = -T_IJ V_JJ
// The lower tiles of sS are never read as matrix data (the Cholesky reads
// the upper triangle), and (J, I) lies outside the diagonal tile being
// factored while this runs.
template <int LD, int PB>
__device__ __forceinline__ void inv_column_par(float *sS, float *sV, int J, int t0, int nthr, int bar)
{
    const int total = J * PB * PB;
    for (int e = t0; e < total; e += nthr) {
        const int I = e / (PB * PB), w = e - I * PB * PB;
        const int a = w % PB, c = w / PB;
        float s0 = 0.f, s1 = 0.f;
        for (int P = I; P < J; ++P)
#pragma unroll
            for (int q = 0; q < PB; q += 4) {
                const float4 u = *reinterpret_cast<const float4 *>(sS + (PB * P + q) + (PB * J + c) * LD);  // U_PJ(q.., c)
                const float *vr = sV + (PB * I + a) + (PB * P + q) * LD;                                   // V_IP(a, q..)
                s0 = fmaf(vr[0], u.x, s0);
                s1 = fmaf(vr[LD], u.y, s1);
                s0 = fmaf(vr[2 * LD], u.z, s0);
                s1 = fmaf(vr[3 * LD], u.w, s1);
            }
        sS[(PB * J + a) + (PB * I + c) * LD] = s0 + s1;
    }
    if (bar == 0)
        __syncthreads();
    else
        asm volatile("bar.sync %0, %1;" ::"r"(bar), "r"(nthr) : "memory");
    for (int e = t0; e < total; e += nthr) {
        const int I = e / (PB * PB), w = e - I * PB * PB;
        const int a = w % PB, b = w / PB;
        float s0 = 0.f, s1 = 0.f;
#pragma unroll
        for (int c = 0; c < PB; c += 4) {
            const float4 v = *reinterpret_cast<const float4 *>(sV + (PB * J + c) + (PB * J + b) * LD);  // V_JJ(c.., b)
            const float *tr = sS + (PB * J + a) + (PB * I + c) * LD;                                   // T(a, c..)
            s0 = fmaf(tr[0], v.x, s0);
            s1 = fmaf(tr[LD], v.y, s1);
            s0 = fmaf(tr[2 * LD], v.z, s0);
            s1 = fmaf(tr[3 * LD], v.w, s1);
        }
        sV[(PB * I + a) + (PB * J + b) * LD] = -(s0 + s1);
    }
}

// Factor the tile in sS into sV = U^{-1}.  Returns nonzero (in every thread)
// if a pivot failed.  Ends with a __syncthreads.  Per panel K: warp 0
// factors the diagonal tile while (FP32) the other warps form V's block
// column K-1; then warp 1 inverts the diagonal tile while the rest solve the
// row panel; then the trailing update.  V's last block column follows the
// loop (FP32); FP64 forms V's off-diagonal tiles in stages after it.
// The FAST form of tiles of 128 and more looks one panel ahead: once panel
// K's row panel is solved, warp 0 updates only the next diagonal tile and
// factors it at once, while the other warps update the rest of the trailing
// matrix and then form V's block column K (its diagonal tile was inverted
// with the row panel).  Measured on GB300 in the chain kernels: the 128 tile
// 71K -> 62K cycles per step; the 64 tile (four panels) gained nothing, and
// keeps the panel-by-panel order.
// INL: the panel helpers are inlined into the caller (no call saves and
// restores of the caller's registers on the critical warp); the default
// calls them out of line, which keeps register-heavy callers from spilling.
// FAST (FP32, with INL; `row` = 64 floats of shared memory): the FP32 forms
// above; the named barrier 1 joins the THREADS - 32 threads that form V's
// block columns during the panels.
// `idle(K)` runs on warps 1.. while warp 0 factors diagonal tile K and they
// have nothing else to do (panel-by-panel order: K < 2 in FP32, every K in
// FP64): the caller's own work, which must not touch sS, sV or dinv.
struct CholNoIdle {
    __device__ __forceinline__ void operator()(int) const {}
};

template <class T, int NB, int THREADS, bool INL = false, bool FAST = false, class Idle = CholNoIdle>
__device__ __forceinline__ int chol_inv_blocked(T *sS, T *sV, T *dinv, int *sflag, int tid, T *row = nullptr,
                                                Idle idle = Idle())
{
    static_assert(!FAST || (INL && sizeof(T) == 4), "the fast forms are inlined FP32");
    static_assert(THREADS > 32, "two warps at least");
    constexpr int LD = Geo<T, NB>::LD;
    constexpr int PB = Panel<NB>::PB;
    constexpr int KP = NB / PB;
    const int warp = tid >> 5, lane = tid & 31;
    if (tid == 0) *sflag = 0;
    if constexpr (FAST && NB >= 128) {
        if (warp == 0) {
            const int bad = warp_chol_row<LD, PB>(sS, dinv, row, 0, lane);
            if (bad && lane == 0) *sflag = 1;
        }
        __syncthreads();
#pragma unroll 1
        for (int K = 0; K < KP; ++K) {
            const int o = PB * K;
            // V_KK (warp 1) and the row panel U(K, K+1:) (the others)
            if (warp == 1)
                warp_inv_i<T, LD, PB>(sS, dinv, sV, o, lane);
            else if (K + 1 < KP)
                panel_trsm_i<T, LD, NB, PB>(sS, dinv, o, warp == 0 ? lane : tid - 32, THREADS - 32);
            __syncthreads();
            if (K + 1 < KP) {
                if (warp == 0) {  // the next diagonal tile, updated and factored by one warp
                    tile_update_f32<LD, PB>(sS, o, lane);
                    __syncwarp();
                    const int bad = warp_chol_row<LD, PB>(sS, dinv, row, o + PB, lane);
                    if (bad && lane == 0) *sflag = 1;
                } else {  // the rest of the trailing matrix, then V's block column K
                    trailing_update_f32<LD, NB, PB>(sS, o, PB, warp - 1, THREADS / 32 - 1, lane);
                    if (K >= 1) inv_column_par<LD, PB>(sS, sV, K, tid - 32, THREADS - 32, 1);
                }
            } else if (K >= 1) {
                inv_column_par<LD, PB>(sS, sV, K, tid, THREADS, 0);  // the last block column, all threads
            }
            __syncthreads();
        }
        return *sflag;
    } else {
#pragma unroll 1
    for (int K = 0; K < KP; ++K) {
        const int o = PB * K;
        if (warp == 0) {
            int bad;
            if constexpr (FAST)
                bad = warp_chol_row<LD, PB>(sS, dinv, row, o, lane);
            else if constexpr (INL)
                bad = warp_chol_i<T, LD, PB>(sS, dinv, o, lane);
            else
                bad = warp_chol<T, LD, PB>(sS, dinv, o, lane);
            if (bad && lane == 0) *sflag = 1;
        } else if (K >= 2 && sizeof(T) == 4) {
            if constexpr (FAST)
                inv_column_par<LD, PB>(sS, sV, K - 1, tid - 32, THREADS - 32, 1);
            else if constexpr (INL)
                inv_column_i<T, LD, PB>(sS, sV, K - 1, tid - 32, THREADS - 32);
            else
                inv_column<T, LD, PB>(sS, sV, K - 1, tid - 32, THREADS - 32);
        } else {
            idle(K);
        }
        __syncthreads();
        if (warp == 1) {
            if constexpr (INL)
                warp_inv_i<T, LD, PB>(sS, dinv, sV, o, lane);
            else
                warp_inv<T, LD, PB>(sS, dinv, sV, o, lane);
        }
        if (K + 1 < KP) {
            const int t0 = warp == 0 ? lane : tid - 32;
            if (warp != 1) {
                if constexpr (INL)
                    panel_trsm_i<T, LD, NB, PB>(sS, dinv, o, t0, THREADS - 32);
                else
                    panel_trsm<T, LD, NB, PB>(sS, dinv, o, t0, THREADS - 32);
            }
            __syncthreads();
            if constexpr (FAST)
                trailing_update_f32<LD, NB, PB>(sS, o, 0, warp, THREADS / 32, lane);
            else if constexpr (INL)
                trailing_update_i<T, LD, NB, PB>(sS, o, tid, THREADS);
            else
                trailing_update<T, LD, NB, PB>(sS, o, tid, THREADS);
        }
        __syncthreads();
    }
    if constexpr (sizeof(T) == 8) {
        inverse_stages<T, LD, NB, PB>(sS, sV, tid, THREADS);
    } else if (KP > 1) {
        if constexpr (FAST)
            inv_column_par<LD, PB>(sS, sV, KP - 1, tid, THREADS, 0);
        else if constexpr (INL)
            inv_column_i<T, LD, PB>(sS, sV, KP - 1, tid, THREADS);
        else
            inv_column<T, LD, PB>(sS, sV, KP - 1, tid, THREADS);
        __syncthreads();
    }
    return *sflag;
    }
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
    int variant;      // FACTOR_* bits: which kernel factors the chain
};

// kernel variants of a factorization (bits of ChainFactorArgs::variant),
// chosen per handle (the defaults, or the autotuner's choice per (n, dtype))
enum {
    FACTOR_FMA_CHAIN = 1,  // 33 <= n <= 64, FP32 factors: CUDA-core chain kernel instead of the tensor-core one
    FACTOR_WIDE_L2 = 2,    // 65 <= n <= 128, FP32 factors: the L2-staged wide kernel instead of chain128_tc
    FACTOR_VARIANTS = 3,   // every bit
};

template <class T, int NB>
constexpr size_t chain_factor_smem()
{
    return (size_t)(6 * Geo<T, NB>::SLOT + NB) * sizeof(T) + 16;
}

// one partition's chain (or the whole sequential chain when g.seq)
template <class Tin, class T, int NB>
__device__ __forceinline__ void chain_factor_body(const ChainFactorArgs<Tin, T> &g, const long long p)
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
                tn_acc2<T, NB, TN_SYM, TN_FULL>(accS, accZ, sW, sW, sY, ti, tj);
                store_tile_smem<T, NB>(sZ, accZ, ti, tj, T(-1));
            } else {
                tn_acc<T, NB, TN_SYM>(accS, sW, sW, ti, tj);
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
        const int bad = chol_inv_blocked<T, NB, TL::THREADS, NB == 64>(sS, sV, dinv, sflag, tid);
        if (bad && tid == 0) record_bad_pivot(g.st, g.level, i);

        T accY[TL::RA][TL::RB], accW[TL::RA][TL::RB];
        zero_tile<T, NB>(accY);
        zero_tile<T, NB>(accW);
        if (!seq)
            tn_acc2<T, NB, TN_TRI, TN_TRI>(accY, accW, sV, sZ, sB, ti, tj);
        else if (has_next)
            tn_acc<T, NB, TN_TRI>(accW, sV, sB, ti, tj);

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
        if (!seq) tn_acc<T, NB, TN_SYM>(accLL, sY, sY, ti, tj);
    }

    if (!seq) {
        T accRR[TL::RA][TL::RB], accLR[TL::RA][TL::RB];
        zero_tile<T, NB>(accRR);
        zero_tile<T, NB>(accLR);
        tn_acc<T, NB, TN_SYM>(accRR, sW, sW, ti, tj);
        tn_acc<T, NB, TN_FULL>(accLR, sY, sW, ti, tj);
        T *Cp = g.C + p * 3 * nn;
        store_sym_global<T, NB>(Cp, accLL, n, ti, tj);
        store_sym_global<T, NB>(Cp + nn, accRR, n, ti, tj);
        store_tile_global<T, NB>(Cp + 2 * nn, accLR, n, ti, tj, T(1));
    }
}

// work item of the batched (queue) kernels: descriptor index, partition
struct WorkItem {
    int desc;
    int p;
};

template <class Tin, class T, int NB>
__global__ void __launch_bounds__(Tile<NB>::THREADS, sizeof(T) == 4 ? 2 : 1) chain_factor_kernel(ChainFactorArgs<Tin, T> g)
{
    chain_factor_body<Tin, T, NB>(g, blockIdx.x);
}

// Persistent form for many systems: each CTA pulls (system, partition)
// items from a device queue (longest chains first, placed so by the host)
// until it is empty.  *head must be zero at launch.
template <class Tin, class T, int NB>
__global__ void __launch_bounds__(Tile<NB>::THREADS, sizeof(T) == 4 ? 2 : 1)
    chain_factor_queue_kernel(const ChainFactorArgs<Tin, T> *__restrict__ descs, const WorkItem *__restrict__ items,
                              int nitems, int *head)
{
    __shared__ int cur;
    for (;;) {
        if (threadIdx.x == 0) cur = atomicAdd(head, 1);
        __syncthreads();
        const int it = cur;
        __syncthreads();
        if (it >= nitems) break;
        const WorkItem w = items[it];
        const ChainFactorArgs<Tin, T> g = descs[w.desc];
        chain_factor_body<Tin, T, NB>(g, w.p);
        __syncthreads();
    }
}

// ---------------------------------------------------------------------------
// wide chain factor (n > 64): the recursion step of chain_factor_body with
// every n x n matrix of the chain in global memory -- the factor outputs
// V_i, W_i, Y_i are written there anyway, and a partition's working set
// (a few n x n blocks) stays in L2 -- processed in 64 x 64 tiles staged
// through shared memory (the Tile<64> products and the 64-wide blocked
// Cholesky of the fused path).  Per step, with tiles (I, J) of size 64:
//   S = A_i - W_{i-1}^T W_{i-1}                     (upper tiles, into V_i's slot)
//   Z = -W_{i-1}^T Y_{i-1}   (first step: B_sL^T)   (into Y_i's slot)
//   blocked Cholesky S = U^T U: diagonal tile K -> V_KK = U_KK^{-1} (stored in
//     place), row panel U(K,J) = V_KK^T S(K,J), trailing S(J1,J2) -= U^T U
//   V = U^{-1} in place: V(I,J) = -V_II sum_{P=I+1..J} U(I,P) V(P,J), columns
//     right to left, rows bottom-up (so every U read is not yet overwritten)
//   Y_i = V^T Z, W_i = V^T B_i    in place, row tiles bottom-up (V^T is lower)
//   S_LL += Y_i^T Y_i
// Data written in this kernel is read back with ld.global.cg (L2), never
// through the non-coherent read-only path.
// ---------------------------------------------------------------------------
constexpr int WT = 64;  // tile edge of the wide path

__device__ __forceinline__ float ld_cg(const float *p) { return __ldcg(p); }
__device__ __forceinline__ double ld_cg(const double *p) { return __ldcg(p); }

// tile (I, J) of op(M) (op = transpose or identity) of a column-major n x n
// matrix into the thread's Tile<64> registers; outside n x n: identity on
// the diagonal (diag_pad) or zero
template <class Tg, class T>
__device__ __forceinline__ void wload(T (&dst)[4][4], const Tg *g, int n, int I, int J, bool diag_pad,
                                      bool transpose)
{
    const int ti = threadIdx.x % 16, tj = threadIdx.x / 16;
#pragma unroll
    for (int a = 0; a < 4; ++a)
#pragma unroll
        for (int b = 0; b < 4; ++b) {
            const int gr = WT * I + ti + 16 * a, gc = WT * J + tj + 16 * b;
            T v;
            if (gr < n && gc < n)
                v = (T)(transpose ? ld_cg(g + gc + (size_t)gr * n) : ld_cg(g + gr + (size_t)gc * n));
            else
                v = (diag_pad && gr == gc) ? T(1) : T(0);
            dst[a][b] = v;
        }
}

template <class T>
__device__ __forceinline__ void wstore(T *g, const T (&src)[4][4], int n, int I, int J, T scale)
{
    const int ti = threadIdx.x % 16, tj = threadIdx.x / 16;
#pragma unroll
    for (int a = 0; a < 4; ++a)
#pragma unroll
        for (int b = 0; b < 4; ++b) {
            const int gr = WT * I + ti + 16 * a, gc = WT * J + tj + 16 * b;
            if (gr < n && gc < n) g[gr + (size_t)gc * n] = scale * src[a][b];
        }
}

// acc += sum_{K=k0..k1} op(X)(K, I)^T Y(K, J)  (tiles; op(X) = X^T when tx)
template <class Tx, class Ty, class T>
__device__ __forceinline__ void wide_tn(T (&acc)[4][4], const Tx *X, const Ty *Y, int n, int I, int J, int k0,
                                        int k1, T *sX, T *sY, bool tx)
{
    const int ti = threadIdx.x % 16, tj = threadIdx.x / 16;
    for (int K = k0; K <= k1; ++K) {
        T r[4][4];
        wload<Tx, T>(r, X, n, K, I, false, tx);
        store_tile_smem<T, 64>(sX, r, ti, tj, T(1));
        wload<Ty, T>(r, Y, n, K, J, false, false);
        store_tile_smem<T, 64>(sY, r, ti, tj, T(1));
        __syncthreads();
        tn_acc<T, 64, TN_FULL>(acc, sX, sY, ti, tj);
        __syncthreads();
    }
}

// shared memory of the wide kernel: four 64 x 64 tiles (sX, sY, sS, sV), the
// pivot reciprocals and a flag; the TC form puts the tensor-core operand
// stage first (128-byte aligned), the control words (mbarriers, TMEM
// address, abort flag) after it, and overlays sX and sY on the stage (the
// tile products of the Cholesky phase never overlap a tensor-core product)
template <class T, bool TC>
constexpr size_t wide_factor_smem()
{
    return TC ? (size_t)TC_NSTAGE * TC_STAGE_BYTES + 128 + (size_t)(2 * Geo<T, 64>::SLOT + WT) * sizeof(T) + 16
              : (size_t)(4 * Geo<T, 64>::SLOT + WT) * sizeof(T) + 16;
}

// tensor-core form of the wide kernel: FP32 chains of blocks up to 128
template <class T>
__host__ __device__ constexpr bool wide_uses_tc(int n)
{
    return std::is_same<T, float>::value && n <= 128;
}

constexpr int WIDE_THREADS = 256;

template <class Tin, class T, bool TC>
__device__ __noinline__ void wide_chain_factor_body(const ChainFactorArgs<Tin, T> &g, const long long p, TcCtx &tcc)
{
    constexpr int SLOT = Geo<T, 64>::SLOT;
    constexpr int LD = Geo<T, 64>::LD;
    extern __shared__ __align__(128) unsigned char smem_wide[];
    unsigned char *tc_stage = smem_wide;  // TC form only
    static_assert(!TC || 2 * SLOT * sizeof(T) <= TC_STAGE_BYTES, "sX, sY overlay the tensor-core stage");
    T *sX = reinterpret_cast<T *>(smem_wide);
    T *sY = sX + SLOT;
    T *sS = TC ? reinterpret_cast<T *>(smem_wide + TC_NSTAGE * TC_STAGE_BYTES + 128) : sY + SLOT;
    T *sV = sS + SLOT;
    T *dinv = sV + SLOT;
    int *sflag = reinterpret_cast<int *>(dinv + WT);
    const int tid = threadIdx.x, ti = tid % 16, tj = tid / 16;
    const int n = g.n;
    const int NT = (n + WT - 1) / WT;
    const long long nn = (long long)n * n;
    const bool seq = g.seq != 0;
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
    for (int e = tid; e < SLOT; e += WIDE_THREADS) sV[e] = T(0);  // V_KK's strictly lower panels stay zero
    __syncthreads();

    for (long long i = first; i <= last; ++i) {
        const long long t = i - first;
        const bool has_next = !seq || (i < g.N - 1);
        T *Vg = g.A_f + i * nn;
        const Tin *Ag = g.A_in + i * nn;
        const T *Wp = g.B_f + (i - 1) * nn;  // used when t > 0
        T *Zg = seq ? nullptr : g.Y + i * nn;
        const T *Yp = seq ? nullptr : g.Y + (i - 1) * nn;

        bool dead = false;  // TC form: a tensor-core wait expired
        if constexpr (TC) {
            if (t > 0) {
                tc_tn<T>(tcc, Wp, Wp, n, tc_stage);
                tc_store<Tin>(tcc, Vg, n, -1.f, Ag);  // V slot <- A_i - W^T W (whole block)
                if (!seq) {
                    tc_tn<T>(tcc, Wp, Yp, n, tc_stage);
                    tc_store<T>(tcc, Zg, n, -1.f, (const T *)nullptr);
                }
            } else {
                for (long long e = tid; e < nn; e += WIDE_THREADS) Vg[e] = (T)Ag[e];
            }
            dead = *tcc.abort != 0;
        } else
        // S = A_i - W_{i-1}^T W_{i-1}, upper tiles (every thread rewrites only its own elements)
        for (int I = 0; I < NT; ++I)
            for (int J = I; J < NT; ++J) {
                T acc[4][4];
                zero_tile<T, 64>(acc);
                if (t > 0) wide_tn<T, T, T>(acc, Wp, Wp, n, I, J, 0, NT - 1, sX, sY, false);
                T a[4][4];
                wload<Tin, T>(a, Ag, n, I, J, I == J, false);
#pragma unroll
                for (int x = 0; x < 4; ++x)
#pragma unroll
                    for (int y = 0; y < 4; ++y) a[x][y] -= acc[x][y];
                wstore<T>(Vg, a, n, I, J, T(1));
            }
        if (!seq) {
            if (t > 0) {
                if constexpr (!TC)
                for (int I = 0; I < NT; ++I)
                    for (int J = 0; J < NT; ++J) {
                        T acc[4][4];
                        zero_tile<T, 64>(acc);
                        wide_tn<T, T, T>(acc, Wp, Yp, n, I, J, 0, NT - 1, sX, sY, false);
                        wstore<T>(Zg, acc, n, I, J, T(-1));
                    }
            } else {
                const Tin *Bs = g.B_in + sL * nn;  // Z = B_sL^T
                for (long long e = tid; e < nn; e += WIDE_THREADS) {
                    const long long r = e % n, c = e / n;
                    Zg[e] = (T)Bs[c + r * n];
                }
            }
        }
        __syncthreads();

        // blocked Cholesky; diagonal tiles end as V_KK, off-diagonal upper tiles as U(K, J)
        for (int K = 0; K < NT; ++K) {
            {
                T a[4][4];
                wload<T, T>(a, Vg, n, K, K, true, false);
                store_tile_smem<T, 64>(sS, a, ti, tj, T(1));
            }
            __syncthreads();
            const int bad = chol_inv_blocked<T, 64, WIDE_THREADS>(sS, sV, dinv, sflag, tid);
            if (bad && tid == 0) record_bad_pivot(g.st, g.level, i);
            {
                T v[4][4];
#pragma unroll
                for (int x = 0; x < 4; ++x)
#pragma unroll
                    for (int y = 0; y < 4; ++y) v[x][y] = sV[(ti + 16 * x) + (tj + 16 * y) * LD];
                wstore<T>(Vg, v, n, K, K, T(1));
            }
            for (int J = K + 1; J < NT; ++J) {
                T r[4][4];
                wload<T, T>(r, Vg, n, K, J, false, false);
                store_tile_smem<T, 64>(sY, r, ti, tj, T(1));
                __syncthreads();
                T acc[4][4];
                zero_tile<T, 64>(acc);
                tn_acc<T, 64, TN_TRI>(acc, sV, sY, ti, tj);
                __syncthreads();
                wstore<T>(Vg, acc, n, K, J, T(1));
            }
            __syncthreads();
            for (int J1 = K + 1; J1 < NT; ++J1)
                for (int J2 = J1; J2 < NT; ++J2) {
                    T acc[4][4];
                    zero_tile<T, 64>(acc);
                    wide_tn<T, T, T>(acc, Vg, Vg, n, J1, J2, K, K, sX, sY, false);
                    T s[4][4];
                    wload<T, T>(s, Vg, n, J1, J2, false, false);
#pragma unroll
                    for (int x = 0; x < 4; ++x)
#pragma unroll
                        for (int y = 0; y < 4; ++y) s[x][y] -= acc[x][y];
                    wstore<T>(Vg, s, n, J1, J2, T(1));
                }
            __syncthreads();
        }
        // V = U^{-1}: off-diagonal tiles in place
        for (int J = NT - 1; J >= 1; --J)
            for (int I = J - 1; I >= 0; --I) {
                T acc[4][4];
                zero_tile<T, 64>(acc);
                for (int P = I + 1; P <= J; ++P) {
                    T r[4][4];
                    wload<T, T>(r, Vg, n, P, I, false, true);  // U(I, P)^T
                    store_tile_smem<T, 64>(sX, r, ti, tj, T(1));
                    wload<T, T>(r, Vg, n, P, J, false, false);  // V(P, J)
                    store_tile_smem<T, 64>(sY, r, ti, tj, T(1));
                    __syncthreads();
                    tn_acc<T, 64, TN_FULL>(acc, sX, sY, ti, tj);
                    __syncthreads();
                }
                store_tile_smem<T, 64>(sY, acc, ti, tj, T(1));
                {
                    T r[4][4];
                    wload<T, T>(r, Vg, n, I, I, false, true);  // V_II^T
                    store_tile_smem<T, 64>(sX, r, ti, tj, T(1));
                }
                __syncthreads();
                T acc2[4][4];
                zero_tile<T, 64>(acc2);
                tn_acc<T, 64, TN_FULL>(acc2, sX, sY, ti, tj);
                __syncthreads();
                wstore<T>(Vg, acc2, n, I, J, T(-1));
                __syncthreads();
            }
        for (long long e = tid; e < nn; e += WIDE_THREADS) {  // strictly lower tiles of V are zero
            const long long r = e % n, c = e / n;
            if (r / WT > c / WT) Vg[e] = T(0);
        }
        __syncthreads();

        // Y_i = V^T Z and W_i = V^T B_i in place, row tiles bottom-up
        // (TC form: the whole product lands in tensor memory first)
        if constexpr (TC) {
            if (!dead && !seq) {
                tc_tn<T>(tcc, Vg, Zg, n, tc_stage);
                tc_store<T>(tcc, Zg, n, 1.f, (const T *)nullptr);
            }
            if (!dead && has_next) {
                tc_tn<Tin>(tcc, Vg, g.B_in + i * nn, n, tc_stage);
                tc_store<T>(tcc, g.B_f + i * nn, n, 1.f, (const T *)nullptr);
            }
            if (!dead && !seq) {
                T *Cll = g.C + p * 3 * nn;
                tc_tn<T>(tcc, Zg, Zg, n, tc_stage);
                tc_store<T>(tcc, Cll, n, 1.f, t > 0 ? (const T *)Cll : (const T *)nullptr);
            }
            if (dead || *tcc.abort) {
                if (tid == 0) atomicOr(&g.st->tc_timeout, 1);
                return;
            }
            continue;
        }
        if (!seq)
            for (int I = NT - 1; I >= 0; --I)
                for (int J = 0; J < NT; ++J) {
                    T acc[4][4];
                    zero_tile<T, 64>(acc);
                    wide_tn<T, T, T>(acc, Vg, Zg, n, I, J, 0, I, sX, sY, false);
                    wstore<T>(Zg, acc, n, I, J, T(1));
                }
        if (has_next) {
            const Tin *Bi = g.B_in + i * nn;
            T *Wg = g.B_f + i * nn;
            for (int I = NT - 1; I >= 0; --I)
                for (int J = 0; J < NT; ++J) {
                    T acc[4][4];
                    zero_tile<T, 64>(acc);
                    wide_tn<T, Tin, T>(acc, Vg, Bi, n, I, J, 0, I, sX, sY, false);
                    wstore<T>(Wg, acc, n, I, J, T(1));
                }
        }
        __syncthreads();
        if (!seq) {
            T *Cll = g.C + p * 3 * nn;
            for (int I = 0; I < NT; ++I)
                for (int J = 0; J < NT; ++J) {
                    T acc[4][4];
                    zero_tile<T, 64>(acc);
                    wide_tn<T, T, T>(acc, Zg, Zg, n, I, J, 0, NT - 1, sX, sY, false);
                    if (t > 0) {
                        T c[4][4];
                        wload<T, T>(c, Cll, n, I, J, false, false);
#pragma unroll
                        for (int x = 0; x < 4; ++x)
#pragma unroll
                            for (int y = 0; y < 4; ++y) acc[x][y] += c[x][y];
                    }
                    wstore<T>(Cll, acc, n, I, J, T(1));
                }
            __syncthreads();
        }
    }

    if (!seq) {
        const T *Wl = g.B_f + last * nn;
        const T *Yl = g.Y + last * nn;
        T *Cp = g.C + p * 3 * nn;
        if constexpr (TC) {
            tc_tn<T>(tcc, Wl, Wl, n, tc_stage);
            tc_store<T>(tcc, Cp + nn, n, 1.f, (const T *)nullptr);
            tc_tn<T>(tcc, Yl, Wl, n, tc_stage);
            tc_store<T>(tcc, Cp + 2 * nn, n, 1.f, (const T *)nullptr);
            if (*tcc.abort && tid == 0) atomicOr(&g.st->tc_timeout, 1);
            return;
        }
        for (int I = 0; I < NT; ++I)
            for (int J = 0; J < NT; ++J) {
                T acc[4][4];
                zero_tile<T, 64>(acc);
                wide_tn<T, T, T>(acc, Wl, Wl, n, I, J, 0, NT - 1, sX, sY, false);
                wstore<T>(Cp + nn, acc, n, I, J, T(1));
                zero_tile<T, 64>(acc);
                wide_tn<T, T, T>(acc, Yl, Wl, n, I, J, 0, NT - 1, sX, sY, false);
                wstore<T>(Cp + 2 * nn, acc, n, I, J, T(1));
            }
    }
}

// TC form: the CTA owns a 128-column TMEM accumulator and two mbarriers for
// its lifetime (set up here, released before exit)
template <bool TC>
__device__ __forceinline__ void wide_tc_begin(TcCtx &tcc)
{
    if constexpr (TC) {
        extern __shared__ __align__(128) unsigned char smem_wide[];
        unsigned char *tail = smem_wide + TC_NSTAGE * TC_STAGE_BYTES;  // 128 bytes of control words
        tc_setup(tcc, reinterpret_cast<uint32_t *>(tail + 16), reinterpret_cast<uint64_t *>(tail), smem_wide,
                 reinterpret_cast<int *>(tail + 32));
    }
}

template <bool TC>
__device__ __forceinline__ void wide_tc_end(const TcCtx &tcc)
{
    if constexpr (TC) tc_teardown(tcc);
}

template <class Tin, class T, bool TC>
__global__ void __launch_bounds__(WIDE_THREADS, TC ? 2 : 1) wide_chain_factor_kernel(ChainFactorArgs<Tin, T> g)
{
    TcCtx tcc{};
    wide_tc_begin<TC>(tcc);
    wide_chain_factor_body<Tin, T, TC>(g, blockIdx.x, tcc);
    wide_tc_end<TC>(tcc);
}

template <class Tin, class T, bool TC>
__global__ void __launch_bounds__(WIDE_THREADS, TC ? 2 : 1)
    wide_chain_factor_queue_kernel(const ChainFactorArgs<Tin, T> *__restrict__ descs,
                                   const WorkItem *__restrict__ items, int nitems, int *head)
{
    __shared__ int cur;
    TcCtx tcc{};
    wide_tc_begin<TC>(tcc);
    for (;;) {
        if (threadIdx.x == 0) cur = atomicAdd(head, 1);
        __syncthreads();
        const int it = cur;
        __syncthreads();
        if (it >= nitems) break;
        const WorkItem w = items[it];
        const ChainFactorArgs<Tin, T> g = descs[w.desc];
        wide_chain_factor_body<Tin, T, TC>(g, w.p, tcc);
        __syncthreads();
        if constexpr (TC) {
            if (*tcc.abort) break;  // uniform: set before the body's last barrier
        }
    }
    wide_tc_end<TC>(tcc);
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
    const bool aligned16 = ((((unsigned long long)g) | (unsigned long long)__cvta_generic_to_shared(s)) & 15) == 0;
    if (aligned16 && ((count * (int)sizeof(T)) & 15) == 0) {
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

// out(c, j) (+)= sign * sum_r M(r, c) v(r, j); M n x n (ld n), v/out n x kc (ld n).
// A warp owns 4 output columns at a time; the four shuffle reductions are
// interleaved so their latencies overlap.
template <class T>
__device__ __forceinline__ void cta_tmul(const T *sM, const T *v, T *out, int n, int kc, T sign, bool accumulate)
{
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
    for (int c0 = 4 * warp; c0 < n; c0 += 4 * nw) {
        for (int j = 0; j < kc; ++j) {
            T s[4] = {T(0), T(0), T(0), T(0)};
            for (int r = lane; r < n; r += 32) {
                const T vr = v[r + j * n];
#pragma unroll
                for (int q = 0; q < 4; ++q)
                    if (c0 + q < n) s[q] = fma(sM[r + (c0 + q) * n], vr, s[q]);
            }
#pragma unroll
            for (int o = 16; o > 0; o >>= 1)
#pragma unroll
                for (int q = 0; q < 4; ++q) s[q] += __shfl_xor_sync(0xffffffffu, s[q], o);
            if (lane < 4 && c0 + lane < n) {
                T val = s[0];
#pragma unroll
                for (int q = 1; q < 4; ++q)
                    if (lane == q) val = s[q];
                const int o = c0 + lane + j * n;
                out[o] = accumulate ? out[o] + sign * val : sign * val;
            }
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

// Forms of the two products for blocks read straight from global memory
// (the unstaged solve): the loads of a thread are independent and issued
// together before their FMAs (so a warp waits for memory once per batch of
// loads, not once per element), and every matrix element is used for all
// right-hand-side columns of the pass.
//
// out(c, j) (+)= sign * sum_r M(r, c) v(r, j): a warp takes 4 columns; each
// lane holds 4 rows x 4 columns of M (16 loads in flight) per 128-row slab.
template <class T>
__device__ __forceinline__ void cta_tmul_g(const T *M, const T *v, T *out, int n, int kc, T sign, bool accumulate)
{
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
    for (int c0 = 4 * warp; c0 < n; c0 += 4 * nw) {
        for (int j0 = 0; j0 < kc; j0 += 4) {
            T s[4][4];
#pragma unroll
            for (int q = 0; q < 4; ++q)
#pragma unroll
                for (int jj = 0; jj < 4; ++jj) s[q][jj] = T(0);
            for (int rb = 0; rb < n; rb += 128) {
                T m[4][4];
#pragma unroll
                for (int t = 0; t < 4; ++t) {
                    const int r = rb + lane + 32 * t;
#pragma unroll
                    for (int q = 0; q < 4; ++q)
                        m[t][q] = (r < n && c0 + q < n) ? M[r + (size_t)(c0 + q) * n] : T(0);
                }
#pragma unroll
                for (int jj = 0; jj < 4; ++jj) {
                    if (j0 + jj >= kc) break;
#pragma unroll
                    for (int t = 0; t < 4; ++t) {
                        if (rb + 32 * t >= n) break;  // warp-uniform: no FMAs on padding rows
                        const int r = rb + lane + 32 * t;
                        const T vr = r < n ? v[r + (j0 + jj) * n] : T(0);
#pragma unroll
                        for (int q = 0; q < 4; ++q) s[q][jj] = fma(m[t][q], vr, s[q][jj]);
                    }
                }
            }
#pragma unroll
            for (int o = 16; o > 0; o >>= 1)
#pragma unroll
                for (int q = 0; q < 4; ++q)
#pragma unroll
                    for (int jj = 0; jj < 4; ++jj) s[q][jj] += __shfl_xor_sync(0xffffffffu, s[q][jj], o);
            if (lane < 16) {
                const int q = lane >> 2, jj = lane & 3;
                T val = T(0);
#pragma unroll
                for (int a = 0; a < 4; ++a)
#pragma unroll
                    for (int b = 0; b < 4; ++b)
                        if (a == q && b == jj) val = s[a][b];
                if (c0 + q < n && j0 + jj < kc) {
                    const int o = c0 + q + (j0 + jj) * n;
                    out[o] = accumulate ? out[o] + sign * val : sign * val;
                }
            }
        }
    }
}

// out(r, j) = base(r, j) + sign * (sum_c M1(r, c) v1(c, j) [+ sum_c M2(r, c) v2(c, j)]):
// a thread owns one row and up to 8 columns of the pass; blocks of 16
// columns of M are loaded together.  With fewer rows than threads the
// contraction is split over `parts` thread groups reduced through `red`
// (parts x 8 x n elements).  Ends with a barrier.
template <class T>
__device__ __forceinline__ void cta_nmul_g(const T *M1, const T *v1, const T *M2, const T *v2, const T *base, T *out,
                                           T sign, int n, int kc, T *red)
{
    int parts = (int)blockDim.x / n;
    parts = parts < 1 ? 1 : (parts > 8 ? 8 : parts);
    for (int j0 = 0; j0 < kc; j0 += 8) {
        const int jn = kc - j0 < 8 ? kc - j0 : 8;
        for (int w = threadIdx.x; w < parts * n; w += blockDim.x) {
            const int part = w / n, r = w - part * n;
            const int c0 = (part * n) / parts, c1 = ((part + 1) * n) / parts;
            T acc[8];
#pragma unroll
            for (int jj = 0; jj < 8; ++jj) acc[jj] = T(0);
            for (int mi = 0; mi < 2; ++mi) {
                const T *M = mi == 0 ? M1 : M2;
                const T *v = mi == 0 ? v1 : v2;
                if (!M) continue;
                for (int c = c0; c < c1; c += 16) {
                    T m[16];
#pragma unroll
                    for (int u = 0; u < 16; ++u) m[u] = (c + u < c1) ? M[r + (size_t)(c + u) * n] : T(0);
#pragma unroll
                    for (int u = 0; u < 16; ++u) {
                        if (c + u >= c1) break;
#pragma unroll
                        for (int jj = 0; jj < 8; ++jj)
                            if (jj < jn) acc[jj] = fma(m[u], v[(c + u) + (j0 + jj) * n], acc[jj]);
                    }
                }
            }
            if (parts == 1) {
#pragma unroll
                for (int jj = 0; jj < 8; ++jj)
                    if (jj < jn) {
                        const int o = r + (j0 + jj) * n;
                        out[o] = (base ? base[o] : T(0)) + sign * acc[jj];
                    }
            } else {
#pragma unroll
                for (int jj = 0; jj < 8; ++jj)
                    if (jj < jn) red[(part * 8 + jj) * n + r] = acc[jj];
            }
        }
        __syncthreads();
        if (parts > 1) {
            for (int o = threadIdx.x; o < n * jn; o += blockDim.x) {
                const int jj = o / n, r = o - jj * n;
                T sum = T(0);
                for (int q = 0; q < parts; ++q) sum += red[(q * 8 + jj) * n + r];
                const int oo = r + (j0 + jj) * n;
                out[oo] = (base ? base[oo] : T(0)) + sign * sum;
            }
            __syncthreads();
        }
    }
}

// Forms for a block staged in shared memory (leading dimension n, a multiple
// of the vector width W: 4 floats or 2 doubles, 16 bytes) and several
// right-hand-side columns: every thread owns whole outputs, so no cross-lane
// reduction is needed, and walks the contraction in 16-byte steps; the lanes
// of a shared-memory wavefront start their walks at different offsets
// (W (lane % 8) mod n) so that they hit distinct banks.
//
// out(c, j) (+)= sign * sum_r M(r, c) v(r, j): thread = (column c, the
// right-hand sides jg, jg + tpc, ... with tpc = threads / n).
template <class T>
__device__ __forceinline__ void cta_tmul_s(const T *sM, const T *v, T *out, int n, int kc, T sign, bool accumulate)
{
    using VT = typename Vec<T>::type;
    constexpr int W = Vec<T>::W;
    const int tpc = (int)blockDim.x / n;
    const int c = threadIdx.x % n, jg = threadIdx.x / n;
    if (jg >= tpc) return;
    const int rot = (W * (threadIdx.x & 7)) % n;
    const T *mc = sM + (size_t)c * n;
    for (int j0 = jg; j0 < kc; j0 += 4 * tpc) {
        T acc[4] = {T(0), T(0), T(0), T(0)};
        for (int r4 = 0; r4 < n; r4 += W) {
            int r = r4 + rot;
            if (r >= n) r -= n;
            const VT m = *reinterpret_cast<const VT *>(mc + r);
#pragma unroll
            for (int q = 0; q < 4; ++q) {
                const int j = j0 + tpc * q;
                if (j < kc) fma_vec(acc[q], m, *reinterpret_cast<const VT *>(v + r + (size_t)j * n));
            }
        }
#pragma unroll
        for (int q = 0; q < 4; ++q) {
            const int j = j0 + tpc * q;
            if (j < kc) {
                const int o = c + j * n;
                out[o] = accumulate ? out[o] + sign * acc[q] : sign * acc[q];
            }
        }
    }
}

// out(r, j) = base(r, j) + sign * (sum_c M1(r, c) v1(c, j) [+ sum_c M2(r, c)
// v2(c, j)]) (base may be null, may be out): thread = (row r, right-hand sides
// jg, jg + tpc, ...); M read along rows (lanes on consecutive rows), v as
// 16-byte broadcasts.  No barrier.
template <class T>
__device__ __forceinline__ void cta_nmul_s(const T *M1, const T *v1, const T *M2, const T *v2, const T *base,
                                           T *out, T sign, int n, int kc)
{
    using VT = typename Vec<T>::type;
    constexpr int W = Vec<T>::W;
    const int tpc = (int)blockDim.x / n;
    const int r = threadIdx.x % n, jg = threadIdx.x / n;
    if (jg >= tpc) return;
    for (int j0 = jg; j0 < kc; j0 += 4 * tpc) {
        T acc[4] = {T(0), T(0), T(0), T(0)};
        for (int mi = 0; mi < 2; ++mi) {
            const T *M = mi == 0 ? M1 : M2;
            const T *v = mi == 0 ? v1 : v2;
            if (!M) continue;
            for (int c = 0; c < n; c += W) {
                T mrow[W];
#pragma unroll
                for (int w = 0; w < W; ++w) mrow[w] = M[r + (size_t)(c + w) * n];
#pragma unroll
                for (int q = 0; q < 4; ++q) {
                    const int j = j0 + tpc * q;
                    if (j < kc) {
                        const VT x = *reinterpret_cast<const VT *>(v + c + (size_t)j * n);
                        const T *xs = reinterpret_cast<const T *>(&x);
#pragma unroll
                        for (int w = 0; w < W; ++w) acc[q] = fma(mrow[w], xs[w], acc[q]);
                    }
                }
            }
        }
#pragma unroll
        for (int q = 0; q < 4; ++q) {
            const int j = j0 + tpc * q;
            if (j < kc) {
                const int o = r + j * n;
                out[o] = (base ? base[o] : T(0)) + sign * acc[q];
            }
        }
    }
}

// Staged blocks: the transpose product takes the register-blocked form when
// there are several right-hand-side columns (every matrix element reused
// across them; lanes run along rows, conflict-free on shared memory, no
// scratch), the one-column form otherwise; the normal product keeps its
// staged form.  Blocks read from global memory take the register-blocked
// forms.
template <bool STAGED, class T>
__device__ __forceinline__ void tmul(const T *M, const T *v, T *out, int n, int kc, T sign, bool accumulate)
{
    if constexpr (STAGED) {
        if (kc > 1 && n % Vec<T>::W == 0 && n <= (int)blockDim.x) {
            cta_tmul_s<T>(M, v, out, n, kc, sign, accumulate);
            return;
        }
    }
    if (STAGED && kc == 1)
        cta_tmul<T>(M, v, out, n, kc, sign, accumulate);
    else
        cta_tmul_g<T>(M, v, out, n, kc, sign, accumulate);
}

// the staged multi-column form when there are more outputs than threads (else
// the split contraction of cta_nmul keeps every thread busy)
template <bool STAGED, class T>
__device__ __forceinline__ void nmul(const T *M1, const T *v1, const T *M2, const T *v2, const T *base, T *out,
                                     T sign, int n, int kc, T *red)
{
    if constexpr (STAGED) {
        if (kc > 1 && n % Vec<T>::W == 0 && n * kc > (int)blockDim.x) {
            cta_nmul_s<T>(M1, v1, M2, v2, base, out, sign, n, kc);
            return;
        }
        cta_nmul<T>(M1, v1, M2, v2, base, out, sign, n, kc, red);
    } else {
        cta_nmul_g<T>(M1, v1, M2, v2, base, out, sign, n, kc, red);
    }
}

// Hint a block the CTA will read in its next step into L2: one prefetch per
// 128-byte line, spread over the CTA's threads (no registers, no shared
// memory; the addresses are those of the block itself).
__device__ __forceinline__ void prefetch_l2(const void *p, size_t bytes)
{
    const char *c = static_cast<const char *>(p);
    for (size_t o = (size_t)threadIdx.x * 128; o < bytes; o += (size_t)blockDim.x * 128)
        asm volatile("prefetch.global.L2 [%0];" ::"l"(c + o));
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
    DevStatus *st; // a bounded wait of the streamed sweeps records its expiry here
};

// shared memory: 2 buffers x 3 blocks (staged form only) + 6 vectors +
// reduction scratch.  Blocks too large to stage (n > 64 in FP64, n > 90 in
// FP32) are read straight from global memory, once per step, coalesced.
constexpr size_t SOLVE_SMEM_MAX = 220 * 1024;

template <class T>
__host__ __device__ constexpr int solve_red_elems(int n, int kc, bool staged)
{
    // the staged normal product reduces n*kc partials (or one per thread);
    // the register-blocked one up to 8 parts x 8 columns x n
    return staged ? (n * kc > SOLVE_THREADS ? n * kc : SOLVE_THREADS)
                               : (SOLVE_THREADS / n >= 2 ? (SOLVE_THREADS / n > 8 ? 8 : SOLVE_THREADS / n) * 8 * n : 0) +
                                     SOLVE_THREADS;
}

template <class T>
__host__ __device__ constexpr size_t solve_smem_bytes(int n, int kc, bool staged = true)
{
    return (size_t)((staged ? 6 * n * n : 0) + 6 * n * kc + solve_red_elems<T>(n, kc, staged)) * sizeof(T);
}

// the staged form whenever its double buffer fits for this column chunk
template <class T>
__host__ __device__ constexpr bool solve_staged(int n, int kc)
{
    return solve_smem_bytes<T>(n, kc, true) <= SOLVE_SMEM_MAX;
}

template <class T>
__device__ __forceinline__ const T *rhs_ptr(const T *g, long long blk, int n, int k, int j0)
{
    return g + blk * (long long)n * k + (long long)j0 * n;
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
template <class T, bool STAGED>
__device__ __forceinline__ void chain_fwd_body(const SolveArgs<T> &g, const long long p)
{
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int n = g.n, kc = g.kc;
    const int nn = n * n, nkc = n * kc;
    T *buf = reinterpret_cast<T *>(smem_raw);  // [2][3][nn]: V, W, Y (STAGED only)
    T *srb = buf + (STAGED ? 6 * nn : 0);      // [2][nkc]: RHS block of the step (prefetched)
    T *sy = srb + 2 * nkc;
    T *sbL = sy + nkc;
    T *sbR = sbL + nkc;
    T *sx = sbR + nkc;
    T *red = sx + nkc;
    const bool seq = g.seq != 0;
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
    for (int e = threadIdx.x; e < nkc; e += blockDim.x) sbL[e] = T(0);
    // step i uses V_i (slot 0), W_{i-1} (slot 1), Y_{i-1} (slot 2) and d_i in buffer
    // (i - first) & 1: the products with W_{i-1} (into this step's RHS) and Y_{i-1}
    // (into bL) both read y_{i-1}, so they share the step's first phase, and y_{i-1}
    // is stored there too; the step's second phase is y_i = V_i^T r_i
    if (STAGED) async_copy(buf, g.Af + first * (long long)nn, nn);
    async_copy(srb, rhs_ptr<T>(g.d, first, n, g.k, g.j0), nkc);
    cp_async_commit();
    for (long long i = first; i <= last; ++i) {
        const int cb = (int)((i - first) & 1);
        T *cur = buf + cb * 3 * nn;
        T *nxt = buf + (cb ^ 1) * 3 * nn;
        T *sr = srb + cb * nkc;
        cp_async_wait_all();
        __syncthreads();
        // prefetch step i+1: V_{i+1} and d_{i+1}, and W_i, Y_i for its first phase
        // (after the last step, W_last and Y_last for bR and the last bL term)
        if (i < last) {
            if (STAGED) async_copy(nxt, g.Af + (i + 1) * (long long)nn, nn);
            async_copy(srb + (cb ^ 1) * nkc, rhs_ptr<T>(g.d, i + 1, n, g.k, g.j0), nkc);
        }
        if (STAGED && (!seq || i < last)) async_copy(nxt + nn, g.Bf + i * (long long)nn, nn);
        if (STAGED && !seq) async_copy(nxt + 2 * nn, g.Y + i * (long long)nn, nn);
        cp_async_commit();
        // matrices of step i: staged in shared memory, or read straight from global
        // memory (then the next step's are hinted into L2 while this one runs)
        if (!STAGED && i < last) {
            prefetch_l2(g.Af + (i + 1) * (long long)nn, (size_t)nn * sizeof(T));
            prefetch_l2(g.Bf + i * (long long)nn, (size_t)nn * sizeof(T));
            if (!seq) prefetch_l2(g.Y + i * (long long)nn, (size_t)nn * sizeof(T));
        }
        const T *mV = STAGED ? cur : g.Af + i * (long long)nn;
        if (i > first) {
            const T *mW = STAGED ? cur + nn : g.Bf + (i - 1) * (long long)nn;
            const T *mY = STAGED ? cur + 2 * nn : g.Y + (i - 1) * (long long)nn;
            store_rhs(g.d, sy, i - 1, n, g.k, g.j0, kc);
            tmul<STAGED>(mW, sy, sr, n, kc, T(-1), true);
            if (!seq) tmul<STAGED>(mY, sy, sbL, n, kc, T(1), true);
            __syncthreads();
        }
        tmul<STAGED>(mV, sr, sy, n, kc, T(1), false);
    }
    cp_async_wait_all();
    __syncthreads();
    store_rhs(g.d, sy, last, n, g.k, g.j0, kc);
    if (!seq) {
        // bL += Y_last^T y_last, bR = W_last^T y_last (both prefetched in the last step)
        const T *nb = buf + ((last + 1 - first) & 1) * 3 * nn;
        const T *wl = STAGED ? nb + nn : g.Bf + last * (long long)nn;
        const T *yl = STAGED ? nb + 2 * nn : g.Y + last * (long long)nn;
        tmul<STAGED>(yl, sy, sbL, n, kc, T(1), true);
        tmul<STAGED>(wl, sy, sbR, n, kc, T(1), false);
        __syncthreads();
        T *bp = g.bvec + p * 2 * (long long)nkc;
        for (int e = threadIdx.x; e < nkc; e += blockDim.x) {
            bp[e] = sbL[e];
            bp[nkc + e] = sbR[e];
        }
        return;
    }
    __syncthreads();  // every y_i is stored before the backward sweep reads them back
    // sequential level, backward: x_i = V_i (y_i - W_i x_{i+1}); step i uses
    // V_i (slot 0), W_i (slot 1) and y_i
    if (STAGED) async_copy(buf, g.Af + last * (long long)nn, nn);
    async_copy(srb, rhs_ptr<T>(g.d, last, n, g.k, g.j0), nkc);
    cp_async_commit();
    for (long long i = last; i >= first; --i) {
        const int cb = (int)((last - i) & 1);
        T *cur = buf + cb * 3 * nn;
        T *nxt = buf + (cb ^ 1) * 3 * nn;
        T *sr = srb + cb * nkc;
        cp_async_wait_all();
        __syncthreads();
        if (i > first) {
            if (STAGED) {
                async_copy(nxt, g.Af + (i - 1) * (long long)nn, nn);
                async_copy(nxt + nn, g.Bf + (i - 1) * (long long)nn, nn);
            }
            async_copy(srb + (cb ^ 1) * nkc, rhs_ptr<T>(g.d, i - 1, n, g.k, g.j0), nkc);
        }
        cp_async_commit();
        if (!STAGED && i > first) {
            prefetch_l2(g.Af + (i - 1) * (long long)nn, (size_t)nn * sizeof(T));
            prefetch_l2(g.Bf + (i - 1) * (long long)nn, (size_t)nn * sizeof(T));
        }
        const T *mV = STAGED ? cur : g.Af + i * (long long)nn;
        const T *mW = STAGED ? cur + nn : g.Bf + i * (long long)nn;
        if (i < last) {
            nmul<STAGED, T>(mW, sx, nullptr, nullptr, sr, sr, T(-1), n, kc, red);
            __syncthreads();
        }
        nmul<STAGED, T>(mV, sr, nullptr, nullptr, nullptr, sx, T(1), n, kc, red);
        __syncthreads();
        store_rhs(g.d, sx, i, n, g.k, g.j0, kc);
    }
    cp_async_wait_all();
}

template <class T, bool STAGED>
__global__ void __launch_bounds__(SOLVE_THREADS, 2) chain_fwd_kernel(SolveArgs<T> g)
{
    chain_fwd_body<T, STAGED>(g, blockIdx.x);
}

template <class T, bool STAGED>
__global__ void __launch_bounds__(SOLVE_THREADS, 2)
    chain_fwd_queue_kernel(const SolveArgs<T> *__restrict__ descs, const WorkItem *__restrict__ items, int nitems,
                           int *head)
{
    __shared__ int cur;
    for (;;) {
        if (threadIdx.x == 0) cur = atomicAdd(head, 1);
        __syncthreads();
        const int it = cur;
        __syncthreads();
        if (it >= nitems) break;
        const WorkItem w = items[it];
        const SolveArgs<T> g = descs[w.desc];
        chain_fwd_body<T, STAGED>(g, w.p);
        __syncthreads();
    }
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
template <class T, class Tsep, bool STAGED>
__device__ __forceinline__ void chain_bwd_body(const SolveArgs<T> &g, const long long p)
{
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int n = g.n, kc = g.kc;
    const int nn = n * n;
    const int nkc = n * kc;
    T *buf = reinterpret_cast<T *>(smem_raw);  // [2][3][nn]: V_i, W_i, Y_i (STAGED only)
    T *szb = buf + (STAGED ? 6 * nn : 0);      // [2][nkc]: y_i of the step (prefetched)
    T *sxL = szb + 2 * nkc;
    T *sxn = sxL + nkc;
    T *sxt = sxn + nkc;
    T *red = sxt + nkc;
    const long long sL = (p * (g.N - 1)) / g.Q;
    const long long sR = ((p + 1) * (g.N - 1)) / g.Q;
    const long long first = sL + 1, last = sR - 1;
    const Tsep *xs = reinterpret_cast<const Tsep *>(g.xsep);
    if (STAGED) {
        async_copy(buf, g.Af + last * (long long)nn, nn);
        async_copy(buf + nn, g.Bf + last * (long long)nn, nn);
        async_copy(buf + 2 * nn, g.Y + last * (long long)nn, nn);
    }
    async_copy(szb, rhs_ptr<T>(g.d, last, n, g.k, g.j0), nkc);
    cp_async_commit();
    load_rhs(sxL, xs, p, n, g.k, g.j0, kc);
    load_rhs(sxn, xs, p + 1, n, g.k, g.j0, kc);
    __syncthreads();
    store_rhs(g.d, sxL, sL, n, g.k, g.j0, kc);
    if (p == g.Q - 1) store_rhs(g.d, sxn, sR, n, g.k, g.j0, kc);
    for (long long i = last; i >= first; --i) {
        const int cb = (int)((last - i) & 1);
        T *cur = buf + cb * 3 * nn;
        T *nxt = buf + (cb ^ 1) * 3 * nn;
        T *sz = szb + cb * nkc;
        cp_async_wait_all();
        __syncthreads();
        if (i > first) {
            if (STAGED) {
                async_copy(nxt, g.Af + (i - 1) * (long long)nn, nn);
                async_copy(nxt + nn, g.Bf + (i - 1) * (long long)nn, nn);
                async_copy(nxt + 2 * nn, g.Y + (i - 1) * (long long)nn, nn);
            }
            async_copy(szb + (cb ^ 1) * nkc, rhs_ptr<T>(g.d, i - 1, n, g.k, g.j0), nkc);
        }
        cp_async_commit();
        if (!STAGED && i > first) {
            prefetch_l2(g.Af + (i - 1) * (long long)nn, (size_t)nn * sizeof(T));
            prefetch_l2(g.Bf + (i - 1) * (long long)nn, (size_t)nn * sizeof(T));
            prefetch_l2(g.Y + (i - 1) * (long long)nn, (size_t)nn * sizeof(T));
        }
        const T *mV = STAGED ? cur : g.Af + i * (long long)nn;
        const T *mW = STAGED ? cur + nn : g.Bf + i * (long long)nn;
        const T *mY = STAGED ? cur + 2 * nn : g.Y + i * (long long)nn;
        nmul<STAGED, T>(mY, sxL, mW, sxn, sz, sz, T(-1), n, kc, red);
        __syncthreads();
        nmul<STAGED, T>(mV, sz, nullptr, nullptr, nullptr, sxt, T(1), n, kc, red);
        __syncthreads();
        for (int e = threadIdx.x; e < n * kc; e += blockDim.x) sxn[e] = sxt[e];
        store_rhs(g.d, sxt, i, n, g.k, g.j0, kc);
        __syncthreads();
    }
    cp_async_wait_all();
}

template <class T, class Tsep, bool STAGED>
__global__ void __launch_bounds__(SOLVE_THREADS) chain_bwd_kernel(SolveArgs<T> g)
{
    chain_bwd_body<T, Tsep, STAGED>(g, blockIdx.x);
}

template <class T, class Tsep, bool STAGED>
__global__ void __launch_bounds__(SOLVE_THREADS)
    chain_bwd_queue_kernel(const SolveArgs<T> *__restrict__ descs, const WorkItem *__restrict__ items, int nitems,
                           int *head)
{
    __shared__ int cur;
    for (;;) {
        if (threadIdx.x == 0) cur = atomicAdd(head, 1);
        __syncthreads();
        const int it = cur;
        __syncthreads();
        if (it >= nitems) break;
        const WorkItem w = items[it];
        const SolveArgs<T> g = descs[w.desc];
        chain_bwd_body<T, Tsep, STAGED>(g, w.p);
        __syncthreads();
    }
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

// r = d - T x in FP64 over the block-tridiagonal operator.  The FP64 FMA
// pipe (~2 per clock per SM on GB300) bounds this kernel, not HBM, so it is
// shaped to keep that pipe fed: several small CTAs per SM, each owning a
// contiguous range of blocks.  For block i a thread (row r, column part p)
// reads A_i(r, c) and B_i(r, c) straight from global memory (coalesced along
// r) for t_i = A_i x_i + B_i x_{i+1}, and drops B_i into shared memory
// (ld n+1) for u_{i+1} = B_i^T x_i, the next block's sub-diagonal term; every
// A and B block is read from HBM once.  Writes r (as Tr; may be null) and
// folds max|r|, max|x| -- and, when with_norm, the row sums of |T|
// (||T||_inf) -- into the status.  Columns j0 .. j0+k-1 per launch.
constexpr int RES_THREADS = 256;

template <class T>
__host__ __device__ constexpr size_t residual_smem_bytes(int n, int k)
{
    // sB (n(n+1)), x ring [3][nk], u ping-pong [2][nk], partials [2][parts<=8][nk],
    // norm partials [3][8][n] and the carried |B^T| row sums [2][n]
    return (size_t)(n * (n + 1) + 3 * n * k + 2 * n * k + 16 * n * k + 26 * n) * sizeof(double);
}

// |x| of an FP64 value as an approximate FP32 (truncated mantissa, 2^-20
// relative), using integer operations only: on GB300 every warp-instruction
// on the FP64 pipe costs ~16 cycles, which the operator-norm sums must not add
__device__ __forceinline__ float abs_f32_approx(double v)
{
    const unsigned long long b = (unsigned long long)__double_as_longlong(v);
    const int e = (int)((b >> 52) & 0x7FF) - 1023 + 127;
    if (e <= 0) return 0.0f;
    if (e >= 255) return __int_as_float(0x7F800000);
    return __int_as_float((e << 23) | (int)((b >> 29) & 0x7FFFFF));
}
__device__ __forceinline__ float abs_f32_approx(float v) { return fabsf(v); }

// one pass of RHS columns jb .. jb+KB-1 over this thread's column range
template <int KB, class T>
__device__ __forceinline__ void residual_rows(const T *__restrict__ Ag, const T *__restrict__ Bg, bool has_b, int c0,
                                              int c1, int n, int LDp, const double *x0, const double *x1, double *sB,
                                              bool stage_b, double *out, int stride)
{
    double acc[KB];
#pragma unroll
    for (int q = 0; q < KB; ++q) acc[q] = 0.0;
    if (has_b) {
#pragma unroll 4
        for (int c = c0; c < c1; ++c) {
            const double a = (double)Ag[(long long)c * n];
            const double b = (double)Bg[(long long)c * n];
            if (stage_b) sB[c * LDp] = b;
#pragma unroll
            for (int q = 0; q < KB; ++q) acc[q] = fma(a, x0[c + q * n], fma(b, x1[c + q * n], acc[q]));
        }
    } else {
#pragma unroll 4
        for (int c = c0; c < c1; ++c) {
            const double a = (double)Ag[(long long)c * n];
#pragma unroll
            for (int q = 0; q < KB; ++q) acc[q] = fma(a, x0[c + q * n], acc[q]);
        }
    }
#pragma unroll
    for (int q = 0; q < KB; ++q) out[q * stride] = acc[q];
}

template <class T, class Tr>
__device__ __forceinline__ void residual_body(const T *__restrict__ A, const T *__restrict__ B,
                                              const T *__restrict__ x, const T *__restrict__ d, Tr *__restrict__ r,
                                              long long N, int n, int ktot, int j0, int k, long long b0_, long long b1_,
                                              int with_norm, DevStatus *st)
{
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int LDp = n + 1;
    const int nk = n * k;
    const long long bstride = (long long)n * ktot, coff = (long long)j0 * n;
    double *sB = reinterpret_cast<double *>(smem_raw);
    double *sxr = sB + n * LDp;     // [3][nk]
    double *sub = sxr + 3 * nk;     // [2][nk] u_i ping-pong
    double *red = sub + 2 * nk;     // [2][8][nk]
    double *rowred = red + 16 * nk; // [3][8][n]
    double *rowu = rowred + 24 * n; // [2][n]
    int parts = RES_THREADS / n;
    parts = parts < 1 ? 1 : (parts > 8 ? 8 : parts);
    const int tid = threadIdx.x;
    const int row = tid % n, part = tid / n;
    const bool active = part < parts;
    const int c0 = active ? (part * n) / parts : 0, c1 = active ? ((part + 1) * n) / parts : 0;
    const long long nn = (long long)n * n;
    const long long b0 = b0_;
    const long long b1 = b1_ < N ? b1_ : N;
    if (b0 >= N) return;
    if (with_norm < 0) with_norm = st->need_anorm;  // graph mode: decided on the device
    double rmax = 0.0, xmax = 0.0, amax = 0.0;
    auto xs = [&](long long blk) { return sxr + (int)((blk - b0 + 3) % 3) * nk; };  // blk in [b0-1, b1]

    // prologue: x_{b0-1}, x_{b0}, x_{b0+1}; u_{b0} = B_{b0-1}^T x_{b0-1}
    for (int e = tid; e < nk; e += blockDim.x) {
        xs(b0)[e] = (double)x[b0 * bstride + coff + e];
        if (b0 + 1 < N) xs(b0 + 1)[e] = (double)x[(b0 + 1) * bstride + coff + e];
        sub[e] = 0.0;
    }
    for (int e = tid; e < n; e += blockDim.x) rowu[e] = 0.0;
    if (b0 > 0) {
        double *xm = xs(b0 - 1);
        for (int e = tid; e < nk; e += blockDim.x) xm[e] = (double)x[(b0 - 1) * bstride + coff + e];
        for (int e = tid; e < (int)nn; e += blockDim.x) {
            const int c = e / n, rr = e - c * n;
            sB[rr + c * LDp] = (double)B[(b0 - 1) * nn + e];
        }
        __syncthreads();
        for (int o = tid; o < nk; o += blockDim.x) {
            const int j = o / n, rr = o - j * n;
            double s = 0.0;
            for (int c = 0; c < n; ++c) s = fma(sB[c + rr * LDp], xm[c + j * n], s);
            sub[o] = s;
        }
        if (with_norm)
            for (int rr = tid; rr < n; rr += blockDim.x) {
                double s = 0.0;
                for (int c = 0; c < n; ++c) s += fabs(sB[c + rr * LDp]);
                rowu[rr] = s;
            }
    }
    __syncthreads();

    for (long long i = b0; i < b1; ++i) {
        const int par = (int)((i - b0) & 1);
        const bool has_b = i + 1 < N;
        const double *x0 = xs(i);
        const double *x1 = xs(i + 1);
        double *su = sub + par * nk;        // u_i
        double *sun = sub + (par ^ 1) * nk;  // u_{i+1}
        double *rw = rowu + par * 0;         // carried row sums (same slot, owner-updated)
        // phase 1: t partials from global A_i, B_i; B_i into shared memory
        if (active) {
            const T *Ag = A + i * nn + row;
            const T *Bg = B + i * nn + row;
            // right-hand sides in compile-time groups (4, then 1): no predicated FP64 FMAs
            int jb = 0;
            for (; jb + 4 <= k; jb += 4)
                residual_rows<4, T>(Ag, Bg, has_b, c0, c1, n, LDp, x0 + jb * n, x1 + jb * n, sB + row, jb == 0,
                                    red + (part * k + jb) * n + row, n);
            for (; jb < k; ++jb)
                residual_rows<1, T>(Ag, Bg, has_b, c0, c1, n, LDp, x0 + jb * n, x1 + jb * n, sB + row, jb == 0,
                                    red + (part * k + jb) * n + row, n);
            if (!has_b)
                for (int c = c0; c < c1; ++c) sB[row + c * LDp] = 0.0;
            if (with_norm) {
                float sa = 0.0f;
                for (int c = c0; c < c1; ++c)
                    sa += abs_f32_approx(Ag[(long long)c * n]) + (has_b ? abs_f32_approx(Bg[(long long)c * n]) : 0.0f);
                rowred[part * n + row] = sa;
            }
        }
        __syncthreads();
        // phase 2: u_{i+1} partials from the staged B_i
        if (active && has_b) {
            for (int j = 0; j < k; ++j) {
                double u = 0.0;
                for (int c = c0; c < c1; ++c) u = fma(sB[c + row * LDp], x0[c + j * n], u);
                red[8 * nk + (part * k + j) * n + row] = u;
            }
            if (with_norm) {
                float sbt = 0.0f;
                for (int c = c0; c < c1; ++c) sbt += abs_f32_approx(sB[c + row * LDp]);
                rowred[16 * n + part * n + row] = sbt;
            }
        }
        __syncthreads();
        // phase 3: outputs; fetch x_{i+2}
        for (int o = tid; o < nk; o += blockDim.x) {
            const int j = o / n, rr = o - j * n;
            double t = 0.0, u = 0.0;
            for (int q = 0; q < parts; ++q) t += red[(q * k + j) * n + rr];
            if (has_b)
                for (int q = 0; q < parts; ++q) u += red[8 * nk + (q * k + j) * n + rr];
            const double res = (double)d[i * bstride + coff + o] - t - su[o];
            if (r) r[i * bstride + coff + o] = (Tr)res;
            rmax = fmax(rmax, fabs(res));
            xmax = fmax(xmax, fabs(x0[o]));
            sun[o] = u;
        }
        if (with_norm)
            for (int rr = tid; rr < n; rr += blockDim.x) {
                double s = rw[rr], s2 = 0.0;
                for (int q = 0; q < parts; ++q) {
                    s += rowred[q * n + rr];
                    if (has_b) s2 += rowred[16 * n + q * n + rr];
                }
                amax = fmax(amax, s);
                rw[rr] = has_b ? s2 : 0.0;
            }
        if (i + 2 < N && i + 1 < b1) {
            double *x2 = xs(i + 2);
            for (int e = tid; e < nk; e += blockDim.x) x2[e] = (double)x[(i + 2) * bstride + coff + e];
        }
        __syncthreads();
    }
    for (int o = 16; o > 0; o >>= 1) {
        rmax = fmax(rmax, __shfl_xor_sync(0xffffffffu, rmax, o));
        xmax = fmax(xmax, __shfl_xor_sync(0xffffffffu, xmax, o));
        amax = fmax(amax, __shfl_xor_sync(0xffffffffu, amax, o));
    }
    if ((threadIdx.x & 31) == 0) {
        atomic_max_nonneg(&st->rnorm, rmax);
        atomic_max_nonneg(&st->xnorm, xmax);
        if (with_norm) atomic_max_nonneg(&st->anorm, amax);
    }
}

template <class T, class Tr>
__global__ void __launch_bounds__(RES_THREADS, 3) residual_kernel(const T *__restrict__ A, const T *__restrict__ B,
                                                               const T *__restrict__ x, const T *__restrict__ d,
                                                               Tr *__restrict__ r, long long N, int n, int ktot,
                                                               int j0, int k, long long per_cta, int with_norm,
                                                               DevStatus *st)
{
    const long long b0 = (long long)blockIdx.x * per_cta;
    residual_body<T, Tr>(A, B, x, d, r, N, n, ktot, j0, k, b0, b0 + per_cta, with_norm, st);
}

// ---------------------------------------------------------------------------
// Refinement residual on the FP32 pipe ("double-float"): r = d - T x for FP64
// A, B, x, d without FP64 instructions in the inner loops.  On GB300 the FP64
// pipe retires ~2 FMA/clk/SM, which bounds the FP64 residual at 3 n^2 FMAs per
// block (0.32 ms at N = 16384, n = 64) against 0.16 ms to stream A and B from
// HBM; here every product runs on the 128-lane FP32 pipe.
//
// Representation: an FP64 value a becomes (a_hi, a_lo), a_hi = a truncated to
// 24 significant bits and a_lo = the next 23 bits, both exact FP32 values, so
// |a - a_hi - a_lo| < 2^-46 |a| (split with integer operations only; values
// below 2^-126 in magnitude become 0).  A product a x is a_hi x_hi, made
// exact with an FMA (TwoProd: p + e), plus a_hi x_lo + a_lo x_hi (each within
// 2^-48 |a x|); a_lo x_lo (< 2^-46 |a x|) is dropped.  Sums keep the high
// parts exact with TwoSum and gather every lower-order term in an FP32 low
// word.  The computed r differs from d - T x by less than about
// 2^-45 (|d| + |T| |x|) per entry -- far below the refinement's normwise
// target (1e-12) -- and the r handed to the FP32 correction is rounded to
// FP32 anyway.  The p and TwoSum operations use the _rn intrinsics so that
// no FMA contraction can change them.
// ---------------------------------------------------------------------------
__device__ __forceinline__ float2 split_df(double a)
{
    const unsigned hi = (unsigned)__double2hiint(a), lo = (unsigned)__double2loint(a);
    const unsigned mag = hi & 0x7FFFFFFFu;
    // exponent rebiased 1023 -> 127, then the top 23 mantissa bits (20 from
    // the high word, 3 from the low word) shifted in; sign restored
    const unsigned hb0 = __funnelshift_l(lo, mag - 0x38000000u, 3) | (hi & 0x80000000u);
    const unsigned hb = mag < 0x38100000u ? 0u : hb0;  // |a| < 2^-126: 0
    // the next 23 bits (low word bits 6 .. 28) as an integer q < 2^23:
    // float(2^23 + q) - 2^23 is exact, scaled by 2^-46 in the same FMA, then
    // by the signed power of two of a_hi (its sign and exponent bits)
    const float q = fmaf(__uint_as_float(((lo >> 6) & 0x7FFFFFu) | 0x4B000000u), 0x1p-46f, -0x1p-23f);
    return make_float2(__uint_as_float(hb), q * __uint_as_float(hb & 0xFF800000u));
}

// (sh, sl) += (ah + al) (xh + xl)
__device__ __forceinline__ void df_mac(float ah, float al, float xh, float xl, float &sh, float &sl)
{
    const float p = __fmul_rn(ah, xh);
    const float e = fmaf(ah, xh, -p);
    const float s = __fadd_rn(sh, p);
    const float bb = __fsub_rn(s, sh);
    const float err = __fadd_rn(__fsub_rn(sh, __fsub_rn(s, bb)), __fsub_rn(p, bb));
    sh = s;
    sl += (e + err) + fmaf(ah, xl, al * xh);
}

// (sh, sl) += (bh, bl)
__device__ __forceinline__ void df_add(float bh, float bl, float &sh, float &sl)
{
    const float s = __fadd_rn(sh, bh);
    const float bb = __fsub_rn(s, sh);
    const float err = __fadd_rn(__fsub_rn(sh, __fsub_rn(s, bb)), __fsub_rn(bh, bb));
    sh = s;
    sl += err + bl;
}

// one pass of RHS columns jb .. jb+KB-1 over this thread's column range:
// t = A_i(row, c0:c1) x_i + B_i(row, c0:c1) x_{i+1}; B_i staged (split) for
// the transposed product; the |A| + |B| row-sum partial when asked
template <int KB, bool NORM>
__device__ __forceinline__ void residual_rows_df(const double *__restrict__ Ag, const double *__restrict__ Bg,
                                                 bool has_b, int c0, int c1, int n, int LDp, const float2 *x0,
                                                 const float2 *x1, float2 *sB, bool stage_b, float2 *out, int stride,
                                                 float *rowsum)
{
    float sh[KB], sl[KB];
#pragma unroll
    for (int q = 0; q < KB; ++q) sh[q] = sl[q] = 0.0f;
    float sa = 0.0f;
    if (has_b) {
#pragma unroll 4
        for (int c = c0; c < c1; ++c) {
            const float2 a = split_df(Ag[(long long)c * n]);
            const float2 b = split_df(Bg[(long long)c * n]);
            if (stage_b) sB[c * LDp] = b;
            if (NORM) sa += fabsf(a.x) + fabsf(b.x);
#pragma unroll
            for (int q = 0; q < KB; ++q) {
                const float2 u = x0[c + q * n], v = x1[c + q * n];
                df_mac(a.x, a.y, u.x, u.y, sh[q], sl[q]);
                df_mac(b.x, b.y, v.x, v.y, sh[q], sl[q]);
            }
        }
    } else {
#pragma unroll 4
        for (int c = c0; c < c1; ++c) {
            const float2 a = split_df(Ag[(long long)c * n]);
            if (NORM) sa += fabsf(a.x);
#pragma unroll
            for (int q = 0; q < KB; ++q) {
                const float2 u = x0[c + q * n];
                df_mac(a.x, a.y, u.x, u.y, sh[q], sl[q]);
            }
        }
    }
#pragma unroll
    for (int q = 0; q < KB; ++q) out[q * stride] = make_float2(sh[q], sl[q]);
    if (NORM) *rowsum = sa;
}

// column parts per block row for a CTA of THREADS threads (1 .. 8)
template <int THREADS>
__host__ __device__ constexpr int res_parts(int n)
{
    return THREADS / n < 1 ? 1 : (THREADS / n > 8 ? 8 : THREADS / n);
}

// largest dynamic shared memory of one CTA on sm_103a
constexpr size_t SMEM_CTA_MAX = 227 * 1024;

// threads of a double-float residual CTA: 512 for blocks wider than 64 (one
// CTA per SM fits the staged B_i), else 256
__host__ __device__ constexpr int res_df_threads(int n) { return n > 64 ? 512 : 256; }

// largest shared memory of one residual CTA when choosing the column chunk:
// a 256-thread CTA keeps at least two CTAs per SM (many columns in one pass
// would leave one 8-warp CTA per SM, which costs more than re-reading A and
// B per chunk); a 512-thread CTA may take a whole SM
template <int THREADS>
__host__ __device__ constexpr size_t residual_df_smem_cap()
{
    return THREADS == 256 ? (size_t)112 * 1024 : SMEM_CTA_MAX;
}

// shared memory of residual_body_df: staged B_i (n (n+1)), x ring (3 nk),
// u ping-pong (2 nk), d ping-pong (2 nk) and the t / u partials (2 parts nk)
// as (hi, lo) pairs, plus the FP32 norm partials (25 n); with RAW, the raw
// FP64 A_i and B_i (16-byte aligned) and their mbarrier
template <int THREADS, bool RAW = false>
__host__ __device__ constexpr size_t residual_df_smem_bytes(int n, int k)
{
    return ((((size_t)(n * (n + 1) + 7 * n * k + 2 * res_parts<THREADS>(n) * n * k) * 8 + (size_t)25 * n * 4) + 15) /
            16 * 16) +
           (RAW ? (size_t)2 * n * n * 8 + 16 : 0);
}

// Same decomposition as residual_body (thread = (row, column part); B_i
// staged in shared memory for u_{i+1} = B_i^T x_i; x ring and u ping-pong in
// shared memory), in double-float: shared arrays hold (hi, lo) float pairs.
// The last phase of a block has three independent jobs -- the outputs r_i,
// the next block's d (into its ping-pong slot) and x_{i+2} (into the ring) --
// and a CTA has more threads than n k outputs when k is small, so each job
// starts at a different quarter of the CTA (for k = 1, n = 64 on 256 threads:
// two warps each), and the norm partials at the fourth: their global-memory
// latencies overlap instead of queueing on the output threads.
// Shared memory: residual_df_smem_bytes<THREADS, RAW>(n, k).
// RAW (even n, 16-byte-aligned A and B): each block's FP64 A_i and B_i come
// into shared memory by bulk copies (cp.async.bulk on an mbarrier), the next
// block's issued as soon as this block's first phase has read them, so the
// copy runs during the second and third phases (and the other CTAs' work);
// thread 0 alone waits, bounded by ~1 s of SM clock, and an expired wait
// stops the CTA and records a timeout in the status.
template <class Tr, int THREADS, bool RAW = false>
__device__ __forceinline__ void residual_body_df(const double *__restrict__ A, const double *__restrict__ B,
                                                 const double *__restrict__ x, const double *__restrict__ d,
                                                 Tr *__restrict__ r, long long N, int n, int ktot, int j0, int k,
                                                 long long b0_, long long b1_, int with_norm, DevStatus *st)
{
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int LDp = n + 1;
    const int nk = n * k;
    const long long bstride = (long long)n * ktot, coff = (long long)j0 * n;
    float2 *sB = reinterpret_cast<float2 *>(smem_raw);
    float2 *sxr = sB + n * LDp;      // [3][nk]
    float2 *sub = sxr + 3 * nk;      // [2][nk] u_i ping-pong
    float2 *sdd = sub + 2 * nk;      // [2][nk] d_i ping-pong (split)
    const int parts = res_parts<THREADS>(n);
    float2 *red = sdd + 2 * nk;      // [2][parts][nk]
    float2 *redu = red + parts * nk;  // u partials
    float *rowred = reinterpret_cast<float *>(red + 2 * parts * nk);  // [3][8][n]
    float *rowu = rowred + 24 * n;   // [n]
    const int tid = threadIdx.x;
    const int row = tid % n, part = tid / n;
    const bool active = part < parts;
    const int c0 = active ? (part * n) / parts : 0, c1 = active ? ((part + 1) * n) / parts : 0;
    const long long nn = (long long)n * n;
    const long long b0 = b0_;
    const long long b1 = b1_ < N ? b1_ : N;
    if (b0 >= N) return;
    // RAW: A_i, B_i in shared memory (after the arrays above, 16-byte aligned)
    const size_t raw_off = residual_df_smem_bytes<THREADS, false>(n, k);
    double *rawA = reinterpret_cast<double *>(smem_raw + raw_off);
    double *rawB = rawA + nn;
    uint64_t *rbar = reinterpret_cast<uint64_t *>(rawB + nn);
    int *rabort = reinterpret_cast<int *>(rbar + 1);
    const uint32_t raw_bytes = (uint32_t)(nn * 8);
    uint32_t rphase = 0;
    auto issue_raw = [&](long long blk) {  // thread 0: A_blk (and B_blk when it exists)
        const uint32_t mb = smem_u32(rbar);
        const bool hb = blk + 1 < N;
        fence_async_smem();
        mbar_expect_tx(mb, hb ? 2u * raw_bytes : raw_bytes);
        bulk_g2s(smem_u32(rawA), A + blk * nn, raw_bytes, mb);
        if (hb) bulk_g2s(smem_u32(rawB), B + blk * nn, raw_bytes, mb);
    };
    if constexpr (RAW) {
        if (tid == 0) {
            asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(rbar)) : "memory");
            asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
            *rabort = 0;
            issue_raw(b0);
        }
    }
    if (with_norm < 0) with_norm = st->need_anorm;  // graph mode: decided on the device
    float rmax = 0.0f, xmax = 0.0f, amax = 0.0f;
    auto xs = [&](long long blk) { return sxr + (int)((blk - b0 + 3) % 3) * nk; };  // blk in [b0-1, b1]

    // the first thread of a job that starts at quarter s of the CTA
    const int T = blockDim.x;
    auto rot = [&](int q4) { return (tid + T - (q4 * T) / 4) % T; };
    // prologue: x_{b0-1}, x_{b0}, x_{b0+1}, d_{b0}; u_{b0} = B_{b0-1}^T x_{b0-1}
    for (int e = tid; e < nk; e += blockDim.x) {
        sdd[e] = split_df(d[b0 * bstride + coff + e]);
        xs(b0)[e] = split_df(x[b0 * bstride + coff + e]);
        if (b0 + 1 < N) xs(b0 + 1)[e] = split_df(x[(b0 + 1) * bstride + coff + e]);
        sub[e] = make_float2(0.0f, 0.0f);
    }
    for (int e = tid; e < n; e += blockDim.x) rowu[e] = 0.0f;
    if (b0 > 0) {
        float2 *xm = xs(b0 - 1);
        for (int e = tid; e < nk; e += blockDim.x) xm[e] = split_df(x[(b0 - 1) * bstride + coff + e]);
        for (int e = tid; e < (int)nn; e += blockDim.x) {
            const int c = e / n, rr = e - c * n;
            sB[rr + c * LDp] = split_df(B[(b0 - 1) * nn + e]);
        }
        __syncthreads();
        for (int o = tid; o < nk; o += blockDim.x) {
            const int j = o / n, rr = o - j * n;
            float sh = 0.0f, sl = 0.0f;
            for (int c = 0; c < n; ++c) {
                const float2 b = sB[c + rr * LDp], v = xm[c + j * n];
                df_mac(b.x, b.y, v.x, v.y, sh, sl);
            }
            sub[o] = make_float2(sh, sl);
        }
        if (with_norm)
            for (int rr = tid; rr < n; rr += blockDim.x) {
                float s = 0.0f;
                for (int c = 0; c < n; ++c) s += fabsf(sB[c + rr * LDp].x);
                rowu[rr] = s;
            }
    }
    __syncthreads();

    for (long long i = b0; i < b1; ++i) {
        const int par = (int)((i - b0) & 1);
        const bool has_b = i + 1 < N;
        const float2 *x0 = xs(i);
        const float2 *x1 = xs(i + 1);
        float2 *su = sub + par * nk;         // u_i
        float2 *sun = sub + (par ^ 1) * nk;  // u_{i+1}
        // phase 1: t partials from A_i, B_i; B_i into shared memory (split).
        // RAW: A_i, B_i from their bulk copies; else from global memory, the
        // next block's A and B hinted into L2 meanwhile
        if constexpr (RAW) {
            if (tid == 0) {
                const long long t0 = clock64();
                while (!mbar_test(smem_u32(rbar), rphase))
                    if (clock64() - t0 > C64_WAIT_CYCLES) {
                        *rabort = 1;
                        break;
                    }
                rphase ^= 1u;
            }
            __syncthreads();
            if (*rabort) break;
        } else if (i + 1 < b1) {
            prefetch_l2(A + (i + 1) * nn, (size_t)nn * sizeof(double));
            if (i + 2 < N) prefetch_l2(B + (i + 1) * nn, (size_t)nn * sizeof(double));
        }
        if (active) {
            const double *Ag = (RAW ? rawA : A + i * nn) + row;
            const double *Bg = (RAW ? rawB : B + i * nn) + row;
            // right-hand sides in compile-time groups (4, then 1); the first
            // group also stages B_i and, when asked, the |A| + |B| row sums
            float *rs = rowred + part * n + row;
            float2 *o = red + part * k * n + row;
            int jb = 0;
            if (k >= 4) {
                if (with_norm)
                    residual_rows_df<4, true>(Ag, Bg, has_b, c0, c1, n, LDp, x0, x1, sB + row, true, o, n, rs);
                else
                    residual_rows_df<4, false>(Ag, Bg, has_b, c0, c1, n, LDp, x0, x1, sB + row, true, o, n, rs);
                jb = 4;
            } else {
                if (with_norm)
                    residual_rows_df<1, true>(Ag, Bg, has_b, c0, c1, n, LDp, x0, x1, sB + row, true, o, n, rs);
                else
                    residual_rows_df<1, false>(Ag, Bg, has_b, c0, c1, n, LDp, x0, x1, sB + row, true, o, n, rs);
                jb = 1;
            }
            for (; jb + 4 <= k; jb += 4)
                residual_rows_df<4, false>(Ag, Bg, has_b, c0, c1, n, LDp, x0 + jb * n, x1 + jb * n, sB + row, false,
                                           o + jb * n, n, rs);
            for (; jb < k; ++jb)
                residual_rows_df<1, false>(Ag, Bg, has_b, c0, c1, n, LDp, x0 + jb * n, x1 + jb * n, sB + row, false,
                                           o + jb * n, n, rs);
        }
        __syncthreads();
        if constexpr (RAW) {  // A_i and B_i are read: the next block's copies
            if (tid == 0 && i + 1 < b1) issue_raw(i + 1);
        }
        // phase 2: u_{i+1} partials from the staged B_i
        if (active && has_b) {
            for (int j = 0; j < k; ++j) {
                float sh = 0.0f, sl = 0.0f;
                for (int c = c0; c < c1; ++c) {
                    const float2 b = sB[c + row * LDp], v = x0[c + j * n];
                    df_mac(b.x, b.y, v.x, v.y, sh, sl);
                }
                redu[(part * k + j) * n + row] = make_float2(sh, sl);
            }
            if (with_norm) {
                float sbt = 0.0f;
                for (int c = c0; c < c1; ++c) sbt += fabsf(sB[c + row * LDp].x);
                rowred[16 * n + part * n + row] = sbt;
            }
        }
        __syncthreads();
        // phase 3: r_i = d_i - t - u_i; fetch d_{i+1} and x_{i+2}
        const float2 *sd = sdd + par * nk;
        for (int o = tid; o < nk; o += blockDim.x) {
            const int j = o / n, rr = o - j * n;
            const float2 dd = sd[o];
            float rh = dd.x, rl = dd.y;
            float uh = 0.0f, ul = 0.0f;
            for (int q = 0; q < parts; ++q) {
                const float2 t = red[(q * k + j) * n + rr];
                df_add(-t.x, -t.y, rh, rl);
            }
            df_add(-su[o].x, -su[o].y, rh, rl);
            if (has_b)
                for (int q = 0; q < parts; ++q) {
                    const float2 u = redu[(q * k + j) * n + rr];
                    df_add(u.x, u.y, uh, ul);
                }
            float res_f;
            if constexpr (std::is_same<Tr, double>::value) {
                const double res = (double)rh + (double)rl;
                if (r) r[i * bstride + coff + o] = res;
                res_f = (float)res;
            } else {
                res_f = rh + rl;
                if (r) r[i * bstride + coff + o] = (Tr)res_f;
            }
            rmax = fmaxf(rmax, fabsf(res_f));
            xmax = fmaxf(xmax, fabsf(x0[o].x));
            sun[o] = make_float2(uh, ul);
        }
        if (i + 1 < b1) {
            float2 *sdn = sdd + (par ^ 1) * nk;
            for (int e = rot(1); e < nk; e += T) sdn[e] = split_df(d[(i + 1) * bstride + coff + e]);
        }
        if (with_norm)
            for (int rr = rot(3); rr < n; rr += T) {
                float s = rowu[rr], s2 = 0.0f;
                for (int q = 0; q < parts; ++q) {
                    s += rowred[q * n + rr];
                    if (has_b) s2 += rowred[16 * n + q * n + rr];
                }
                amax = fmaxf(amax, s);
                rowu[rr] = has_b ? s2 : 0.0f;
            }
        if (i + 2 < N && i + 1 < b1) {
            float2 *x2 = xs(i + 2);
            for (int e = rot(2); e < nk; e += T) x2[e] = split_df(x[(i + 2) * bstride + coff + e]);
        }
        __syncthreads();
    }
    if constexpr (RAW) {
        if (*rabort) {  // a copy wait expired: wait (bounded) for the copy in flight, record, stop
            if (tid == 0) {
                const long long t0 = clock64();
                while (!mbar_test(smem_u32(rbar), rphase) && clock64() - t0 < C64_WAIT_CYCLES) {
                }
                atomicExch(&st->tc_timeout, 1);
            }
            return;
        }
    }
    for (int o = 16; o > 0; o >>= 1) {
        rmax = fmaxf(rmax, __shfl_xor_sync(0xffffffffu, rmax, o));
        xmax = fmaxf(xmax, __shfl_xor_sync(0xffffffffu, xmax, o));
        amax = fmaxf(amax, __shfl_xor_sync(0xffffffffu, amax, o));
    }
    if ((threadIdx.x & 31) == 0) {
        atomic_max_nonneg(&st->rnorm, (double)rmax);
        atomic_max_nonneg(&st->xnorm, (double)xmax);
        if (with_norm) atomic_max_nonneg(&st->anorm, (double)amax);
    }
}

template <class Tr, int THREADS, bool RAW = false>
__global__ void __launch_bounds__(THREADS, THREADS == 256 ? (RAW ? 2 : 3) : 1)
    residual_df_kernel(const double *__restrict__ A, const double *__restrict__ B, const double *__restrict__ x,
                       const double *__restrict__ d, Tr *__restrict__ r, long long N, int n, int ktot, int j0, int k,
                       long long per_cta, int with_norm, DevStatus *st)
{
    const long long b0 = (long long)blockIdx.x * per_cta;
    residual_body_df<Tr, THREADS, RAW>(A, B, x, d, r, N, n, ktot, j0, k, b0, b0 + per_cta, with_norm, st);
}

// many systems: one CTA per (system, block range) item
template <class Tr>
struct ResidualDesc {
    const double *A, *B, *x, *d;
    Tr *r;
    long long N;
    int n, k;
    int j0, kc;    // column chunk of this descriptor
    int norm;      // -1: ||T||_inf when the status asks for it (first chunk), 0: never
    long long per_cta;
    DevStatus *st;
};

template <class Tr, int THREADS>
__global__ void __launch_bounds__(THREADS, THREADS == 256 ? 3 : 1)
    residual_batch_kernel(const ResidualDesc<Tr> *__restrict__ descs, const WorkItem *__restrict__ items)
{
    const WorkItem w = items[blockIdx.x];
    const ResidualDesc<Tr> g = descs[w.desc];
    const long long b0 = (long long)w.p * g.per_cta;
    residual_body_df<Tr, THREADS>(g.A, g.B, g.x, g.d, g.r, g.N, g.n, g.k, g.j0, g.kc, b0, b0 + g.per_cta, g.norm,
                                  g.st);
}

// one refinement decision on the device (graph mode): relative residual,
// convergence, and the two conditional-node values (loop again / apply a
// correction) -- no host round trip per refinement step
static __global__ void relres_control_kernel(DevStatus *st, double tol, int max_refine,
                                             cudaGraphConditionalHandle hloop, cudaGraphConditionalHandle hcorr)
{
    if (threadIdx.x == 0 && blockIdx.x == 0) {
        const double rn = __longlong_as_double((long long)st->rnorm);
        const double xn = __longlong_as_double((long long)st->xnorm);
        const double dn = __longlong_as_double((long long)st->dnorm);
        const double an = __longlong_as_double((long long)st->anorm);
        const double den = an * xn + dn;
        const double rel = den > 0.0 ? rn / den : 0.0;
        const int done = (rel <= tol) ? 1 : 0;
        const int cont = (!done && st->iters < max_refine) ? 1 : 0;
        st->relres = rel;
        st->done = done;
        st->need_anorm = 0;
        if (cont) {
            st->iters += 1;
            st->iters_total += 1;
        }
        cudaGraphSetConditional(hloop, (unsigned)cont);
        cudaGraphSetConditional(hcorr, (unsigned)cont);
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

// ---------------------------------------------------------------------------
// many-system (batch) helpers: descriptor arrays + work items
// ---------------------------------------------------------------------------
constexpr int BATCH_CHUNK = 4096;  // elements per work item of the elementwise batch kernels

template <class Tsrc, class T, class Tdst>
struct AsmSchurDesc {
    const Tsrc *A_src;
    const T *C;
    Tdst *A_next;
    Tdst *B_next;
    long long N, Q;
    int n;
};

template <class Tsrc, class T, class Tdst>
__global__ void assemble_schur_batch_kernel(const AsmSchurDesc<Tsrc, T, Tdst> *__restrict__ descs,
                                            const WorkItem *__restrict__ items)
{
    const WorkItem w = items[blockIdx.x];
    const AsmSchurDesc<Tsrc, T, Tdst> g = descs[w.desc];
    const long long nn = (long long)g.n * g.n;
    const long long totalA = (g.Q + 1) * nn, total = totalA + g.Q * nn;
    const long long e0 = (long long)w.p * BATCH_CHUNK;
    for (long long e = e0 + threadIdx.x; e < total && e < e0 + BATCH_CHUNK; e += blockDim.x) {
        if (e < totalA) {
            const long long s = e / nn, q = e % nn;
            const long long blk = (s * (g.N - 1)) / g.Q;
            double v = (double)g.A_src[blk * nn + q];
            if (s < g.Q) v -= (double)g.C[s * 3 * nn + q];
            if (s > 0) v -= (double)g.C[(s - 1) * 3 * nn + nn + q];
            g.A_next[e] = (Tdst)v;
        } else {
            const long long f = e - totalA;
            const long long s = f / nn, q = f % nn;
            g.B_next[f] = (Tdst)(-g.C[s * 3 * nn + 2 * nn + q]);
        }
    }
}

template <class T, class Tn>
struct AsmRhsDesc {
    const T *d;
    const T *bvec;
    Tn *dn;
    long long N, Q;
    int n, k, j0, kc;
};

template <class T, class Tn>
__global__ void assemble_rhs_batch_kernel(const AsmRhsDesc<T, Tn> *__restrict__ descs,
                                          const WorkItem *__restrict__ items)
{
    const WorkItem w = items[blockIdx.x];
    const AsmRhsDesc<T, Tn> g = descs[w.desc];
    const long long per = (long long)g.n * g.kc;
    const long long total = (g.Q + 1) * per;
    const long long e0 = (long long)w.p * BATCH_CHUNK;
    for (long long e = e0 + threadIdx.x; e < total && e < e0 + BATCH_CHUNK; e += blockDim.x) {
        const long long s = e / per, q = e % per;
        const long long blk = (s * (g.N - 1)) / g.Q;
        const long long off = (long long)g.j0 * g.n + q;
        double v = (double)g.d[blk * (long long)g.n * g.k + off];
        if (s < g.Q) v -= (double)g.bvec[s * 2 * per + q];
        if (s > 0) v -= (double)g.bvec[(s - 1) * 2 * per + per + q];
        g.dn[s * (long long)g.n * g.k + off] = (Tn)v;
    }
}

// per-system vector operations of the batched refinement loop
enum { VEC_ABSMAX = 0, VEC_TO_CORR = 1, VEC_SET = 2, VEC_ADD = 3, VEC_COPY_OUT = 4 };

template <class Tc>
struct VecDesc {
    double *x;           // FP64 solution accumulator
    Tc *c;               // correction / RHS in the factor precision
    double *d;           // the user's FP64 right-hand side (solution on exit)
    long long count;
    DevStatus *st;
};

template <class Tc>
__global__ void vec_batch_kernel(const VecDesc<Tc> *__restrict__ descs, const WorkItem *__restrict__ items, int op)
{
    const WorkItem w = items[blockIdx.x];
    const VecDesc<Tc> g = descs[w.desc];
    const long long e0 = (long long)w.p * BATCH_CHUNK;
    double m = 0.0;
    for (long long e = e0 + threadIdx.x; e < g.count && e < e0 + BATCH_CHUNK; e += blockDim.x) {
        switch (op) {
        case VEC_ABSMAX: m = fmax(m, fabs(g.d[e])); break;
        case VEC_TO_CORR: g.c[e] = (Tc)g.d[e]; break;
        case VEC_SET: g.x[e] = (double)g.c[e]; break;
        case VEC_ADD:
            if (g.st->active) g.x[e] += (double)g.c[e];
            break;
        default: g.d[e] = g.x[e]; break;
        }
    }
    if (op == VEC_ABSMAX) {
        for (int o = 16; o > 0; o >>= 1) m = fmax(m, __shfl_xor_sync(0xffffffffu, m, o));
        if ((threadIdx.x & 31) == 0) atomic_max_nonneg(&g.st->dnorm, m);
    }
}

// per-system decision of the batched refinement loop; *any_cont collects
// "some system still needs a correction"
static __global__ void batch_decide_kernel(DevStatus *const *__restrict__ sts, int nsys, double tol, int max_refine,
                                    int *any_cont)
{
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= nsys) return;
    DevStatus *st = sts[s];
    const double rn = __longlong_as_double((long long)st->rnorm);
    const double xn = __longlong_as_double((long long)st->xnorm);
    const double dn = __longlong_as_double((long long)st->dnorm);
    const double an = __longlong_as_double((long long)st->anorm);
    const double den = an * xn + dn;
    const double rel = den > 0.0 ? rn / den : 0.0;
    const int done = (rel <= tol) ? 1 : 0;
    st->relres = rel;
    st->done = done;
    st->need_anorm = 0;
    st->rnorm = 0ULL;
    st->xnorm = 0ULL;
    // a system stops taking corrections exactly where it would alone, so its
    // result does not depend on the other systems of the batch
    const int cont = (!done && st->iters < max_refine) ? 1 : 0;
    st->active = cont;
    if (cont) {
        st->iters += 1;
        st->iters_total += 1;
        atomicOr(any_cont, 1);
    }
}

static __global__ void batch_set_conditional_kernel(int *any_cont, int *round, int max_refine,
                                                    cudaGraphConditionalHandle hloop, cudaGraphConditionalHandle hcorr)
{
    if (threadIdx.x == 0 && blockIdx.x == 0) {
        const int cont = (*any_cont != 0 && *round < max_refine) ? 1 : 0;
        *any_cont = 0;
        *round += 1;
        cudaGraphSetConditional(hloop, (unsigned)cont);
        cudaGraphSetConditional(hcorr, (unsigned)cont);
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

#include "bss_chain64_tc.cuh"
#include "bss_chain128_tc.cuh"
#include "bss_stream.cuh"
