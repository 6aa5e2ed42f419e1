// Streamed solve sweeps for blocks too large to double-buffer whole in
// shared memory (FP32 90 < n <= 128, FP64 64 < n <= 128; n a multiple of 16):
// the forward and backward chain sweeps of a partitioned level (reference
// solve!, src/gpu_batched.jl:229-258: the Schur RHS of compute_schur_RHS!
// and the boundary update of update_boundary!, src/backbone_cuda.jl:159-184,
// fused as in chain_fwd_body / chain_bwd_body), with every n x n block
// passing through a ring of four shared-memory slots.
//
// A block is column-major, so a quarter of its columns (n/4 columns, n^2/4
// elements) is contiguous: one bulk copy (cp.async.bulk) per slot, completing
// on that slot's mbarrier.  The ring holds one block.  The blocks a sweep
// needs come in a fixed order (forward step i: W_{i-1}, V_i, Y_i, and W_last
// at the end; backward step i: Y_i, W_i, V_i), so as soon as the CTA has used
// quarter q of a block, thread 0 issues quarter q of the next block into the
// same slot: each copy has three quarters of compute to land, and the block
// after that is hinted into L2 (cp.async.bulk.prefetch.L2).  The hint runs
// one block ahead, not one step: the three blocks of a step over all
// partitions (58 MB in FP32 at n = 128) held twice would exceed the 126 MB L2
// and be evicted before their copies read them.
// The forward products (M^T v, one result per column of the slot) give each
// column 8 lanes that read its rows in interleaved vector chunks and sum by
// shuffles; the backward product (M x, a result per row) gives each thread
// four rows and four right-hand sides over a share of the columns, the
// shares summed through shared memory once per block product.
//
// Thread 0 alone waits on the mbarriers (a spin on mbarrier.test_wait,
// bounded by ~1 s of SM clock); the others meet it at a CTA barrier.  An
// expired wait stops the sweep, thread 0 waits (bounded) for its copies
// still in flight, and the status records a timeout (the solution is void).
#pragma once

namespace bss {

// the forward product gives each column of a quarter slot (n / 4 columns) 8
// lanes and needs whole warps (n a multiple of 16); the backward one holds
// at most 8 right-hand sides per row group
template <class T>
__host__ __device__ constexpr bool solve_streamed(int n, int kc)
{
    return n % 16 == 0 && n <= 128 && !solve_staged<T>(n, kc) && kc <= 8;
}

// partial sums of the backward product: (column parts) x n x kc <= 4096 elements
constexpr int STREAM_PARTIAL = 4096;

// ring (one block) + 6 vectors of n x kc + the backward partials + 4 mbarriers + abort flag
template <class T>
__host__ __device__ constexpr size_t stream_smem_bytes(int n, int kc)
{
    return (size_t)n * n * sizeof(T) + (size_t)6 * n * kc * sizeof(T) + (size_t)STREAM_PARTIAL * sizeof(T) + 64;
}

struct StreamRing {
    uint32_t base;     // shared address of slot 0
    uint32_t bars;     // shared address of mbarrier 0 (8 bytes each)
    uint32_t qbytes;   // bytes per quarter
    uint32_t phase;    // bit q: parity of slot q's outstanding completion
    uint32_t pending;  // bit q: a copy into slot q not yet waited for
};

// thread 0: quarter q of block M into slot q
template <class T>
__device__ __forceinline__ void ring_issue(StreamRing &rg, const T *M, int q, int qelems)
{
    const uint32_t bar = rg.bars + 8u * (uint32_t)q;
    mbar_expect_tx(bar, rg.qbytes);
    bulk_g2s(rg.base + (uint32_t)q * rg.qbytes, M + (long long)q * qelems, rg.qbytes, bar);
    rg.pending |= 1u << q;
}

// thread 0: wait for slot q, at most C64_WAIT_CYCLES; false when it expired
__device__ __forceinline__ bool ring_wait(StreamRing &rg, int q)
{
    if (!(rg.pending & (1u << q))) return true;
    const uint32_t bar = rg.bars + 8u * (uint32_t)q;
    const uint32_t par = (rg.phase >> q) & 1u;
    const long long t0 = clock64();
    while (!mbar_test(bar, par))
        if (clock64() - t0 > C64_WAIT_CYCLES) return false;
    rg.phase ^= 1u << q;
    rg.pending &= ~(1u << q);
    return true;
}

// out(c0 + c, j) (+)= sign * sum_r M(r, c) v(r, j) for the qc columns of a
// slot, in groups of four right-hand sides: the 8 lanes (c, part) of a
// quarter-warp share column c, lane `part` takes the vector chunks part,
// part + 8, ... of the column (so a quarter-warp reads 128 contiguous bytes
// of M and of v per step: no bank conflicts), multiplies each with all four
// v columns, and a 3-level shuffle sums the 8 parts. qc is a multiple of 4,
// so whole warps leave together.
template <class T>
__device__ __forceinline__ void slot_tmul8(const T *sM, int qc, const T *v, T *out, int c0, int n, int kc, T sign,
                                           bool accumulate)
{
    using VT = typename Vec<T>::type;
    constexpr int W = Vec<T>::W;
    const int part = threadIdx.x & 7, c = threadIdx.x >> 3;
    if (c >= qc) return;
    const T *mc = sM + (size_t)c * n;
    for (int j0 = 0; j0 < kc; j0 += 4) {
        T acc[4] = {T(0), T(0), T(0), T(0)};
        for (int r = part * W; r < n; r += 8 * W) {
            const VT m = *reinterpret_cast<const VT *>(mc + r);
#pragma unroll
            for (int q = 0; q < 4; ++q)
                if (j0 + q < kc) fma_vec(acc[q], m, *reinterpret_cast<const VT *>(v + r + (size_t)(j0 + q) * n));
        }
#pragma unroll
        for (int o = 4; o > 0; o >>= 1)
#pragma unroll
            for (int q = 0; q < 4; ++q) acc[q] += __shfl_xor_sync(0xffffffffu, acc[q], o);
        if (part == 0) {
#pragma unroll
            for (int q = 0; q < 4; ++q)
                if (j0 + q < kc) {
                    const int oo = c0 + c + (j0 + q) * n;
                    out[oo] = accumulate ? out[oo] + sign * acc[q] : sign * acc[q];
                }
        }
    }
}

// Backward product mapping: thread (rg, jg, part) owns rows 4 rg .. 4 rg + 3
// and right-hand sides 4 jg .. 4 jg + 3 of M x, summed over the slot columns
// c = part, part + np, ...: one 128-bit read of M's column segment (lanes on
// consecutive row groups: conflict-free) and broadcast reads of x feed 16
// FMAs; the np column parts are summed through shared memory per block.
struct BwdMap {
    int rg, jg, part, np;
    bool active;
};

__device__ __forceinline__ BwdMap bwd_map(int n, int kc)
{
    const int ngr = n / 4, njg = (kc + 3) / 4;
    BwdMap m;
    m.np = SOLVE_THREADS / (ngr * njg);
    m.rg = threadIdx.x % ngr;
    const int rest = threadIdx.x / ngr;
    m.jg = rest % njg;
    m.part = rest / njg;
    m.active = m.part < m.np;
    return m;
}

// acc[u][q] += sum_c M(4 rg + u, c) x(c0 + c, 4 jg + q) over this thread's
// columns of a slot (qc columns, leading dimension n)
template <class T>
__device__ __forceinline__ void slot_nmul4(const T *sM, int qc, const T *x, int c0, int n, int kc, const BwdMap &bm,
                                           T (&acc)[4][4])
{
    if (!bm.active) return;
    const int j0 = 4 * bm.jg;
    for (int c = bm.part; c < qc; c += bm.np) {
        const T *mc = sM + (size_t)c * n + 4 * bm.rg;
        T m[4];
        if constexpr (sizeof(T) == 4) {
            const float4 v = *reinterpret_cast<const float4 *>(mc);
            m[0] = v.x;
            m[1] = v.y;
            m[2] = v.z;
            m[3] = v.w;
        } else {
            const double2 v0 = *reinterpret_cast<const double2 *>(mc);
            const double2 v1 = *reinterpret_cast<const double2 *>(mc + 2);
            m[0] = v0.x;
            m[1] = v0.y;
            m[2] = v1.x;
            m[3] = v1.y;
        }
#pragma unroll
        for (int q = 0; q < 4; ++q) {
            if (j0 + q < kc) {
                const T xv = x[c0 + c + (j0 + q) * n];
#pragma unroll
                for (int u = 0; u < 4; ++u) acc[u][q] = fma(m[u], xv, acc[u][q]);
            }
        }
    }
}

// the column parts' sums: every thread writes its partial block, then each
// output e of the n x kc result is the sum over the parts (ends with the
// outputs handed to `out(e, sum)`; barriers before and after)
template <class T, class F>
__device__ __forceinline__ void bwd_reduce(T *red, T (&acc)[4][4], int n, int kc, const BwdMap &bm, F out)
{
    const int nkc = n * kc;
    if (bm.active) {
#pragma unroll
        for (int q = 0; q < 4; ++q) {
            const int j = 4 * bm.jg + q;
            if (j < kc) {
#pragma unroll
                for (int u = 0; u < 4; ++u) red[bm.part * nkc + j * n + 4 * bm.rg + u] = acc[u][q];
            }
        }
    }
#pragma unroll
    for (int u = 0; u < 4; ++u)
#pragma unroll
        for (int q = 0; q < 4; ++q) acc[u][q] = T(0);
    __syncthreads();
    for (int e = threadIdx.x; e < nkc; e += blockDim.x) {
        T s = T(0);
        for (int q = 0; q < bm.np; ++q) s += red[q * nkc + e];
        out(e, s);
    }
    __syncthreads();
}

// one pass of a block through the ring: `use(q, slot)` for each quarter,
// then quarter q of `next` (when not null) issued into the freed slot;
// `after` (the block following `next`, or null) is hinted into L2.
// Returns false (in every thread) when a wait expired.
template <class T, class F>
__device__ __forceinline__ bool ring_pass(StreamRing &rg, T *ring, int qelems, const T *next, const T *after,
                                          int *abort, F use)
{
    if (threadIdx.x == 32 && after) bulk_prefetch_l2(after, 4u * rg.qbytes);
#pragma unroll 1
    for (int q = 0; q < 4; ++q) {
        if (threadIdx.x == 0 && !ring_wait(rg, q)) *abort = 1;
        __syncthreads();
        if (*abort) return false;
        use(q, ring + (size_t)q * qelems);
        __syncthreads();
        if (threadIdx.x == 0 && next) {
            fence_async_smem();
            ring_issue<T>(rg, next, q, qelems);
        }
    }
    return true;
}

template <class T>
__device__ __forceinline__ void ring_setup(StreamRing &rg, T *ring, uint64_t *bars, int *abort, int n)
{
    rg.base = smem_u32(ring);
    rg.bars = smem_u32(bars);
    rg.qbytes = (uint32_t)((size_t)n * n / 4 * sizeof(T));
    rg.phase = 0u;
    rg.pending = 0u;
    if (threadIdx.x == 0) {
        for (int q = 0; q < 4; ++q)
            asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(&bars[q])) : "memory");
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        *abort = 0;
    }
    __syncthreads();
}

// on an expired wait: thread 0 waits (bounded) for its copies in flight and
// records the timeout
__device__ __forceinline__ void ring_abort(StreamRing &rg, DevStatus *st)
{
    if (threadIdx.x != 0) return;
    for (int q = 0; q < 4; ++q) ring_wait(rg, q);
    if (st) atomicExch(&st->tc_timeout, 1);
}

// forward sweep of partition p: y_i = V_i^T (d_i - W_{i-1}^T y_{i-1}),
// bL = sum Y_i^T y_i, bR = W_last^T y_last (as chain_fwd_body)
template <class T>
__device__ __forceinline__ void chain_fwd_stream_body(const SolveArgs<T> &g, const long long p)
{
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int n = g.n, kc = g.kc;
    const int nn = n * n, nkc = n * kc, qelems = nn / 4, qc = n / 4;
    T *ring = reinterpret_cast<T *>(smem_raw);
    T *sr = ring + nn;
    T *sy = sr + nkc;
    T *sbL = sy + nkc;
    T *sbR = sbL + nkc;
    uint64_t *bars = reinterpret_cast<uint64_t *>(sbR + nkc + 2 * nkc);
    int *abort = reinterpret_cast<int *>(bars + 4);
    const long long sL = (p * (g.N - 1)) / g.Q;
    const long long sR = ((p + 1) * (g.N - 1)) / g.Q;
    const long long first = sL + 1, last = sR - 1;
    StreamRing rg;
    ring_setup<T>(rg, ring, bars, abort, n);
    if (threadIdx.x == 0)
        for (int q = 0; q < 4; ++q) ring_issue<T>(rg, g.Af + first * (long long)nn, q, qelems);
    for (int e = threadIdx.x; e < nkc; e += blockDim.x) sbL[e] = T(0);
    for (long long i = first; i <= last; ++i) {
        if (threadIdx.x == 64 && i < last)
            bulk_prefetch_l2(rhs_ptr<T>(g.d, i + 1, n, g.k, g.j0), (uint32_t)(nkc * sizeof(T)));
        load_rhs(sr, g.d, i, n, g.k, g.j0, kc);
        if (i > first) {
            __syncthreads();
            // sr -= W_{i-1}^T y_{i-1}; the ring holds W_{i-1}, then V_i
            if (!ring_pass<T>(rg, ring, qelems, g.Af + i * (long long)nn, g.Y + i * (long long)nn, abort,
                              [&](int q, const T *slot) { slot_tmul8<T>(slot, qc, sy, sr, q * qc, n, kc, T(-1), true); }))
                return ring_abort(rg, g.st);
        }
        __syncthreads();
        // y_i = V_i^T sr; then Y_i
        if (!ring_pass<T>(rg, ring, qelems, g.Y + i * (long long)nn, g.Bf + i * (long long)nn, abort,
                          [&](int q, const T *slot) { slot_tmul8<T>(slot, qc, sr, sy, q * qc, n, kc, T(1), false); }))
            return ring_abort(rg, g.st);
        // bL += Y_i^T y_i; then W_i (the next step's W_{i-1}, or W_last)
        const T *after = i < last ? g.Af + (i + 1) * (long long)nn : (const T *)nullptr;
        if (!ring_pass<T>(rg, ring, qelems, g.Bf + i * (long long)nn, after, abort,
                          [&](int q, const T *slot) { slot_tmul8<T>(slot, qc, sy, sbL, q * qc, n, kc, T(1), true); }))
            return ring_abort(rg, g.st);
        store_rhs(g.d, sy, i, n, g.k, g.j0, kc);
    }
    // bR = W_last^T y_last
    if (!ring_pass<T>(rg, ring, qelems, (const T *)nullptr, (const T *)nullptr, abort,
                      [&](int q, const T *slot) { slot_tmul8<T>(slot, qc, sy, sbR, q * qc, n, kc, T(1), false); }))
        return ring_abort(rg, g.st);
    T *bp = g.bvec + p * 2 * (long long)nkc;
    for (int e = threadIdx.x; e < nkc; e += blockDim.x) {
        bp[e] = sbL[e];
        bp[nkc + e] = sbR[e];
    }
}

// backward sweep of partition p: x_i = V_i (y_i - Y_i x_L - W_i x_{i+1})
// with x_{last+1} = x_R (as chain_bwd_body); separators copied from xsep
template <class T, class Tsep>
__device__ __forceinline__ void chain_bwd_stream_body(const SolveArgs<T> &g, const long long p)
{
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int n = g.n, kc = g.kc;
    const int nn = n * n, nkc = n * kc, qelems = nn / 4, qc = n / 4;
    T *ring = reinterpret_cast<T *>(smem_raw);
    T *sz = ring + nn;
    T *sxL = sz + nkc;
    T *sxn = sxL + nkc;
    T *sxt = sxn + nkc;
    T *red = sxt + 3 * nkc;  // STREAM_PARTIAL elements
    uint64_t *bars = reinterpret_cast<uint64_t *>(red + STREAM_PARTIAL);
    int *abort = reinterpret_cast<int *>(bars + 4);
    const long long sL = (p * (g.N - 1)) / g.Q;
    const long long sR = ((p + 1) * (g.N - 1)) / g.Q;
    const long long first = sL + 1, last = sR - 1;
    const Tsep *xs = reinterpret_cast<const Tsep *>(g.xsep);
    StreamRing rg;
    ring_setup<T>(rg, ring, bars, abort, n);
    if (threadIdx.x == 0)
        for (int q = 0; q < 4; ++q) ring_issue<T>(rg, g.Y + last * (long long)nn, q, qelems);
    load_rhs(sxL, xs, p, n, g.k, g.j0, kc);
    load_rhs(sxn, xs, p + 1, n, g.k, g.j0, kc);
    __syncthreads();
    store_rhs(g.d, sxL, sL, n, g.k, g.j0, kc);
    if (p == g.Q - 1) store_rhs(g.d, sxn, sR, n, g.k, g.j0, kc);
    const BwdMap bm = bwd_map(n, kc);
    T acc[4][4];
#pragma unroll
    for (int u = 0; u < 4; ++u)
#pragma unroll
        for (int q = 0; q < 4; ++q) acc[u][q] = T(0);
    for (long long i = last; i >= first; --i) {
        if (threadIdx.x == 64 && i > first)
            bulk_prefetch_l2(rhs_ptr<T>(g.d, i - 1, n, g.k, g.j0), (uint32_t)(nkc * sizeof(T)));
        load_rhs(sz, g.d, i, n, g.k, g.j0, kc);
        // acc = Y_i x_L (ring: Y_i, then W_i)
        if (!ring_pass<T>(rg, ring, qelems, g.Bf + i * (long long)nn, g.Af + i * (long long)nn, abort,
                          [&](int q, const T *slot) { slot_nmul4<T>(slot, qc, sxL, q * qc, n, kc, bm, acc); }))
            return ring_abort(rg, g.st);
        // acc += W_i x_{i+1} (ring: W_i, then V_i)
        const T *prevY = i > first ? g.Y + (i - 1) * (long long)nn : (const T *)nullptr;
        if (!ring_pass<T>(rg, ring, qelems, g.Af + i * (long long)nn, prevY, abort,
                          [&](int q, const T *slot) { slot_nmul4<T>(slot, qc, sxn, q * qc, n, kc, bm, acc); }))
            return ring_abort(rg, g.st);
        bwd_reduce<T>(red, acc, n, kc, bm, [&](int e, T s) { sz[e] -= s; });
        // x_i = V_i z (ring: V_i, then Y_{i-1})
        const T *prevW = i > first ? g.Bf + (i - 1) * (long long)nn : (const T *)nullptr;
        if (!ring_pass<T>(rg, ring, qelems, prevY, prevW, abort,
                          [&](int q, const T *slot) { slot_nmul4<T>(slot, qc, sz, q * qc, n, kc, bm, acc); }))
            return ring_abort(rg, g.st);
        bwd_reduce<T>(red, acc, n, kc, bm, [&](int e, T s) { sxt[e] = s; });
        for (int e = threadIdx.x; e < nkc; e += blockDim.x) sxn[e] = sxt[e];
        store_rhs(g.d, sxt, i, n, g.k, g.j0, kc);
        __syncthreads();
    }
}

template <class T>
__global__ void __launch_bounds__(SOLVE_THREADS) chain_fwd_stream_kernel(SolveArgs<T> g)
{
    chain_fwd_stream_body<T>(g, blockIdx.x);
}

template <class T, class Tsep>
__global__ void __launch_bounds__(SOLVE_THREADS) chain_bwd_stream_kernel(SolveArgs<T> g)
{
    chain_bwd_stream_body<T, Tsep>(g, blockIdx.x);
}

}  // namespace bss
