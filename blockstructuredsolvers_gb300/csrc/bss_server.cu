// Kalman-smoother block builder on the device and the request server
// (continuous batching under an HBM budget, resident factors, per-request
// latency).  Neither has a counterpart in the reference's solver API; the
// builder restates build_kf_blocks (benchmark/benchmark_kf.jl:105-154).
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <mutex>
#include <thread>
#include <unordered_map>
#include <vector>

#include "bss_internal.h"

using namespace bss;

// ---------------------------------------------------------------------------
// Kalman-smoother blocks
// ---------------------------------------------------------------------------
namespace {

// scratch of the builder (FP64, n x n unless noted)
struct KfScratch {
    double *QF, *FQF, *HRH, *RH /* m x n */, *Aint, *Afirst, *Alast, *Bup, *p0x /* n */;
    static size_t doubles(long long n, long long m) { return 7 * n * n + m * n + n; }
    void carve(double *base, long long n, long long m)
    {
        QF = base;
        FQF = QF + n * n;
        HRH = FQF + n * n;
        RH = HRH + n * n;
        Aint = RH + m * n;
        Afirst = Aint + n * n;
        Alast = Afirst + n * n;
        Bup = Alast + n * n;
        p0x = Bup + n * n;
    }
};

// one CTA: the per-model blocks (O(n^3) once per model)
__global__ void kf_prepare_kernel(int n, int m, const double *F, const double *H, const double *Qinv,
                                  const double *Rinv, const double *P0inv, const double *x0, KfScratch w)
{
    const int nn = n * n;
    for (int e = threadIdx.x; e < nn; e += blockDim.x) {  // QF = Q^{-1} F
        const int r = e % n, c = e / n;
        double s = 0.0;
        for (int j = 0; j < n; ++j) s = fma(Qinv[r + j * n], F[j + c * n], s);
        w.QF[e] = s;
    }
    for (int e = threadIdx.x; e < m * n; e += blockDim.x) {  // RH = R^{-1} H
        const int r = e % m, c = e / m;
        double s = 0.0;
        for (int j = 0; j < m; ++j) s = fma(Rinv[r + j * m], H[j + c * m], s);
        w.RH[e] = s;
    }
    __syncthreads();
    for (int e = threadIdx.x; e < nn; e += blockDim.x) {  // F^T Q^{-1} F and H^T R^{-1} H
        const int r = e % n, c = e / n;
        double s = 0.0, t = 0.0;
        for (int j = 0; j < n; ++j) s = fma(F[j + r * n], w.QF[j + c * n], s);
        for (int j = 0; j < m; ++j) t = fma(H[j + r * m], w.RH[j + c * m], t);
        w.FQF[e] = s;
        w.HRH[e] = t;
    }
    for (int e = threadIdx.x; e < n; e += blockDim.x) {
        double s = 0.0;
        if (P0inv && x0)
            for (int j = 0; j < n; ++j) s = fma(P0inv[e + j * n], x0[j], s);
        w.p0x[e] = s;
    }
    __syncthreads();
    for (int e = threadIdx.x; e < nn; e += blockDim.x) {
        const int r = e % n, c = e / n;
        const int u = r <= c ? e : c + r * n;  // upper-triangle source (Symmetric(Akk))
        const double hrh = w.HRH[u], fqf = w.FQF[u], qi = Qinv[u];
        w.Aint[e] = hrh + qi + fqf;
        w.Afirst[e] = P0inv ? hrh + P0inv[u] + fqf : hrh + qi + fqf;
        w.Alast[e] = P0inv ? hrh + qi : hrh + qi + fqf;
        w.Bup[e] = -w.QF[c + r * n];  // -(Q^{-1} F)^T
    }
}

__global__ void kf_fill_ab_kernel(long long N, int n, KfScratch w, double *A, double *B)
{
    const long long nn = (long long)n * n;
    const long long totalA = N * nn, total = totalA + (N - 1) * nn;
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < total;
         e += (long long)gridDim.x * blockDim.x) {
        if (e < totalA) {
            const long long i = e / nn, q = e - i * nn;
            A[e] = (i == 0) ? w.Afirst[q] : (i == N - 1 ? w.Alast[q] : w.Aint[q]);
        } else {
            B[e - totalA] = w.Bup[(e - totalA) % nn];
        }
    }
}

// d_i(:, j) = (R^{-1} H)^T y_i(:, j) (+ P0^{-1} x0 at i = 0)
__global__ void kf_fill_d_kernel(long long N, int n, int m, int k, KfScratch w, const double *y, double *d)
{
    const long long total = N * n * k;
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < total;
         e += (long long)gridDim.x * blockDim.x) {
        const long long r = e % n, col = e / n;  // col = i * k + j
        const long long i = col / k;
        const double *yc = y + col * m;
        double s = (i == 0) ? w.p0x[r] : 0.0;
        for (int l = 0; l < m; ++l) s = fma(w.RH[l + r * m], yc[l], s);
        d[e] = s;
    }
}

int kf_grid(long long work) { return (int)std::max(1LL, std::min((work + 255) / 256, 152LL * 8)); }

cudaError_t kf_launch_prepare(long long n, long long m, const double *F, const double *H, const double *Qinv,
                              const double *Rinv, const double *P0inv, const double *x0, const KfScratch &w,
                              cudaStream_t s)
{
    kf_prepare_kernel<<<1, 256, 0, s>>>((int)n, (int)m, F, H, Qinv, Rinv, P0inv, x0, w);
    count_launch();
    return cudaGetLastError();
}

cudaError_t kf_launch_fill(long long N, long long n, long long m, long long k, const KfScratch &w, const double *y,
                           double *A, double *B, double *d, cudaStream_t s)
{
    if (A) {
        kf_fill_ab_kernel<<<kf_grid((2 * N - 1) * n * n), 256, 0, s>>>(N, (int)n, w, A, B);
        count_launch();
        const cudaError_t e = cudaGetLastError();
        if (e != cudaSuccess) return e;
    }
    kf_fill_d_kernel<<<kf_grid(N * n * k), 256, 0, s>>>(N, (int)n, (int)m, (int)k, w, y, d);
    count_launch();
    return cudaGetLastError();
}

}  // namespace

extern "C" int bss_kf_build(int64_t N, int64_t n, int64_t m, int64_t k, const double *F, const double *H,
                            const double *Qinv, const double *Rinv, const double *P0inv, const double *x0,
                            const double *y, double *A, double *B, double *d, void *stream)
{
    if (N < 1 || n < 1 || m < 1 || k < 1 || !F || !H || !Qinv || !Rinv || !y || !A || !d || (N > 1 && !B))
        return fail(BSS_ERR_ARG, "bss_kf_build: bad argument");
    cudaStream_t s = (cudaStream_t)stream;
    double *scratch = nullptr;
    BSS_CUDA(cudaMallocAsync((void **)&scratch, KfScratch::doubles(n, m) * sizeof(double), s));
    KfScratch w;
    w.carve(scratch, n, m);
    cudaError_t e = kf_launch_prepare(n, m, F, H, Qinv, Rinv, P0inv, x0, w, s);
    if (e == cudaSuccess) e = kf_launch_fill(N, n, m, k, w, y, A, B, d, s);
    cudaFreeAsync(scratch, s);
    if (e != cudaSuccess) return cuda_fail(e, "bss_kf_build");
    return BSS_OK;
}

// ---------------------------------------------------------------------------
// request server
// ---------------------------------------------------------------------------
namespace {

using Clock = std::chrono::steady_clock;

enum { RQ_SYSTEM = 0, RQ_KALMAN = 1, RQ_RHS = 2 };
enum { PH_QUEUED = 0, PH_SOLVE = 1, PH_REFINE = 2, PH_FINISH = 3, PH_DONE = 4 };

struct Factor {
    uint64_t id = 0;
    bss_handle *h = nullptr;
    size_t bytes = 0;         // handle arena + Kalman model buffers
    int slot = 0;
    int users = 0;            // requests queued or running on it
    bool keep = false;
    bool kalman = false;
    bool released = false;    // release requested: free once idle
    long long m = 0;          // Kalman observation size
    double *kf_buf = nullptr; // model (F, H, Qinv, Rinv, P0inv, x0), scratch, y
    double *kf_y = nullptr;
    KfScratch kf{};
    Clock::time_point last_use;
};

struct Request {
    uint64_t id = 0;
    int kind = RQ_SYSTEM;
    uint64_t factor_id = 0;
    long long N = 0, n = 0, k = 1, m = 0;
    const double *A = nullptr, *B = nullptr, *d = nullptr, *F = nullptr, *H = nullptr, *Qinv = nullptr,
                 *Rinv = nullptr, *P0inv = nullptr, *x0 = nullptr, *y = nullptr;
    double *x_out = nullptr;
    bool keep = false;
    int phase = PH_QUEUED;
    int status = BSS_OK;
    int refine = 0;
    double relres = -1.0;
    int ev = -1;    // event slot
    int stslot = -1;  // pinned status slot
    Factor *f = nullptr;
    Clock::time_point t_submit, t_start, t_done;
    bool reserved = false;  // RHS request holding a user count on its factor since submit
    bool finished = false;  // result ready (set under the server lock)
};

}  // namespace

struct bss_server {
    bss_server_options opt{};
    int device = 0;
    std::vector<cudaStream_t> streams;
    cudaMemPool_t pool = nullptr;
    std::vector<cudaEvent_t> events;
    std::vector<int> free_events;
    DevStatus *pinned = nullptr;  // one status per in-flight request
    std::vector<int> free_status;
    std::mutex mu;
    std::condition_variable cv_work, cv_done;
    std::deque<Request *> pending;
    std::vector<Request *> running;  // worker-private
    std::unordered_map<uint64_t, Request *> requests;
    std::unordered_map<uint64_t, Factor *> factors;
    size_t bytes_in_use = 0, bytes_peak = 0;
    uint64_t next_id = 1;
    int rr = 0;
    std::thread worker;
    bool stop = false;
    // statistics
    std::vector<double> lat_ms;
    long long submitted = 0, completed = 0, failed = 0, evictions = 0;
    Clock::time_point t_first, t_last;
    bool any = false;
    int worker_error = BSS_OK;
};

namespace {

void free_factor(bss_server *S, Factor *f)
{
    cudaStream_t st = S->streams[f->slot];
    if (f->h) {
        if (f->h->arena) cudaFreeAsync(f->h->arena, st);
        f->h->arena = nullptr;
        f->h->h_st = nullptr;
        delete f->h;
    }
    if (f->kf_buf) cudaFreeAsync(f->kf_buf, st);
    S->bytes_in_use -= f->bytes;
    S->factors.erase(f->id);
    delete f;
}

// evict idle resident factors, least recently used first, until `need` fits
bool make_room(bss_server *S, size_t need)
{
    while (S->bytes_in_use + need > (size_t)S->opt.hbm_budget_bytes) {
        Factor *victim = nullptr;
        for (auto &kv : S->factors) {
            Factor *f = kv.second;
            if (f->users == 0 && (!victim || f->last_use < victim->last_use)) victim = f;
        }
        if (!victim) return false;
        ++S->evictions;
        free_factor(S, victim);
    }
    return true;
}

size_t kf_model_doubles(long long n, long long m, long long k, long long N)
{
    return 3 * n * n + m * n + m * m + n + KfScratch::doubles(n, m) + m * k * N;
}

// plan a new factor for request r (host only); nullptr + status on failure
Factor *plan_factor(bss_server *S, Request *r)
{
    bss_handle *h = new bss_handle();
    bss_default_options(&h->opt);
    h->opt.precision = S->opt.precision;
    h->opt.max_refine = S->opt.max_refine;
    h->opt.tol = S->opt.tol;
    h->opt.use_graphs = 0;
    h->N_user = r->N;
    h->N = r->N;  // no padding
    h->n = r->n;
    h->k = r->k;
    h->dtype = F64;
    h->device = S->device;
    h->kc_max = solve_kc_max((int)r->n, (int)r->k, 8);
    plan_handle(h);
    h->arena_bytes = (h->arena_bytes + 255) & ~(size_t)255;
    Factor *f = new Factor();
    f->h = h;
    f->bytes = h->arena_bytes;
    f->kalman = r->kind == RQ_KALMAN;
    f->m = r->m;
    if (f->kalman) f->bytes += kf_model_doubles(r->n, r->m, r->k, r->N) * sizeof(double);
    f->keep = r->keep;
    f->id = r->id;
    return f;
}

// enqueue the first GPU work of a request on its factor's stream
int start_request(bss_server *S, Request *r)
{
    Factor *f = r->f;
    bss_handle *h = f->h;
    cudaStream_t st = S->streams[f->slot];
    const long long nn = r->n * r->n;
    h->h_st = S->pinned + r->stslot;
    h->ls = h->stream = st;
    if (r->kind != RQ_RHS) {
        BSS_CUDA(cudaMallocFromPoolAsync((void **)&h->arena, h->arena_bytes, S->pool, st));
        int rc = bind_handle(h, h->arena, false);
        if (rc) return rc;
        if (r->kind == RQ_SYSTEM) {
            BSS_CUDA(cudaMemcpyAsync(h->A, r->A, r->N * nn * sizeof(double), cudaMemcpyHostToDevice, st));
            if (r->N > 1)
                BSS_CUDA(cudaMemcpyAsync(h->B, r->B, (r->N - 1) * nn * sizeof(double), cudaMemcpyHostToDevice, st));
            BSS_CUDA(cudaMemcpyAsync(h->d, r->d, r->N * r->n * r->k * sizeof(double), cudaMemcpyHostToDevice, st));
        } else {
            const long long n = r->n, m = r->m;
            BSS_CUDA(cudaMallocFromPoolAsync((void **)&f->kf_buf, kf_model_doubles(n, m, r->k, r->N) * sizeof(double),
                                             S->pool, st));
            double *F = f->kf_buf, *H = F + n * n, *Qi = H + m * n, *Ri = Qi + n * n, *P0 = Ri + m * m,
                   *x0 = P0 + n * n, *scr = x0 + n;
            f->kf.carve(scr, n, m);
            f->kf_y = scr + KfScratch::doubles(n, m);
            BSS_CUDA(cudaMemcpyAsync(F, r->F, n * n * 8, cudaMemcpyHostToDevice, st));
            BSS_CUDA(cudaMemcpyAsync(H, r->H, m * n * 8, cudaMemcpyHostToDevice, st));
            BSS_CUDA(cudaMemcpyAsync(Qi, r->Qinv, n * n * 8, cudaMemcpyHostToDevice, st));
            BSS_CUDA(cudaMemcpyAsync(Ri, r->Rinv, m * m * 8, cudaMemcpyHostToDevice, st));
            if (r->P0inv) BSS_CUDA(cudaMemcpyAsync(P0, r->P0inv, n * n * 8, cudaMemcpyHostToDevice, st));
            if (r->x0) BSS_CUDA(cudaMemcpyAsync(x0, r->x0, n * 8, cudaMemcpyHostToDevice, st));
            BSS_CUDA(cudaMemcpyAsync(f->kf_y, r->y, m * r->k * r->N * 8, cudaMemcpyHostToDevice, st));
            BSS_CUDA(kf_launch_prepare(n, m, F, H, Qi, Ri, r->P0inv ? P0 : nullptr, r->x0 ? x0 : nullptr, f->kf, st));
            BSS_CUDA(kf_launch_fill(r->N, n, m, r->k, f->kf, f->kf_y, (double *)h->A, (double *)h->B,
                                    (double *)h->d, st));
        }
        int rc2 = bss_factorize(h);
        if (rc2) return rc2;
    } else if (f->kalman) {
        BSS_CUDA(cudaMemcpyAsync(f->kf_y, r->y, f->m * r->k * r->N * 8, cudaMemcpyHostToDevice, st));
        BSS_CUDA(kf_launch_fill(r->N, r->n, f->m, r->k, f->kf, f->kf_y, nullptr, nullptr, (double *)h->d, st));
    } else {
        BSS_CUDA(cudaMemcpyAsync(h->d, r->d, r->N * r->n * r->k * sizeof(double), cudaMemcpyHostToDevice, st));
    }
    h->ls = st;
    if (h->opt.precision == BSS_PRECISION_MIXED) {
        int rc = mixed_begin(h);
        if (rc) return rc;
        r->phase = PH_SOLVE;
    } else {
        int rc = bss_solve(h);
        if (rc) return rc;
        BSS_CUDA(cudaMemcpyAsync(h->h_st, h->st, sizeof(DevStatus), cudaMemcpyDeviceToHost, st));
        BSS_CUDA(cudaMemcpyAsync(r->x_out, h->d, r->N * r->n * r->k * sizeof(double), cudaMemcpyDeviceToHost, st));
        r->phase = PH_FINISH;
    }
    BSS_CUDA(cudaEventRecord(S->events[r->ev], st));
    return BSS_OK;
}

// a request's event completed: next phase (refinement step, finish) or done
int advance_request(bss_server *S, Request *r)
{
    Factor *f = r->f;
    bss_handle *h = f->h;
    cudaStream_t st = S->streams[f->slot];
    const DevStatus &hs = *h->h_st;
    if (hs.tc_timeout && r->kind != RQ_RHS) {
        r->status = BSS_ERR_TIMEOUT;
        r->phase = PH_DONE;
        return BSS_OK;
    }
    if (r->phase == PH_FINISH) {
        if (hs.bad_key != ~0ULL && r->kind != RQ_RHS) r->status = BSS_ERR_NOT_SPD;
        r->phase = PH_DONE;
        return BSS_OK;
    }
    // PH_SOLVE / PH_REFINE: the status holds the residual of the current x
    if (hs.bad_key != ~0ULL && r->kind != RQ_RHS) {
        r->status = BSS_ERR_NOT_SPD;
        r->phase = PH_DONE;
        return BSS_OK;
    }
    r->relres = hs.relres;
    h->ls = st;
    if (!hs.done && r->refine < S->opt.max_refine) {
        ++r->refine;
        int rc = mixed_correct(h);
        if (rc) return rc;
        r->phase = PH_REFINE;
    } else {
        if (!hs.done) r->status = BSS_ERR_NOT_CONVERGED;
        int rc = mixed_finish(h);
        if (rc) return rc;
        BSS_CUDA(cudaMemcpyAsync(r->x_out, h->d, r->N * r->n * r->k * sizeof(double), cudaMemcpyDeviceToHost, st));
        r->phase = PH_FINISH;
    }
    BSS_CUDA(cudaEventRecord(S->events[r->ev], st));
    return BSS_OK;
}

// under the lock: move admissible pending requests to `start`
void admit(bss_server *S, std::vector<Request *> &start)
{
    for (auto it = S->pending.begin(); it != S->pending.end();) {
        if ((int)(S->running.size() + start.size()) >= S->opt.max_inflight || S->free_events.empty() ||
            S->free_status.empty())
            break;
        Request *r = *it;
        if (r->kind == RQ_RHS) {
            auto fi = S->factors.find(r->factor_id);
            if (fi == S->factors.end()) {  // evicted, released or failed before it ran
                r->status = BSS_ERR_STATE;
                r->phase = PH_DONE;
                r->finished = true;
                r->t_start = r->t_done = Clock::now();
                ++S->failed;
                it = S->pending.erase(it);
                S->cv_done.notify_all();
                continue;
            }
            Factor *f = fi->second;
            if (!r->reserved) {
                f->users += 1;
                r->reserved = true;
            }
            bool busy = false;  // an earlier request on this factor is still on the GPU
            for (Request *q : S->running) busy |= q->f == f;
            for (Request *q : start) busy |= q->f == f;
            if (busy) {
                ++it;
                continue;
            }
            r->f = f;
        } else {
            Factor *f = plan_factor(S, r);
            if (f->bytes > (size_t)S->opt.hbm_budget_bytes) {
                r->status = BSS_ERR_OOM;
                r->phase = PH_DONE;
                r->finished = true;
                r->t_start = r->t_done = Clock::now();
                ++S->failed;
                delete f->h;
                delete f;
                it = S->pending.erase(it);
                S->cv_done.notify_all();
                continue;
            }
            if (!make_room(S, f->bytes)) {  // FIFO on memory: nothing behind overtakes
                delete f->h;
                delete f;
                break;
            }
            f->slot = S->rr++ % (int)S->streams.size();
            f->h->stream = S->streams[f->slot];
            S->bytes_in_use += f->bytes;
            S->bytes_peak = std::max(S->bytes_peak, S->bytes_in_use);
            S->factors[f->id] = f;
            f->users = 1;
            r->f = f;
        }
        r->ev = S->free_events.back();
        S->free_events.pop_back();
        r->stslot = S->free_status.back();
        S->free_status.pop_back();
        r->t_start = Clock::now();
        start.push_back(r);
        it = S->pending.erase(it);
    }
}

void worker_main(bss_server *S)
{
    cudaSetDevice(S->device);
    std::vector<Request *> start, finished;
    for (;;) {
        start.clear();
        finished.clear();
        {
            std::unique_lock<std::mutex> lk(S->mu);
            if (S->running.empty() && S->pending.empty()) {
                if (S->stop) break;
                S->cv_work.wait(lk, [&] { return S->stop || !S->pending.empty(); });
                if (S->stop && S->pending.empty()) break;
            }
            admit(S, start);
        }
        for (Request *r : start) {
            const int rc = start_request(S, r);
            if (rc != BSS_OK) {
                r->status = rc;
                r->phase = PH_DONE;
            }
            S->running.push_back(r);
        }
        bool progressed = !start.empty();
        for (size_t i = 0; i < S->running.size();) {
            Request *r = S->running[i];
            if (r->phase != PH_DONE) {
                const cudaError_t q = cudaEventQuery(S->events[r->ev]);
                if (q == cudaErrorNotReady) {
                    ++i;
                    continue;
                }
                progressed = true;
                const int rc = q == cudaSuccess ? advance_request(S, r) : cuda_fail(q, "request event");
                if (rc != BSS_OK) {
                    r->status = rc;
                    r->phase = PH_DONE;
                }
                if (r->phase != PH_DONE) {
                    ++i;
                    continue;
                }
            }
            r->t_done = Clock::now();
            finished.push_back(r);
            S->running[i] = S->running.back();
            S->running.pop_back();
        }
        if (!finished.empty()) {
            std::lock_guard<std::mutex> lk(S->mu);
            for (Request *r : finished) {
                Factor *f = r->f;
                r->factor_id = (f && (f->keep || r->kind == RQ_RHS)) ? f->id : 0;
                if (f) {
                    f->users -= 1;
                    f->last_use = r->t_done;
                    if (f->h) f->h->h_st = nullptr;
                    const bool bad = r->status != BSS_OK && r->status != BSS_ERR_NOT_CONVERGED && r->kind != RQ_RHS;
                    if (bad) f->released = true;  // a failed factorization is never reused
                    const bool drop = (!f->keep || f->released) && f->users == 0;
                    if (drop) free_factor(S, f);
                }
                S->free_events.push_back(r->ev);
                S->free_status.push_back(r->stslot);
                r->finished = true;
                if (r->status == BSS_OK || r->status == BSS_ERR_NOT_CONVERGED) {
                    ++S->completed;
                    S->lat_ms.push_back(std::chrono::duration<double, std::milli>(r->t_done - r->t_submit).count());
                } else {
                    ++S->failed;
                }
                S->t_last = r->t_done;
            }
            S->cv_done.notify_all();
        }
        if (!progressed) std::this_thread::sleep_for(std::chrono::microseconds(10));
    }
}

Request *new_request(bss_server *S)
{
    Request *r = new Request();
    r->id = S->next_id++;
    r->t_submit = Clock::now();
    if (!S->any) {
        S->any = true;
        S->t_first = r->t_submit;
    }
    ++S->submitted;
    S->requests[r->id] = r;
    return r;
}

}  // namespace

extern "C" void bss_server_default_options(bss_server_options *o)
{
    if (!o) return;
    std::memset(o, 0, sizeof(*o));
    o->hbm_budget_bytes = 100LL * 1000 * 1000 * 1000;
    o->streams = 8;
    o->max_inflight = 64;
    o->precision = BSS_PRECISION_MIXED;
    o->max_refine = 10;
    o->tol = 1e-12;
}

extern "C" int bss_server_create(const bss_server_options *opt, bss_server **out)
{
    if (!out) return fail(BSS_ERR_ARG, "out is NULL");
    *out = nullptr;
    bss_server *S = new bss_server();
    if (opt)
        S->opt = *opt;
    else
        bss_server_default_options(&S->opt);
    S->opt.streams = std::max(1, S->opt.streams);
    S->opt.max_inflight = std::max(1, S->opt.max_inflight);
    S->opt.max_refine = std::max(0, S->opt.max_refine);
    if (S->opt.hbm_budget_bytes <= 0 ||
        (S->opt.precision != BSS_PRECISION_MIXED && S->opt.precision != BSS_PRECISION_PLAIN)) {
        delete S;
        return fail(BSS_ERR_ARG, "bss_server_create: bad options");
    }
    cudaError_t e = cudaGetDevice(&S->device);
    for (int i = 0; e == cudaSuccess && i < S->opt.streams; ++i) {
        cudaStream_t st;
        e = cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking);
        if (e == cudaSuccess) S->streams.push_back(st);
    }
    if (e == cudaSuccess) {
        cudaMemPoolProps props{};
        props.allocType = cudaMemAllocationTypePinned;
        props.location.type = cudaMemLocationTypeDevice;
        props.location.id = S->device;
        e = cudaMemPoolCreate(&S->pool, &props);
        if (e == cudaSuccess) {
            unsigned long long thr = (unsigned long long)S->opt.hbm_budget_bytes;
            e = cudaMemPoolSetAttribute(S->pool, cudaMemPoolAttrReleaseThreshold, &thr);
        }
    }
    for (int i = 0; e == cudaSuccess && i < S->opt.max_inflight; ++i) {
        cudaEvent_t ev;
        e = cudaEventCreateWithFlags(&ev, cudaEventDisableTiming);
        if (e == cudaSuccess) {
            S->events.push_back(ev);
            S->free_events.push_back(i);
        }
    }
    if (e == cudaSuccess) e = cudaMallocHost((void **)&S->pinned, sizeof(DevStatus) * S->opt.max_inflight);
    if (e != cudaSuccess) {
        for (auto st : S->streams) cudaStreamDestroy(st);
        for (auto ev : S->events) cudaEventDestroy(ev);
        if (S->pool) cudaMemPoolDestroy(S->pool);
        delete S;
        return cuda_fail(e, "bss_server_create");
    }
    for (int i = S->opt.max_inflight - 1; i >= 0; --i) S->free_status.push_back(i);
    S->worker = std::thread(worker_main, S);
    *out = S;
    return BSS_OK;
}

extern "C" int bss_server_destroy(bss_server *S)
{
    if (!S) return BSS_OK;
    {
        std::lock_guard<std::mutex> lk(S->mu);
        S->stop = true;
    }
    S->cv_work.notify_all();
    if (S->worker.joinable()) S->worker.join();
    for (auto st : S->streams) cudaStreamSynchronize(st);
    std::vector<Factor *> fs;
    for (auto &kv : S->factors) fs.push_back(kv.second);
    for (Factor *f : fs) free_factor(S, f);
    for (auto st : S->streams) cudaStreamSynchronize(st);
    for (auto &kv : S->requests) delete kv.second;
    for (auto st : S->streams) cudaStreamDestroy(st);
    for (auto ev : S->events) cudaEventDestroy(ev);
    if (S->pool) cudaMemPoolDestroy(S->pool);
    if (S->pinned) cudaFreeHost(S->pinned);
    delete S;
    return BSS_OK;
}

static int check_shape(long long N, long long n, long long k)
{
    if (N < 1 || n < 1 || k < 1) return fail(BSS_ERR_ARG, "N, n and k must be >= 1");
    if (tile_for((int)n) == 0) return fail(BSS_ERR_UNSUPPORTED, "block size too large");
    if (residual_smem_bytes<double>((int)n, 1) > (size_t)200 * 1024)
        return fail(BSS_ERR_UNSUPPORTED, "the server supports n <= 128");
    return BSS_OK;
}

extern "C" int bss_server_submit(bss_server *S, int64_t N, int64_t n, int64_t k, const double *A, const double *B,
                                 const double *d, int32_t keep, double *x_out, uint64_t *request_id,
                                 uint64_t *factor_id)
{
    if (!S || !A || !d || !x_out || !request_id || (N > 1 && !B)) return fail(BSS_ERR_ARG, "bad argument");
    int rc = check_shape(N, n, k);
    if (rc) return rc;
    {
        std::lock_guard<std::mutex> lk(S->mu);
        Request *r = new_request(S);
        r->kind = RQ_SYSTEM;
        r->N = N;
        r->n = n;
        r->k = k;
        r->A = A;
        r->B = B;
        r->d = d;
        r->x_out = x_out;
        r->keep = keep != 0;
        S->pending.push_back(r);
        *request_id = r->id;
        if (factor_id) *factor_id = r->keep ? r->id : 0;
    }
    S->cv_work.notify_one();
    return BSS_OK;
}

extern "C" int bss_server_submit_kalman(bss_server *S, int64_t N, int64_t n, int64_t m, int64_t k, const double *F,
                                        const double *H, const double *Qinv, const double *Rinv, const double *P0inv,
                                        const double *x0, const double *y, int32_t keep, double *x_out,
                                        uint64_t *request_id, uint64_t *factor_id)
{
    if (!S || !F || !H || !Qinv || !Rinv || !y || !x_out || !request_id || m < 1)
        return fail(BSS_ERR_ARG, "bad argument");
    int rc = check_shape(N, n, k);
    if (rc) return rc;
    {
        std::lock_guard<std::mutex> lk(S->mu);
        Request *r = new_request(S);
        r->kind = RQ_KALMAN;
        r->N = N;
        r->n = n;
        r->m = m;
        r->k = k;
        r->F = F;
        r->H = H;
        r->Qinv = Qinv;
        r->Rinv = Rinv;
        r->P0inv = P0inv;
        r->x0 = x0;
        r->y = y;
        r->x_out = x_out;
        r->keep = keep != 0;
        S->pending.push_back(r);
        *request_id = r->id;
        if (factor_id) *factor_id = r->keep ? r->id : 0;
    }
    S->cv_work.notify_one();
    return BSS_OK;
}

extern "C" int bss_server_submit_rhs(bss_server *S, uint64_t factor_id, const double *d_or_y, double *x_out,
                                     uint64_t *request_id)
{
    if (!S || !d_or_y || !x_out || !request_id) return fail(BSS_ERR_ARG, "bad argument");
    {
        std::lock_guard<std::mutex> lk(S->mu);
        auto fi = S->factors.find(factor_id);
        // the factor may still be pending its first request: find its shape there
        const Request *src = nullptr;
        if (fi == S->factors.end()) {
            auto ri = S->requests.find(factor_id);
            if (ri == S->requests.end() || !ri->second->keep || ri->second->phase == PH_DONE)
                return fail(BSS_ERR_STATE, "no resident factor with this id");
            src = ri->second;
        }
        Request *r = new_request(S);
        r->kind = RQ_RHS;
        r->factor_id = factor_id;
        if (src) {
            r->N = src->N;
            r->n = src->n;
            r->k = src->k;
            r->m = src->m;
        } else {
            bss_handle *h = fi->second->h;
            r->N = h->N;
            r->n = h->n;
            r->k = h->k;
            r->m = fi->second->m;
            fi->second->users += 1;  // keeps it from eviction while queued
            r->reserved = true;
        }
        const bool kal = src ? src->kind == RQ_KALMAN : fi->second->kalman;
        if (kal)
            r->y = d_or_y;
        else
            r->d = d_or_y;
        r->x_out = x_out;
        S->pending.push_back(r);
        *request_id = r->id;
    }
    S->cv_work.notify_one();
    return BSS_OK;
}

extern "C" int bss_server_wait(bss_server *S, uint64_t request_id, bss_request_info *info)
{
    if (!S) return fail(BSS_ERR_ARG, "server is NULL");
    std::unique_lock<std::mutex> lk(S->mu);
    auto it = S->requests.find(request_id);
    if (it == S->requests.end()) return fail(BSS_ERR_ARG, "unknown or already collected request id");
    Request *r = it->second;
    S->cv_done.wait(lk, [&] { return r->finished; });
    if (info) {
        info->status = r->status;
        info->refine_steps = r->refine;
        info->rel_residual = r->relres;
        info->latency_ms = std::chrono::duration<double, std::milli>(r->t_done - r->t_submit).count();
        info->queue_ms = std::chrono::duration<double, std::milli>(r->t_start - r->t_submit).count();
        info->factor_id = r->factor_id;
    }
    const int st = r->status;
    S->requests.erase(it);
    delete r;
    if (st != BSS_OK) return fail(st, "request " + std::to_string(request_id) + " failed");
    return BSS_OK;
}

extern "C" int bss_server_poll(bss_server *S, uint64_t request_id, int32_t *done)
{
    if (!S || !done) return fail(BSS_ERR_ARG, "bad argument");
    std::lock_guard<std::mutex> lk(S->mu);
    auto it = S->requests.find(request_id);
    if (it == S->requests.end()) return fail(BSS_ERR_ARG, "unknown or already collected request id");
    *done = it->second->finished ? 1 : 0;
    return BSS_OK;
}

extern "C" int bss_server_release(bss_server *S, uint64_t factor_id)
{
    if (!S) return fail(BSS_ERR_ARG, "server is NULL");
    std::lock_guard<std::mutex> lk(S->mu);
    auto fi = S->factors.find(factor_id);
    if (fi != S->factors.end()) {
        Factor *f = fi->second;
        f->released = true;
        if (f->users == 0) free_factor(S, f);
        return BSS_OK;
    }
    for (Request *r : S->pending)  // not admitted yet: do not keep it
        if (r->id == factor_id) {
            r->keep = false;
            return BSS_OK;
        }
    return fail(BSS_ERR_STATE, "no resident factor with this id");
}

extern "C" int bss_server_get_stats(bss_server *S, bss_server_stats *st)
{
    if (!S || !st) return fail(BSS_ERR_ARG, "bad argument");
    std::lock_guard<std::mutex> lk(S->mu);
    std::memset(st, 0, sizeof(*st));
    st->submitted = S->submitted;
    st->completed = S->completed;
    st->failed = S->failed;
    st->evictions = S->evictions;
    long long res = 0;
    for (auto &kv : S->factors) res += kv.second->keep ? 1 : 0;
    st->resident_factors = res;
    st->bytes_in_use = (int64_t)S->bytes_in_use;
    st->bytes_peak = (int64_t)S->bytes_peak;
    if (!S->lat_ms.empty()) {
        std::vector<double> v = S->lat_ms;
        std::sort(v.begin(), v.end());
        auto pct = [&](double q) {
            const double pos = q * (double)(v.size() - 1);
            const size_t lo = (size_t)pos;
            const size_t hi = std::min(lo + 1, v.size() - 1);
            return v[lo] + (pos - (double)lo) * (v[hi] - v[lo]);
        };
        st->p50_ms = pct(0.50);
        st->p99_ms = pct(0.99);
        double sum = 0.0;
        for (double x : v) sum += x;
        st->mean_ms = sum / (double)v.size();
        st->max_ms = v.back();
        st->busy_s = std::chrono::duration<double>(S->t_last - S->t_first).count();
    }
    return BSS_OK;
}

extern "C" int bss_server_reset_stats(bss_server *S)
{
    if (!S) return fail(BSS_ERR_ARG, "server is NULL");
    std::lock_guard<std::mutex> lk(S->mu);
    S->lat_ms.clear();
    S->submitted = S->completed = S->failed = S->evictions = 0;
    S->any = false;
    S->bytes_peak = S->bytes_in_use;
    return BSS_OK;
}
