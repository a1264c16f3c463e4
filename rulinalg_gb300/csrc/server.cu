// The serving loop: a request queue in front of the GPU solvers with continuous
// batching, device-resident factors and admission by device-memory footprint.
//
// Clients submit requests (LU solve, Cholesky solve, QR least squares, or a re-solve
// against a resident factor) and wait for tickets. Worker threads, each owning a CUDA
// stream, pull work whenever they are free: all admitted small LU/Cholesky requests
// (n <= small_n, up to max_batch) go out together as one batched mixed-precision launch,
// anything else runs alone. Requests that arrive while others are on the GPU join the
// next launch, and the workers' streams overlap on the device. A request is admitted only
// when its device-memory footprint fits in the budget next to everything in flight and
// every resident factor; the oldest waiting request is never bypassed for longer than
// kMaxBypassUs.
#include <algorithm>
#include <chrono>
#include <condition_variable>
#include <deque>
#include <memory>
#include <mutex>
#include <numeric>
#include <thread>
#include <unordered_map>
#include <vector>

#include "mixed_ops.cuh"

using namespace rl;

namespace {

constexpr double kMaxBypassUs = 20000.0;

double now_us() {
    using namespace std::chrono;
    return duration<double, std::micro>(steady_clock::now().time_since_epoch()).count();
}

struct Req {
    uint64_t id = 0;
    rl_request r{};
    rl_result res{};
    double t_submit = 0, t_start = 0, t_done = 0;
    size_t bytes = 0;
    bool done = false;
    bool batchable = false;
};

struct Resident {
    std::unique_ptr<MixedFactor> f;
    std::mutex mu;  // solves against one factor are serialised (the FP64 fallback is built lazily)
    size_t bytes = 0;
    bool released = false;  // set under mu by rl_server_release_factor; a queued re-solve then fails
};

}  // namespace

struct rl_server {
    rl_server_config cfg{};
    size_t budget = 0;
    std::mutex mu;
    std::condition_variable cv_work, cv_done;
    std::deque<Req *> pending;  // submitted, not admitted yet
    std::deque<Req *> ready;    // admitted, waiting for a worker
    std::unordered_map<uint64_t, Req *> reqs;
    std::unordered_map<uint64_t, std::shared_ptr<Resident>> factors;
    size_t bytes_in_use = 0, bytes_peak = 0;
    uint64_t next_id = 1, next_factor = 1;
    bool stop = false;
    std::vector<std::thread> workers;
    void *worker_state = nullptr;            // std::vector<Worker>
    void (*free_workers)(void *) = nullptr;  // destroys it (streams, slots)
    // statistics
    std::vector<double> lat_us;
    uint64_t submitted = 0, completed = 0, failed = 0, batches = 0, batched = 0, rejected = 0;
    size_t in_server = 0;  // submitted and not finished (the backpressure count)
    double t_first = -1, t_last = 0;
};

namespace {

size_t footprint(const rl_request &r) {
    const size_t n = r.n, m = r.m ? r.m : r.n;
    switch (r.kind) {
        case RL_REQ_RESOLVE: return 32 * n + 4096;
        // A (f64), its FP32 QR, R^T, panel buffers, vectors, and the FP64 [A | b] of the fallback
        case RL_REQ_LSTSQ: return 8 * m * n + 4 * m * n + 4 * n * n + 8 * m * 64 + 64 * n * 16 + 8 * m * (n + 2) + 4096;
        default: return 8 * n * n + 4 * n * n + 48 * n + 4096;  // A (f64), FP32 factor, vectors
    }
}

bool is_batchable(const rl_server &s, const rl_request &r) {
    return (r.kind == RL_REQ_LU || r.kind == RL_REQ_CHOLESKY) && !r.retain && r.n <= (size_t)s.cfg.small_n &&
           r.n <= (size_t)CTA_NMAX;
}

// Moves pending requests to ready while they fit (lock held). FIFO, except that a request
// that does not fit may be passed by later ones for at most kMaxBypassUs.
void admit(rl_server &s) {
    const double t = now_us();
    for (auto it = s.pending.begin(); it != s.pending.end();) {
        Req *q = *it;
        if (s.bytes_in_use + q->bytes <= s.budget) {
            s.bytes_in_use += q->bytes;
            s.bytes_peak = std::max(s.bytes_peak, s.bytes_in_use);
            s.ready.push_back(q);
            it = s.pending.erase(it);
            continue;
        }
        if (it == s.pending.begin() && t - q->t_submit > kMaxBypassUs) break;  // hold memory for the oldest
        ++it;
    }
}

void finish(rl_server &s, Req *q, rl_status st) {
    q->res.status = st;
    q->t_done = now_us();
    q->res.queue_us = q->t_start - q->t_submit;
    q->res.latency_us = q->t_done - q->t_submit;
    q->done = true;
    s.in_server--;
    s.lat_us.push_back(q->res.latency_us);
    s.completed++;
    if (st != RL_OK) s.failed++;
    s.t_last = std::max(s.t_last, q->t_done);
}

// ------------------------------------------------------------------ worker jobs --
struct Worker {
    rl_server *s = nullptr;
    int index = 0;
    cudaStream_t stream = nullptr;
    void *work32 = nullptr, *work64 = nullptr;  // batched-kernel slots
    int grid32 = 0, grid64 = 0;
    size_t smem32 = 0, smem64 = 0;
    long long slot = (long long)CTA_NMAX * CTA_NMAX;

    rl_status init() {
        RL_TRY_CUDA(cudaStreamCreateWithFlags(&stream, cudaStreamNonBlocking));
        smem32 = cta_smem_bytes<float>();
        smem64 = cta_smem_bytes<double>();
        auto k32 = batch_solve_kernel<double, float, true>;
        auto k64 = batch_solve_kernel<double, double, false>;
        RL_TRY_CUDA(cudaFuncSetAttribute(k32, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem32));
        RL_TRY_CUDA(cudaFuncSetAttribute(k64, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem64));
        int p32 = 0, p64 = 0;
        RL_TRY_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&p32, k32, CTA_THREADS, smem32));
        RL_TRY_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&p64, k64, CTA_THREADS, smem64));
        grid32 = std::max(1, p32) * num_sms();
        grid64 = std::max(1, p64) * num_sms() / 4 + 1;  // fallbacks are rare
        RL_TRY_CUDA(cudaMalloc(&work32, grid32 * slot * sizeof(float)));
        RL_TRY_CUDA(cudaMalloc(&work64, grid64 * slot * sizeof(double)));
        return RL_OK;
    }
    void destroy() {
        if (work32) cudaFree(work32);
        if (work64) cudaFree(work64);
        if (stream) cudaStreamDestroy(stream);
    }

    // Several small systems in one batched mixed-precision launch.
    rl_status run_batch(std::vector<Req *> &job) {
        NvtxRange nvtx_("rl.server.batch");
        cudaStream_t st = stream;
        const int B = (int)job.size();
        std::vector<int> n(B), order(B);
        std::vector<uint8_t> kind(B);
        std::vector<long long> aoff(B), boff(B);
        long long at = 0, bt = 0;
        for (int i = 0; i < B; i++) {
            n[i] = (int)job[i]->r.n;
            kind[i] = job[i]->r.kind == RL_REQ_CHOLESKY ? 1 : 0;
            aoff[i] = at;
            boff[i] = bt;
            at += (long long)n[i] * n[i];
            bt += n[i];
        }
        std::iota(order.begin(), order.end(), 0);
        std::stable_sort(order.begin(), order.end(), [&](int x, int y) {
            return (double)n[x] * n[x] * n[x] * (kind[x] ? 1 : 2) > (double)n[y] * n[y] * n[y] * (kind[y] ? 1 : 2);
        });
        DevBuf<double> dA, dB, dX, dberr;
        DevBuf<int> dn, dorder, dinfo, diters, dcnt, dfb;
        DevBuf<uint8_t> dkind;
        DevBuf<long long> daoff, dboff;
        RL_TRY(dA.alloc(std::max(1LL, at), st));
        RL_TRY(dB.alloc(std::max(1LL, bt), st));
        RL_TRY(dX.alloc(std::max(1LL, bt), st));
        RL_TRY(dberr.alloc(B, st));
        RL_TRY(dn.alloc(B, st));
        RL_TRY(dorder.alloc(B, st));
        RL_TRY(dinfo.alloc(B, st));
        RL_TRY(diters.alloc(B, st));
        RL_TRY(dcnt.alloc(4, st));
        RL_TRY(dfb.alloc(B, st));
        RL_TRY(dkind.alloc(B, st));
        RL_TRY(daoff.alloc(B, st));
        RL_TRY(dboff.alloc(B, st));
        for (int i = 0; i < B; i++) {
            const rl_request &r = job[i]->r;
            RL_TRY_CUDA(cudaMemcpyAsync(dA.p + aoff[i], r.a, (size_t)n[i] * n[i] * sizeof(double),
                                        cudaMemcpyHostToDevice, st));
            RL_TRY_CUDA(cudaMemcpyAsync(dB.p + boff[i], r.b, (size_t)n[i] * sizeof(double), cudaMemcpyHostToDevice, st));
        }
        RL_TRY_CUDA(cudaMemcpyAsync(dn.p, n.data(), B * sizeof(int), cudaMemcpyHostToDevice, st));
        RL_TRY_CUDA(cudaMemcpyAsync(dorder.p, order.data(), B * sizeof(int), cudaMemcpyHostToDevice, st));
        RL_TRY_CUDA(cudaMemcpyAsync(dkind.p, kind.data(), B, cudaMemcpyHostToDevice, st));
        RL_TRY_CUDA(cudaMemcpyAsync(daoff.p, aoff.data(), B * sizeof(long long), cudaMemcpyHostToDevice, st));
        RL_TRY_CUDA(cudaMemcpyAsync(dboff.p, boff.data(), B * sizeof(long long), cudaMemcpyHostToDevice, st));
        RL_TRY_CUDA(cudaMemsetAsync(dcnt.p, 0, 4 * sizeof(int), st));
        BatchDesc d{};
        d.count = B;
        d.order = dorder.p;
        d.n = dn.p;
        d.kind = dkind.p;
        d.a_off = daoff.p;
        d.b_off = dboff.p;
        d.next = dcnt.p;
        d.fb_list = dfb.p;
        d.fb_count = dcnt.p + 1;
        d.work = work32;
        d.work_stride = slot;
        d.info = dinfo.p;
        d.iters = diters.p;
        d.berr = dberr.p;
        d.iters_tag = 0;
        d.max_iters = 30;
        d.warp_small = 1;  // the order is largest-cost first
    d.warp_cost = (int)tune(RL_TUNE_BATCH_WARP_COST);
    d.wait_ns = wait_ns();
        RL_LAUNCH((batch_solve_kernel<double, float, true>), std::min(grid32, B), CTA_THREADS, smem32, st, d, dA.p,
                  dB.p, dX.p);
        BatchDesc f = d;
        f.count = 0;
        f.count_dev = dcnt.p + 1;
        f.order = dfb.p;
        f.next = dcnt.p + 2;
        f.work = work64;
        f.iters_tag = -1;
        f.warp_small = 0;  // the fallback list is in arrival order
        RL_LAUNCH((batch_solve_kernel<double, double, false>), std::min(grid64, B), CTA_THREADS, smem64, st, f, dA.p,
                  dB.p, dX.p);
        std::vector<int> info(B), iters(B);
        std::vector<double> berr(B);
        for (int i = 0; i < B; i++)
            RL_TRY_CUDA(cudaMemcpyAsync(job[i]->r.x, dX.p + boff[i], (size_t)n[i] * sizeof(double),
                                        cudaMemcpyDeviceToHost, st));
        RL_TRY_CUDA(cudaMemcpyAsync(info.data(), dinfo.p, B * sizeof(int), cudaMemcpyDeviceToHost, st));
        RL_TRY_CUDA(cudaMemcpyAsync(iters.data(), diters.p, B * sizeof(int), cudaMemcpyDeviceToHost, st));
        RL_TRY_CUDA(cudaMemcpyAsync(berr.data(), dberr.p, B * sizeof(double), cudaMemcpyDeviceToHost, st));
        RL_TRY_CUDA(cudaStreamSynchronize(st));
        for (int i = 0; i < B; i++) {
            job[i]->res.status = info[i];
            job[i]->res.iters = iters[i] < 0 ? 0 : iters[i];
            job[i]->res.path = iters[i] < 0 ? RL_PATH_FP64 : RL_PATH_REFINEMENT;
            job[i]->res.berr = berr[i];
        }
        return RL_OK;
    }

    // One LU / Cholesky system through a mixed-precision factor (kept resident on retain).
    rl_status run_single(Req *q) {
        cudaStream_t st = stream;
        const rl_request &r = q->r;
        const int n = (int)r.n;
        double *dA = nullptr;
        RL_TRY_CUDA(cudaMallocAsync(reinterpret_cast<void **>(&dA), std::max<size_t>(1, (size_t)n * n) * sizeof(double), st));
        auto mf = std::make_unique<MixedFactor>();
        RL_TRY_CUDA(cudaMemcpyAsync(dA, r.a, (size_t)n * n * sizeof(double), cudaMemcpyHostToDevice, st));
        RL_TRY(mf->factor(dA, n, n, r.kind == RL_REQ_CHOLESKY ? RL_KIND_CHOLESKY : RL_KIND_LU, false, st, true));
        RL_TRY(solve_with(*mf, q));
        if (r.retain) {
            auto res = std::make_shared<Resident>();
            res->bytes = mf->bytes();
            res->f = std::move(mf);
            std::lock_guard<std::mutex> lk(s->mu);
            const uint64_t h = s->next_factor++;
            s->factors[h] = res;
            q->res.factor = h;
            // the factor keeps its memory: move it from the request to the resident set
            const size_t keep = std::min(q->bytes, res->bytes);
            q->bytes -= keep;
        }
        return RL_OK;
    }

    rl_status solve_with(MixedFactor &mf, Req *q) {
        cudaStream_t st = stream;
        const int n = mf.n;
        DevBuf<double> db, dx;
        RL_TRY(db.alloc(std::max(1, n), st));
        RL_TRY(dx.alloc(std::max(1, n), st));
        RL_TRY_CUDA(cudaMemcpyAsync(db.p, q->r.b, (size_t)n * sizeof(double), cudaMemcpyHostToDevice, st));
        SolveOut o;
        RL_TRY(mf.solve(db.p, 1, dx.p, 1, 1, o, st));
        RL_TRY_CUDA(cudaMemcpyAsync(q->r.x, dx.p, (size_t)n * sizeof(double), cudaMemcpyDeviceToHost, st));
        RL_TRY_CUDA(cudaStreamSynchronize(st));
        q->res.iters = o.iters;
        q->res.path = o.path;
        q->res.berr = o.berr;
        return RL_OK;
    }

    rl_status run_resolve(Req *q) {
        NvtxRange nvtx_("rl.server.resolve");
        std::shared_ptr<Resident> res;
        {
            std::lock_guard<std::mutex> lk(s->mu);
            auto it = s->factors.find(q->r.factor);
            if (it == s->factors.end()) return RL_ERR_INVALID_ARG;
            res = it->second;
        }
        std::lock_guard<std::mutex> lk(res->mu);
        // released between the lookup and this lock: its device buffers are gone
        if (res->released) return RL_ERR_INVALID_ARG;
        if (q->r.n != (size_t)res->f->n) return RL_ERR_SHAPE;
        q->res.factor = q->r.factor;
        return solve_with(*res->f, q);
    }

    // min ||A x - b|| (m >= n) through the mixed-precision least-squares solver (FP32
    // QR, FP64 semi-normal-equation refinement, FP64 QR fallback).
    rl_status run_lstsq(Req *q) {
        NvtxRange nvtx_("rl.server.lstsq");
        cudaStream_t st = stream;
        const rl_request &r = q->r;
        const int m = (int)r.m, n = (int)r.n;
        if (m < n) return RL_ERR_SHAPE;
        DevBuf<double> dA, db, dx;
        RL_TRY(dA.alloc((size_t)m * n, st));
        RL_TRY(db.alloc(m, st));
        RL_TRY(dx.alloc(n, st));
        RL_TRY_CUDA(cudaMemcpyAsync(dA.p, r.a, (size_t)m * n * sizeof(double), cudaMemcpyHostToDevice, st));
        RL_TRY_CUDA(cudaMemcpyAsync(db.p, r.b, (size_t)m * sizeof(double), cudaMemcpyHostToDevice, st));
        SolveOut o;
        RL_TRY(lstsq_mixed(dA.p, n, m, n, db.p, dx.p, o, st));
        RL_TRY_CUDA(cudaMemcpyAsync(r.x, dx.p, (size_t)n * sizeof(double), cudaMemcpyDeviceToHost, st));
        RL_TRY_CUDA(cudaStreamSynchronize(st));
        q->res.iters = o.iters;
        q->res.path = o.path;
        q->res.berr = o.berr;
        return RL_OK;
    }

    // Worker 0 is the fast lane: it takes batchable (small) requests, then re-solves
    // against resident factors, never a large factorisation, so cheap requests do not
    // queue behind one. The other workers take re-solves first (cheap), then the oldest
    // large request, then batchable ones when nothing else waits.
    bool fast_lane() const { return index == 0 && s->cfg.workers > 1; }
    bool has_work() const {
        if (!fast_lane()) return !s->ready.empty();
        for (const Req *q : s->ready)
            if (q->batchable || q->r.kind == RL_REQ_RESOLVE) return true;
        return false;
    }
    // Removes and returns the first ready request matching `pred`, or nullptr.
    template <class Pred>
    Req *take_first(Pred pred) {
        for (auto it = s->ready.begin(); it != s->ready.end(); ++it)
            if (pred(*it)) {
                Req *q = *it;
                s->ready.erase(it);
                return q;
            }
        return nullptr;
    }

    void loop() {
        g_shared_gpu = true;  // this thread's solves run next to the other workers'
        for (;;) {
            std::vector<Req *> job;
            {
                std::unique_lock<std::mutex> lk(s->mu);
                s->cv_work.wait(lk, [&] { return s->stop || has_work(); });
                if (s->stop && !has_work()) return;
                auto is_resolve = [](const Req *q) { return q->r.kind == RL_REQ_RESOLVE; };
                Req *head = nullptr;
                if (fast_lane()) {
                    bool any_batchable = false;
                    for (const Req *q : s->ready) any_batchable |= q->batchable;
                    if (!any_batchable) head = take_first(is_resolve);
                } else {
                    head = take_first(is_resolve);
                    if (!head) head = take_first([](const Req *q) { return !q->batchable; });
                }
                if (head) {
                    job.push_back(head);
                } else {
                    for (auto it = s->ready.begin(); it != s->ready.end() && (int)job.size() < s->cfg.max_batch;) {
                        if ((*it)->batchable) {
                            job.push_back(*it);
                            it = s->ready.erase(it);
                        } else {
                            ++it;
                        }
                    }
                    head = job.front();
                }
                const double t = now_us();
                for (Req *q : job) q->t_start = t;
                if (job.size() > 1 || head->batchable) {
                    s->batches++;
                    s->batched += job.size();
                }
            }
            rl_status st = RL_OK;
            if (job.size() > 1 || job[0]->batchable)
                st = run_batch(job);
            else if (job[0]->r.kind == RL_REQ_RESOLVE)
                st = run_resolve(job[0]);
            else if (job[0]->r.kind == RL_REQ_LSTSQ)
                st = run_lstsq(job[0]);
            else
                st = run_single(job[0]);
            std::lock_guard<std::mutex> lk(s->mu);
            for (Req *q : job) {
                s->bytes_in_use -= q->bytes;
                finish(*s, q, st != RL_OK ? st : q->res.status);
            }
            admit(*s);
            s->cv_done.notify_all();
            s->cv_work.notify_all();
        }
    }
};

}  // namespace

extern "C" {

rl_status rl_server_create(const rl_server_config *cfg, rl_server **out) {
    if (!out) return RL_ERR_INVALID_ARG;
    *out = nullptr;
    RL_TRY(ensure_device());
    auto *s = new rl_server();
    if (cfg) s->cfg = *cfg;
    if (s->cfg.workers <= 0) s->cfg.workers = 8;
    if (s->cfg.max_batch <= 0) s->cfg.max_batch = 4096;
    if (s->cfg.small_n <= 0 || s->cfg.small_n > CTA_NMAX) s->cfg.small_n = CTA_NMAX;
    size_t free_b = 0, total_b = 0;
    if (cudaMemGetInfo(&free_b, &total_b) != cudaSuccess) {
        delete s;
        return RL_ERR_CUDA;
    }
    std::vector<Worker> *ws = new std::vector<Worker>(s->cfg.workers);
    for (size_t i = 0; i < ws->size(); i++) {
        Worker &w = (*ws)[i];
        w.s = s;
        w.index = (int)i;
        rl_status st = w.init();
        if (st != RL_OK) {
            for (auto &x : *ws) x.destroy();
            delete ws;
            delete s;
            return st;
        }
    }
    size_t free_after = 0;
    cudaMemGetInfo(&free_after, &total_b);
    const size_t cap = (size_t)(0.8 * (double)free_after);
    s->budget = s->cfg.hbm_budget_bytes ? std::min(s->cfg.hbm_budget_bytes, cap) : cap;
    s->worker_state = ws;
    s->free_workers = [](void *p) {
        auto *v = static_cast<std::vector<Worker> *>(p);
        for (auto &w : *v) w.destroy();
        delete v;
    };
    for (auto &w : *ws) s->workers.emplace_back([&w] { w.loop(); });
    *out = s;
    return RL_OK;
}

rl_status rl_server_submit(rl_server *s, const rl_request *req, uint64_t *ticket) {
    if (!s || !req || !ticket) return RL_ERR_INVALID_ARG;
    const rl_request &r = *req;
    if (r.kind < RL_REQ_LU || r.kind > RL_REQ_RESOLVE) return RL_ERR_INVALID_ARG;
    if (!r.b || !r.x || (r.kind != RL_REQ_RESOLVE && !r.a)) return RL_ERR_INVALID_ARG;
    if (r.n == 0 || r.n > (size_t)INT32_MAX || (r.kind == RL_REQ_LSTSQ && (r.m < r.n || r.m > (size_t)INT32_MAX)))
        return RL_ERR_SHAPE;
    auto *q = new Req();
    q->r = r;
    if (q->r.m == 0) q->r.m = q->r.n;
    q->bytes = footprint(q->r);
    std::lock_guard<std::mutex> lk(s->mu);
    if (q->bytes > s->budget) {
        delete q;
        return RL_ERR_OUT_OF_MEMORY;  // can never be admitted
    }
    if (r.kind == RL_REQ_RESOLVE && !s->factors.count(r.factor)) {
        delete q;
        return RL_ERR_INVALID_ARG;
    }
    if (s->cfg.max_pending > 0 && s->in_server >= (size_t)s->cfg.max_pending) {
        delete q;
        s->rejected++;
        return RL_ERR_BUSY;
    }
    s->in_server++;
    q->batchable = is_batchable(*s, q->r);
    q->id = s->next_id++;
    q->t_submit = now_us();
    if (s->t_first < 0) s->t_first = q->t_submit;
    s->submitted++;
    s->reqs[q->id] = q;
    s->pending.push_back(q);
    admit(*s);
    s->cv_work.notify_all();
    *ticket = q->id;
    return RL_OK;
}

rl_status rl_server_wait(rl_server *s, uint64_t ticket, double timeout_s, rl_result *res) {
    if (!s || !res) return RL_ERR_INVALID_ARG;
    std::unique_lock<std::mutex> lk(s->mu);
    auto it = s->reqs.find(ticket);
    if (it == s->reqs.end()) return RL_ERR_INVALID_ARG;
    Req *q = it->second;
    const bool ok = timeout_s < 0 ? (s->cv_done.wait(lk, [&] { return q->done; }), true)
                                  : s->cv_done.wait_for(lk, std::chrono::duration<double>(timeout_s),
                                                        [&] { return q->done; });
    if (!ok) return RL_ERR_TIMEOUT;
    *res = q->res;
    s->reqs.erase(it);
    delete q;
    return RL_OK;
}

rl_status rl_server_release_factor(rl_server *s, uint64_t factor) {
    if (!s) return RL_ERR_INVALID_ARG;
    std::shared_ptr<Resident> res;
    {
        std::lock_guard<std::mutex> lk(s->mu);
        auto it = s->factors.find(factor);
        if (it == s->factors.end()) return RL_ERR_INVALID_ARG;
        res = it->second;
        s->factors.erase(it);
    }
    {
        std::lock_guard<std::mutex> lk(res->mu);  // no solve in flight on it any more
        cudaStreamSynchronize(res->f->home);
        res->f->release();
        res->released = true;
    }
    std::lock_guard<std::mutex> lk(s->mu);
    s->bytes_in_use -= std::min(s->bytes_in_use, res->bytes);
    admit(*s);
    s->cv_work.notify_all();
    return RL_OK;
}

rl_status rl_server_stats_get(rl_server *s, rl_server_stats *st) {
    if (!s || !st) return RL_ERR_INVALID_ARG;
    std::lock_guard<std::mutex> lk(s->mu);
    *st = rl_server_stats{};
    st->submitted = s->submitted;
    st->completed = s->completed;
    st->failed = s->failed;
    st->batches = s->batches;
    st->batched_requests = s->batched;
    st->rejected = s->rejected;
    st->bytes_in_use = s->bytes_in_use;
    st->bytes_peak = s->bytes_peak;
    st->bytes_budget = s->budget;
    st->resident_factors = s->factors.size();
    if (!s->lat_us.empty()) {
        std::vector<double> v = s->lat_us;
        std::sort(v.begin(), v.end());
        auto pct = [&](double p) { return v[std::min(v.size() - 1, (size_t)(p * (v.size() - 1) + 0.5))]; };
        st->p50_us = pct(0.50);
        st->p99_us = pct(0.99);
        st->mean_us = std::accumulate(v.begin(), v.end(), 0.0) / v.size();
        const double span = s->t_last - s->t_first;
        st->solves_per_s = span > 0 ? (double)s->completed / (span * 1e-6) : 0.0;
    }
    return RL_OK;
}

rl_status rl_server_reset_stats(rl_server *s) {
    if (!s) return RL_ERR_INVALID_ARG;
    std::lock_guard<std::mutex> lk(s->mu);
    s->lat_us.clear();
    s->submitted = s->completed = s->failed = s->batches = s->batched = s->rejected = 0;
    s->t_first = -1;
    s->t_last = 0;
    s->bytes_peak = s->bytes_in_use;
    return RL_OK;
}

rl_status rl_server_replay(rl_server *s, size_t count, const double *arrival_s, const rl_request *reqs,
                           rl_result *results) {
    if (!s || (count && (!arrival_s || !reqs || !results))) return RL_ERR_INVALID_ARG;
    std::vector<uint64_t> tickets(count, 0);
    std::vector<rl_status> sub(count, RL_OK);
    const auto t0 = std::chrono::steady_clock::now();
    for (size_t i = 0; i < count; i++) {
        std::this_thread::sleep_until(t0 + std::chrono::duration_cast<std::chrono::steady_clock::duration>(
                                               std::chrono::duration<double>(arrival_s[i])));
        sub[i] = rl_server_submit(s, &reqs[i], &tickets[i]);
    }
    for (size_t i = 0; i < count; i++) {
        if (sub[i] != RL_OK) {
            results[i] = rl_result{};
            results[i].status = sub[i];
            continue;
        }
        RL_TRY(rl_server_wait(s, tickets[i], -1.0, &results[i]));
    }
    return RL_OK;
}

rl_status rl_server_destroy(rl_server *s) {
    if (!s) return RL_OK;
    {
        std::lock_guard<std::mutex> lk(s->mu);
        s->stop = true;
    }
    s->cv_work.notify_all();
    for (auto &t : s->workers) t.join();  // the workers drain the admitted requests first
    for (auto &kv : s->reqs) delete kv.second;
    for (auto &kv : s->factors) {
        cudaStreamSynchronize(kv.second->f->home);
        kv.second->f->release();  // while the worker streams still exist
    }
    s->factors.clear();
    cudaDeviceSynchronize();
    if (s->free_workers) s->free_workers(s->worker_state);
    delete s;
    return RL_OK;
}

}  // extern "C"
