// Batched solves: the plan object (sizes, packed layout, largest-first schedule,
// per-CTA workspace slots, captured CUDA graph) and its C entry points.
#include <algorithm>
#include <mutex>
#include <numeric>
#include <type_traits>
#include <vector>

#include "batch.cuh"

using namespace rl;

struct rl_batch_plan {
    int precision = RL_PREC_MIXED;
    size_t count = 0;
    int max_n = 0;
    std::vector<int> n;
    std::vector<uint8_t> kind;
    std::vector<long long> a_off, b_off;
    long long a_total = 0, b_total = 0;

    int *d_n = nullptr, *d_order = nullptr, *d_counters = nullptr, *d_fb_list = nullptr;
    uint8_t *d_kind = nullptr;
    long long *d_aoff = nullptr, *d_boff = nullptr;
    void *d_work = nullptr;   // factor-type slots of the main pass
    double *d_work64 = nullptr;  // FP64 slots of the fallback pass (mixed)
    long long work_stride = 0;
    int grid = 0, grid64 = 0;
    size_t smem = 0, smem64 = 0;

    cudaStream_t cap = nullptr;
    cudaGraphExec_t exec = nullptr;
    const void *key[6] = {};

    // device copies used by the host-pointer entry points
    void *h_a = nullptr, *h_b = nullptr, *h_x = nullptr;
    int *h_info = nullptr, *h_iters = nullptr;
    double *h_berr = nullptr;
    // host-pointer pipeline: contiguous chunks of systems copied one after another on the
    // copy stream while ONE launch solves them in chunk order (largest-first within each
    // chunk), each CTA waiting on the chunk's arrival flag. In the device copies every
    // chunk starts on a 256-byte boundary (a_shift / b_shift elements added to the
    // offsets), so no cache sector holds bytes of two chunks: an SM that read the end of
    // chunk c - 1 cannot have cached bytes of chunk c before they arrived.
    std::vector<int> chunk_first, chunk_count;
    std::vector<long long> a_shift, b_shift;
    long long a_total_h = 0, b_total_h = 0;
    int *d_corder = nullptr, *d_ccounters = nullptr, *d_gate = nullptr, *d_gate_pos = nullptr;
    long long *d_aoff_h = nullptr, *d_boff_h = nullptr;
    int *h_one = nullptr;  // pinned host 1, copied into d_gate[c] after chunk c
    cudaStream_t copy = nullptr;
    cudaEvent_t ev_start = nullptr;

    std::mutex mu;
};

namespace {

template <class TI, class TF, bool MIXED>
rl_status occupancy_grid(size_t smem, int &grid) {
    auto kern = batch_solve_kernel<TI, TF, MIXED>;
    RL_TRY_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    int per_sm = 0;
    RL_TRY_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, CTA_THREADS, smem));
    if (per_sm < 1) return RL_ERR_CUDA;
    const int64_t want = tune(RL_TUNE_BATCH_CTAS_PER_SM);  // 0: as many as fit
    if (want > 0 && want < per_sm) per_sm = (int)want;
    grid = per_sm * num_sms();
    return RL_OK;
}

template <class TI, class TF, bool MIXED>
rl_status record(rl_batch_plan *p, const TI *a, const TI *b, TI *x, int *info, int *iters, double *berr,
                 cudaStream_t s) {
    RL_TRY_CUDA(cudaMemsetAsync(p->d_counters, 0, 4 * sizeof(int), s));
    BatchDesc d{};
    d.count = (int)p->count;
    d.count_dev = nullptr;
    d.order = p->d_order;
    d.n = p->d_n;
    d.kind = p->d_kind;
    d.a_off = p->d_aoff;
    d.b_off = p->d_boff;
    d.next = p->d_counters;
    d.fb_list = p->d_fb_list;
    d.fb_count = p->d_counters + 1;
    d.work = p->d_work;
    d.work_stride = p->work_stride;
    d.info = info;
    d.iters = iters;
    d.berr = berr;
    d.iters_tag = 0;
    d.max_iters = 30;
    d.warp_small = 1;  // the order is largest-cost first
    d.warp_cost = (int)tune(RL_TUNE_BATCH_WARP_COST);
    d.wait_ns = wait_ns();
    RL_LAUNCH((batch_solve_kernel<TI, TF, MIXED>), p->grid, CTA_THREADS, p->smem, s, d, a, b, x);
    if (MIXED) {
        BatchDesc f = d;
        f.count = 0;
        f.count_dev = p->d_counters + 1;
        f.order = p->d_fb_list;
        f.next = p->d_counters + 2;
        f.work = p->d_work64;
        f.iters_tag = -1;
        f.warp_small = 0;  // the fallback list is in arrival order
        RL_LAUNCH((batch_solve_kernel<TI, double, false>), p->grid64, CTA_THREADS, p->smem64, s, f, a, b, x);
    }
    return RL_OK;
}

template <class TI, class TF, bool MIXED>
rl_status run_plan(rl_batch_plan *p, const TI *a, const TI *b, TI *x, int *info, int *iters, double *berr,
                   cudaStream_t s) {
    NvtxRange nvtx_("rl.batch.solve_dev");
    const void *key[6] = {a, b, x, info, iters, berr};
    if (!p->exec || !std::equal(key, key + 6, p->key)) {
        if (p->exec) {
            cudaGraphExecDestroy(p->exec);
            p->exec = nullptr;
        }
        RL_TRY_CUDA(cudaStreamBeginCapture(p->cap, cudaStreamCaptureModeThreadLocal));
        const uint64_t before = g_launches.load();
        rl_status st = record<TI, TF, MIXED>(p, a, b, x, info, iters, berr, p->cap);
        g_launches.store(before);  // capture does not launch anything
        cudaGraph_t g = nullptr;
        cudaError_t e = cudaStreamEndCapture(p->cap, &g);
        if (st != RL_OK) {
            if (g) cudaGraphDestroy(g);
            return st;
        }
        if (e != cudaSuccess) return from_cuda(e);
        e = cudaGraphInstantiate(&p->exec, g, 0);
        cudaGraphDestroy(g);
        if (e != cudaSuccess) {
            p->exec = nullptr;
            return from_cuda(e);
        }
        std::copy(key, key + 6, p->key);
    }
    RL_TRY_CUDA(cudaGraphLaunch(p->exec, s));
    count_launch(MIXED ? 2 : 1);
    return RL_OK;
}

// The host-path launch: the main pass over all chunks, gated per chunk, then (mixed) the
// FP64 pass over the systems it handed on.
template <class TI, class TF, bool MIXED>
rl_status launch_gated(rl_batch_plan *p, const TI *a, const TI *b, TI *x, cudaStream_t s) {
    int *ctr = p->d_ccounters;
    BatchDesc d{};
    d.count = (int)p->count;
    d.count_dev = nullptr;
    d.order = p->d_corder;
    d.n = p->d_n;
    d.kind = p->d_kind;
    d.a_off = p->d_aoff_h;
    d.b_off = p->d_boff_h;
    d.next = ctr;
    d.fb_list = p->d_fb_list;
    d.fb_count = ctr + 1;
    d.work = p->d_work;
    d.work_stride = p->work_stride;
    d.info = p->h_info;
    d.iters = p->h_iters;
    d.berr = p->h_berr;
    d.iters_tag = 0;
    d.max_iters = 30;
    d.warp_small = 1;  // largest-cost first within each chunk: the last chunk's tail
    d.warp_from = p->chunk_first.back();
    d.gate = p->d_gate;
    d.gate_pos = p->d_gate_pos;
    d.gate_n = (int)p->chunk_first.size();
    d.gate_err = ctr + 3;
    d.wait_ns = wait_ns();
    d.warp_cost = (int)tune(RL_TUNE_BATCH_WARP_COST);
    static const cudaError_t attr = cudaFuncSetAttribute(batch_solve_kernel<TI, TF, MIXED, true>,
                                                         cudaFuncAttributeMaxDynamicSharedMemorySize, (int)p->smem);
    RL_TRY_CUDA(attr);
    RL_LAUNCH((batch_solve_kernel<TI, TF, MIXED, true>), std::min<long long>(p->grid, p->count), CTA_THREADS, p->smem,
              s, d, a, b, x);
    if (MIXED) {
        BatchDesc f = d;
        f.count = 0;
        f.count_dev = ctr + 1;
        f.order = d.fb_list;
        f.next = ctr + 2;
        f.work = p->d_work64;
        f.iters_tag = -1;
        f.warp_small = 0;  // the fallback list is in arrival order
        f.warp_from = 0;
        f.gate_n = 0;      // every chunk is in by the time it runs
        RL_LAUNCH((batch_solve_kernel<TI, double, false>), std::min<long long>(p->grid64, p->count), CTA_THREADS,
                  p->smem64, s, f, a, b, x);
    }
    return RL_OK;
}

// Host buffers in, host buffers out. The systems go in contiguous chunks copied on the
// plan's copy stream, each followed by its arrival flag; the solve is one launch on the
// caller's stream that takes chunk c's systems once its flag is set, so the transfer
// and the solve overlap with no drain of the GPU between chunks.
template <class TI>
rl_status solve_host(rl_batch_plan *p, const TI *a, const TI *b, TI *x, int32_t *info, int32_t *iters,
                     double *berr) {
    NvtxRange nvtx_("rl.batch.solve_host");
    cudaStream_t s = cudaStreamPerThread;
    if (p->count == 0) return RL_OK;
    if (!p->h_a) {
        RL_TRY_CUDA(cudaMalloc(&p->h_a, std::max<long long>(1, p->a_total_h) * sizeof(TI)));
        RL_TRY_CUDA(cudaMalloc(&p->h_b, std::max<long long>(1, p->b_total_h) * sizeof(TI)));
        RL_TRY_CUDA(cudaMalloc(&p->h_x, std::max<long long>(1, p->b_total_h) * sizeof(TI)));
        RL_TRY_CUDA(cudaMalloc(&p->h_info, std::max<size_t>(1, p->count) * sizeof(int)));
        RL_TRY_CUDA(cudaMalloc(&p->h_iters, std::max<size_t>(1, p->count) * sizeof(int)));
        RL_TRY_CUDA(cudaMalloc(&p->h_berr, std::max<size_t>(1, p->count) * sizeof(double)));
        RL_TRY_CUDA(cudaMallocHost(&p->h_one, sizeof(int)));
        *p->h_one = 1;
        RL_TRY_CUDA(cudaStreamCreateWithFlags(&p->copy, cudaStreamNonBlocking));
        RL_TRY_CUDA(cudaEventCreateWithFlags(&p->ev_start, cudaEventDisableTiming));
    }
    TI *da = static_cast<TI *>(p->h_a), *db = static_cast<TI *>(p->h_b), *dx = static_cast<TI *>(p->h_x);
    const int nch = (int)p->chunk_first.size();
    RL_TRY_CUDA(cudaMemsetAsync(p->d_ccounters, 0, 4 * sizeof(int), s));
    RL_TRY_CUDA(cudaMemsetAsync(p->d_gate, 0, nch * sizeof(int), s));
    RL_TRY_CUDA(cudaEventRecord(p->ev_start, s));  // earlier work on the buffers, and the resets, first
    RL_TRY_CUDA(cudaStreamWaitEvent(p->copy, p->ev_start, 0));
    const int withhold = (int)tune(RL_TUNE_TEST_WITHHOLD_CHUNK);  // tests: a flag nothing sets
    for (int c = 0; c < nch; c++) {
        const int first = p->chunk_first[c], end = first + p->chunk_count[c];
        const long long a0 = p->a_off[first], a1 = end < (int)p->count ? p->a_off[end] : p->a_total;
        const long long b0 = p->b_off[first], b1 = end < (int)p->count ? p->b_off[end] : p->b_total;
        if (a1 > a0)
            RL_TRY_CUDA(cudaMemcpyAsync(da + a0 + p->a_shift[c], a + a0, (a1 - a0) * sizeof(TI), cudaMemcpyHostToDevice,
                                        p->copy));
        if (b1 > b0)
            RL_TRY_CUDA(cudaMemcpyAsync(db + b0 + p->b_shift[c], b + b0, (b1 - b0) * sizeof(TI), cudaMemcpyHostToDevice,
                                        p->copy));
        if (c != withhold)
            RL_TRY_CUDA(cudaMemcpyAsync(p->d_gate + c, p->h_one, sizeof(int), cudaMemcpyHostToDevice, p->copy));
    }
    rl_status st;
    if (std::is_same<TI, float>::value)
        st = launch_gated<float, float, false>(p, (const float *)da, (const float *)db, (float *)dx, s);
    else if (p->precision == RL_PREC_MIXED)
        st = launch_gated<double, float, true>(p, (const double *)da, (const double *)db, (double *)dx, s);
    else
        st = launch_gated<double, double, false>(p, (const double *)da, (const double *)db, (double *)dx, s);
    RL_TRY(st);
    for (int c = 0; c < nch; c++) {
        const int first = p->chunk_first[c], end = first + p->chunk_count[c];
        const long long b0 = p->b_off[first], b1 = end < (int)p->count ? p->b_off[end] : p->b_total;
        if (b1 > b0)
            RL_TRY_CUDA(cudaMemcpyAsync(x + b0, dx + b0 + p->b_shift[c], (b1 - b0) * sizeof(TI), cudaMemcpyDeviceToHost,
                                        s));
    }
    if (info) RL_TRY_CUDA(cudaMemcpyAsync(info, p->h_info, p->count * sizeof(int), cudaMemcpyDeviceToHost, s));
    if (iters) RL_TRY_CUDA(cudaMemcpyAsync(iters, p->h_iters, p->count * sizeof(int), cudaMemcpyDeviceToHost, s));
    if (berr) RL_TRY_CUDA(cudaMemcpyAsync(berr, p->h_berr, p->count * sizeof(double), cudaMemcpyDeviceToHost, s));
    int gate_err = 0;
    RL_TRY_CUDA(cudaMemcpyAsync(&gate_err, p->d_ccounters + 3, sizeof(int), cudaMemcpyDeviceToHost, s));
    RL_TRY_CUDA(cudaStreamSynchronize(s));
    return gate_err ? RL_ERR_TIMEOUT : RL_OK;
}

template <class T>
rl_status upload(T *&dst, const std::vector<T> &src, cudaStream_t s) {
    RL_TRY_CUDA(cudaMalloc(&dst, std::max<size_t>(1, src.size()) * sizeof(T)));
    if (!src.empty()) RL_TRY_CUDA(cudaMemcpyAsync(dst, src.data(), src.size() * sizeof(T), cudaMemcpyHostToDevice, s));
    return RL_OK;
}

rl_status plan_init(rl_batch_plan *p, size_t count, const int32_t *n, const uint8_t *kind, int precision) {
    p->precision = precision;
    p->count = count;
    p->n.resize(count);
    p->kind.resize(count);
    p->a_off.resize(count);
    p->b_off.resize(count);
    long long a = 0, b = 0;
    for (size_t i = 0; i < count; i++) {
        if (n[i] < 0 || n[i] > CTA_NMAX) return RL_ERR_INVALID_ARG;
        if (kind && kind[i] > 1) return RL_ERR_INVALID_ARG;
        p->n[i] = n[i];
        p->kind[i] = kind ? kind[i] : 0;
        p->a_off[i] = a;
        p->b_off[i] = b;
        a += (long long)n[i] * n[i];
        b += n[i];
        p->max_n = std::max(p->max_n, (int)n[i]);
    }
    p->a_total = a;
    p->b_total = b;
    // Largest work first (LU costs twice Cholesky), so the tail of the launch is short.
    std::vector<int> order(count);
    std::iota(order.begin(), order.end(), 0);
    std::stable_sort(order.begin(), order.end(), [&](int x, int y) {
        const double cx = (double)p->n[x] * p->n[x] * p->n[x] * (p->kind[x] ? 1.0 : 2.0);
        const double cy = (double)p->n[y] * p->n[y] * p->n[y] * (p->kind[y] ? 1.0 : 2.0);
        return cx > cy;
    });
    cudaStream_t s = cudaStreamPerThread;
    RL_TRY(upload(p->d_n, p->n, s));
    RL_TRY(upload(p->d_kind, p->kind, s));
    RL_TRY(upload(p->d_aoff, p->a_off, s));
    RL_TRY(upload(p->d_boff, p->b_off, s));
    RL_TRY(upload(p->d_order, order, s));
    // Host-path chunks: up to RL_TUNE_UPLOAD_CHUNKS (32 by default) contiguous ranges of
    // about equal matrix bytes, each with
    // its own largest-first order. Small chunks shorten both ends of the pipeline (the
    // solve starts after the first chunk's copy and ends a chunk's solve after the last
    // one's); with one gated launch there is no drain between chunks to pay for them.
    {
        const int want = (int)std::min<size_t>((size_t)tune(RL_TUNE_UPLOAD_CHUNKS), std::max<size_t>(1, count));
        std::vector<int> corder;
        corder.reserve(count);
        size_t i = 0;
        for (int c = 0; c < want && i < count; c++) {
            const long long target = (long long)((double)p->a_total * (c + 1) / want);
            size_t e = i + 1;
            while (e < count && (c == want - 1 || p->a_off[e] < target)) e++;
            p->chunk_first.push_back((int)i);
            p->chunk_count.push_back((int)(e - i));
            std::vector<int> part;
            for (int k : order)
                if ((size_t)k >= i && (size_t)k < e) part.push_back(k);
            corder.insert(corder.end(), part.begin(), part.end());
            i = e;
        }
        RL_TRY(upload(p->d_corder, corder, s));
        RL_TRY_CUDA(cudaMalloc(&p->d_ccounters, 4 * std::max<size_t>(1, p->chunk_first.size()) * sizeof(int)));
        // device layout of the host path: chunk starts rounded up to 64 elements (256
        // bytes in FP32, 512 in FP64)
        const int nch = (int)p->chunk_first.size();
        auto round64 = [](long long v) { return (v + 63) & ~63LL; };
        p->a_shift.assign(nch, 0);
        p->b_shift.assign(nch, 0);
        long long a_end = 0, b_end = 0;
        std::vector<long long> aoff_h(count), boff_h(count);
        std::vector<int> gate_pos(nch + 1, (int)count);
        for (int c = 0; c < nch; c++) {
            const int first = p->chunk_first[c], end = first + p->chunk_count[c];
            const long long a0 = p->a_off[first], a1 = end < (int)count ? p->a_off[end] : p->a_total;
            const long long b0 = p->b_off[first], b1 = end < (int)count ? p->b_off[end] : p->b_total;
            p->a_shift[c] = round64(a_end) - a0;
            p->b_shift[c] = round64(b_end) - b0;
            a_end = a1 + p->a_shift[c];
            b_end = b1 + p->b_shift[c];
            for (int k = first; k < end; k++) {
                aoff_h[k] = p->a_off[k] + p->a_shift[c];
                boff_h[k] = p->b_off[k] + p->b_shift[c];
            }
            gate_pos[c] = first;
        }
        p->a_total_h = a_end;
        p->b_total_h = b_end;
        RL_TRY(upload(p->d_aoff_h, aoff_h, s));
        RL_TRY(upload(p->d_boff_h, boff_h, s));
        RL_TRY(upload(p->d_gate_pos, gate_pos, s));
        RL_TRY_CUDA(cudaMalloc(&p->d_gate, std::max(1, nch) * sizeof(int)));
    }
    RL_TRY_CUDA(cudaMalloc(&p->d_counters, 4 * sizeof(int)));
    RL_TRY_CUDA(cudaMalloc(&p->d_fb_list, std::max<size_t>(1, count) * sizeof(int)));
    const long long npad = (p->max_n + 3) & ~3;  // slot row stride rounded up to 4
    p->work_stride = std::max(4LL, npad * npad);
    if (precision == RL_PREC_MIXED) {
        p->smem = cta_smem_bytes<float>();
        RL_TRY((occupancy_grid<double, float, true>(p->smem, p->grid)));
        p->smem64 = cta_smem_bytes<double>();
        RL_TRY((occupancy_grid<double, double, false>(p->smem64, p->grid64)));
        RL_TRY_CUDA(cudaMalloc(&p->d_work, p->grid * p->work_stride * sizeof(float)));
        RL_TRY_CUDA(cudaMalloc(&p->d_work64, p->grid64 * p->work_stride * sizeof(double)));
    } else if (precision == RL_PREC_FP64) {
        p->smem = cta_smem_bytes<double>();
        RL_TRY((occupancy_grid<double, double, false>(p->smem, p->grid)));
        RL_TRY_CUDA(cudaMalloc(&p->d_work, p->grid * p->work_stride * sizeof(double)));
    } else if (precision == RL_PREC_FP32) {
        p->smem = cta_smem_bytes<float>();
        RL_TRY((occupancy_grid<float, float, false>(p->smem, p->grid)));
        RL_TRY_CUDA(cudaMalloc(&p->d_work, p->grid * p->work_stride * sizeof(float)));
    } else {
        return RL_ERR_INVALID_ARG;
    }
    RL_TRY_CUDA(cudaStreamCreateWithFlags(&p->cap, cudaStreamNonBlocking));
    RL_TRY_CUDA(cudaStreamSynchronize(s));
    return RL_OK;
}

void plan_free(rl_batch_plan *p) {
    if (p->exec) cudaGraphExecDestroy(p->exec);
    if (p->cap) cudaStreamDestroy(p->cap);
    if (p->copy) cudaStreamDestroy(p->copy);
    if (p->ev_start) cudaEventDestroy(p->ev_start);
    void *ptrs[] = {p->d_n,   p->d_order, p->d_counters, p->d_fb_list,  p->d_kind,      p->d_aoff,   p->d_boff,
                    p->d_work, p->d_work64, p->h_a,      p->h_b,        p->h_x,         p->h_info,   p->h_iters,
                    p->h_berr, p->d_corder, p->d_ccounters, p->d_gate, p->d_gate_pos, p->d_aoff_h, p->d_boff_h};
    for (void *q : ptrs)
        if (q) cudaFree(q);
    if (p->h_one) cudaFreeHost(p->h_one);
}

}  // namespace

extern "C" {

rl_status rl_batch_plan_create(rl_batch_plan **plan, size_t count, const int32_t *n, const uint8_t *kind,
                               int precision) {
    if (!plan || (count && !n)) return RL_ERR_INVALID_ARG;
    *plan = nullptr;
    if (count > (size_t)INT32_MAX) return RL_ERR_INVALID_ARG;
    RL_TRY(ensure_device());
    rl_batch_plan *p = new rl_batch_plan();
    rl_status st = plan_init(p, count, n, kind, precision);
    if (st != RL_OK) {
        plan_free(p);
        delete p;
        return st;
    }
    *plan = p;
    return RL_OK;
}

rl_status rl_batch_plan_destroy(rl_batch_plan *plan) {
    if (!plan) return RL_OK;
    cudaDeviceSynchronize();
    plan_free(plan);
    delete plan;
    return RL_OK;
}

rl_status rl_batch_plan_layout(const rl_batch_plan *plan, int64_t *a_offset, int64_t *b_offset, int64_t *a_total,
                               int64_t *b_total) {
    if (!plan) return RL_ERR_INVALID_ARG;
    for (size_t i = 0; i < plan->count; i++) {
        if (a_offset) a_offset[i] = plan->a_off[i];
        if (b_offset) b_offset[i] = plan->b_off[i];
    }
    if (a_total) *a_total = plan->a_total;
    if (b_total) *b_total = plan->b_total;
    return RL_OK;
}

rl_status rl_dbatch_solve_dev(rl_batch_plan *plan, const double *a, const double *b, double *x, int32_t *info,
                              int32_t *iters, double *berr, void *stream) {
    if (!plan || !info || (plan->b_total && (!a || !b || !x))) return RL_ERR_INVALID_ARG;
    if (plan->precision == RL_PREC_FP32) return RL_ERR_INVALID_ARG;
    std::lock_guard<std::mutex> lk(plan->mu);
    cudaStream_t s = resolve_stream(stream);
    if (plan->precision == RL_PREC_MIXED) return run_plan<double, float, true>(plan, a, b, x, info, iters, berr, s);
    return run_plan<double, double, false>(plan, a, b, x, info, iters, berr, s);
}

rl_status rl_sbatch_solve_dev(rl_batch_plan *plan, const float *a, const float *b, float *x, int32_t *info,
                              int32_t *iters, double *berr, void *stream) {
    if (!plan || !info || (plan->b_total && (!a || !b || !x))) return RL_ERR_INVALID_ARG;
    if (plan->precision != RL_PREC_FP32) return RL_ERR_INVALID_ARG;
    std::lock_guard<std::mutex> lk(plan->mu);
    return run_plan<float, float, false>(plan, a, b, x, info, iters, berr, resolve_stream(stream));
}

rl_status rl_dbatch_solve(rl_batch_plan *plan, const double *a, const double *b, double *x, int32_t *info,
                          int32_t *iters, double *berr) {
    if (!plan || (plan->b_total && (!a || !b || !x))) return RL_ERR_INVALID_ARG;
    if (plan->precision == RL_PREC_FP32) return RL_ERR_INVALID_ARG;
    std::lock_guard<std::mutex> lk(plan->mu);
    return solve_host<double>(plan, a, b, x, info, iters, berr);
}

rl_status rl_sbatch_solve(rl_batch_plan *plan, const float *a, const float *b, float *x, int32_t *info,
                          int32_t *iters, double *berr) {
    if (!plan || (plan->b_total && (!a || !b || !x))) return RL_ERR_INVALID_ARG;
    if (plan->precision != RL_PREC_FP32) return RL_ERR_INVALID_ARG;
    std::lock_guard<std::mutex> lk(plan->mu);
    return solve_host<float>(plan, a, b, x, info, iters, berr);
}

}  // extern "C"
