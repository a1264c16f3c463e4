// A solve entry point that allocates no memory at all.
//
// Some callers cannot call cudaMalloc: a serving process that reserves all device
// memory when it starts and forbids allocation afterwards (an allocation in the middle
// of a request can block on the driver, fragment the pool or fail under memory
// pressure), or a host framework whose own memory pool owns the GPU's memory. For them,
// rl_dsolve_mixed_noalloc_dev solves one f64 system with the same mixed-precision
// kernels as the batched solver (FP32 factor, FP64 refinement, FP64 refactor fallback),
// with every piece of scratch memory taken from one fixed array compiled into this
// library instead of from an allocator.
//
// The scratch array is a file-scope __device__ variable of a fixed size (kNoallocMaxN^2
// floats for the FP32 factor, kNoallocMaxN^2 doubles for the fallback factor and a small
// work descriptor: about 3 MiB). Every GPU that loads this library holds it until the
// process exits. All calls share it and it keeps the last call's contents, so calls
// that overlap on the GPU (different streams or threads without ordering between them)
// race on it; each call clears the counters that must start at zero before it runs.
#include <mutex>

#include "batch.cuh"

using namespace rl;

namespace {

constexpr int kNoallocMaxN = CTA_NMAX;  // 512
constexpr int kMaxDevices = 64;

struct NoallocScratch {
    int n;            // the system order
    int order;        // schedule: system 0
    int counters[4];  // [0] work counter, [1] fallback count, [2] fallback work counter
    int fb_list[1];
    long long a_off;  // 0
    long long b_off;  // 0
    uint8_t kind;
    float factor32[kNoallocMaxN * kNoallocMaxN];
    double factor64[kNoallocMaxN * kNoallocMaxN];
};

// The scratch memory. In host code this name is only a stand-in for the symbol: its
// device address comes from cudaGetSymbolAddress (scratch_address below).
static __device__ __align__(256) NoallocScratch g_noalloc_scratch;

// Writes the one-system descriptor and zeroes the counters (device code may name the
// array directly).
__global__ void noalloc_prepare_kernel(int n, int kind) {
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    NoallocScratch &s = g_noalloc_scratch;
    s.n = n;
    s.kind = (uint8_t)kind;
    s.order = 0;
    s.a_off = 0;
    s.b_off = 0;
    s.fb_list[0] = 0;
    for (int i = 0; i < 4; i++) s.counters[i] = 0;
}

std::mutex g_mu;
NoallocScratch *g_addr[kMaxDevices] = {};

// Device address of the scratch array on the current device, looked up once per device
// (with that device current) and cached.
rl_status scratch_address(NoallocScratch **out) {
    int dev = 0;
    RL_TRY_CUDA(cudaGetDevice(&dev));
    if (dev < 0 || dev >= kMaxDevices) return RL_ERR_INVALID_ARG;
    std::lock_guard<std::mutex> lk(g_mu);
    if (!g_addr[dev]) {
        void *p = nullptr;
        RL_TRY_CUDA(cudaGetSymbolAddress(&p, g_noalloc_scratch));
        auto k32 = batch_solve_kernel<double, float, true>;
        auto k64 = batch_solve_kernel<double, double, false>;
        RL_TRY_CUDA(cudaFuncSetAttribute(k32, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)cta_smem_bytes<float>()));
        RL_TRY_CUDA(cudaFuncSetAttribute(k64, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)cta_smem_bytes<double>()));
        g_addr[dev] = static_cast<NoallocScratch *>(p);
    }
    *out = g_addr[dev];
    return RL_OK;
}

}  // namespace

extern "C" rl_status rl_dsolve_mixed_noalloc_dev(size_t n, int kind, const double *a, const double *b, double *x,
                                                 int32_t *info, int32_t *iters, double *berr, void *stream) {
    if (n > (size_t)kNoallocMaxN) return RL_ERR_INVALID_ARG;  // beyond the fixed scratch
    if (kind != RL_KIND_LU && kind != RL_KIND_CHOLESKY) return RL_ERR_INVALID_ARG;
    if (!info || (n && (!a || !b || !x))) return RL_ERR_INVALID_ARG;
    RL_TRY(ensure_device());
    NoallocScratch *s = nullptr;
    RL_TRY(scratch_address(&s));
    cudaStream_t st = resolve_stream(stream);

    RL_LAUNCH(noalloc_prepare_kernel, 1, 32, 0, st, (int)n, kind);

    BatchDesc d{};
    d.count = 1;
    d.count_dev = nullptr;
    d.order = &s->order;
    d.n = &s->n;
    d.kind = &s->kind;
    d.a_off = &s->a_off;
    d.b_off = &s->b_off;
    d.next = &s->counters[0];
    d.fb_list = s->fb_list;
    d.fb_count = &s->counters[1];
    d.work = s->factor32;
    d.work_stride = (long long)kNoallocMaxN * kNoallocMaxN;
    d.info = info;
    d.iters = iters;
    d.berr = berr;
    d.iters_tag = 0;
    d.max_iters = 30;
    d.warp_small = 1;  // the order is largest-cost first
    d.warp_cost = (int)tune(RL_TUNE_BATCH_WARP_COST);
    d.wait_ns = wait_ns();
    RL_LAUNCH((batch_solve_kernel<double, float, true>), 1, CTA_THREADS, cta_smem_bytes<float>(), st, d, a, b, x);

    BatchDesc f = d;
    f.count = 0;
    f.count_dev = &s->counters[1];
    f.order = s->fb_list;
    f.next = &s->counters[2];
    f.work = s->factor64;
    f.iters_tag = -1;
    f.warp_small = 0;  // the fallback list is in arrival order
    RL_LAUNCH((batch_solve_kernel<double, double, false>), 1, CTA_THREADS, cta_smem_bytes<double>(), st, f, a, b, x);
    return RL_OK;
}
