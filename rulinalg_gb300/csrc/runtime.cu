// Process-wide runtime state of the library: device check, memory-pool set-up, status
// strings and the launch counter.
#include <mutex>

#include "common.cuh"

namespace rl {

std::atomic<uint64_t> g_launches{0};
thread_local bool g_shared_gpu = false;

static std::once_flag g_dev_once;
static rl_status g_dev_status = RL_ERR_NO_DEVICE;
static int g_num_sms = 0;

rl_status from_cuda(cudaError_t e) {
    if (e == cudaSuccess) return RL_OK;
    if (e == cudaErrorMemoryAllocation) return RL_ERR_OUT_OF_MEMORY;
    if (e == cudaErrorNoDevice || e == cudaErrorInsufficientDriver) return RL_ERR_NO_DEVICE;
    return RL_ERR_CUDA;
}

static void init_device() {
    int count = 0;
    if (cudaGetDeviceCount(&count) != cudaSuccess || count == 0) {
        cudaGetLastError();
        g_dev_status = RL_ERR_NO_DEVICE;
        return;
    }
    int dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceProp prop;
    if (cudaGetDeviceProperties(&prop, dev) != cudaSuccess) {
        g_dev_status = RL_ERR_NO_DEVICE;
        return;
    }
    // The kernels are built for sm_103a only.
    if (prop.major != 10 || prop.minor != 3) {
        g_dev_status = RL_ERR_NO_DEVICE;
        return;
    }
    g_num_sms = prop.multiProcessorCount;
    // Keep freed blocks in the default pool so per-call workspaces are cheap, and never
    // let the pool hand a block freed on one stream to another stream by making the
    // second wait for the first: with several worker streams (the serving loop) those
    // hidden dependencies serialised the workers (measured: p50 latency 113-172 ms with
    // them, 4-8 ms without).
    cudaMemPool_t pool;
    if (cudaDeviceGetDefaultMemPool(&pool, dev) == cudaSuccess) {
        uint64_t threshold = UINT64_MAX;
        cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &threshold);
        int zero = 0;
        cudaMemPoolSetAttribute(pool, cudaMemPoolReuseAllowInternalDependencies, &zero);
    }
    g_dev_status = RL_OK;
}

rl_status ensure_device() {
    std::call_once(g_dev_once, init_device);
    return g_dev_status;
}

int num_sms() {
    ensure_device();
    return g_num_sms > 0 ? g_num_sms : 152;
}

namespace {
struct TuneKey {
    int key;
    int64_t lo, hi, value;
};
// Keys, ranges and defaults of the tunables (rulinalg_gb300.h documents each one).
TuneKey g_tune_keys[] = {
    {RL_TUNE_WAIT_TIMEOUT_NS, 1000000LL, 10000000000LL, 1000000000LL},
    {RL_TUNE_PANEL_CLUSTER_MAX, 0, 16, 16},
    {RL_TUNE_BATCH_CTAS_PER_SM, 0, 8, 0},
    {RL_TUNE_BATCH_WARP_COST, 0, 32768, 32768},
    {RL_TUNE_UPLOAD_CHUNKS, 1, 256, 32},
    {RL_TUNE_MIXED_REFINE_STEPS, 1, 30, 30},
    {RL_TUNE_LU_OUTER_NB, -1, 4096, -1},
    {RL_TUNE_MIXED_SWEEP_INV, 0, 1, 1},
    {RL_TUNE_PANEL_LOOKAHEAD, 0, 1, 0},
    {RL_TUNE_FULLPIV_CTAS_PER_SM, 1, 3, 3},
    {RL_TUNE_TEST_WITHHOLD_CHUNK, -1, 255, -1},
    {RL_TUNE_TEST_WITHHOLD_SWEEP_BLOCK, -1, 1LL << 30, -1},
};
constexpr int kTuneCount = sizeof(g_tune_keys) / sizeof(g_tune_keys[0]);
std::atomic<int64_t> g_tune_values[kTuneCount];
std::once_flag g_tune_once;
void tune_init() {
    for (int i = 0; i < kTuneCount; i++) g_tune_values[i].store(g_tune_keys[i].value);
}
int tune_index(int key) {
    for (int i = 0; i < kTuneCount; i++)
        if (g_tune_keys[i].key == key) return i;
    return -1;
}
}  // namespace

int64_t tune(int key) {
    std::call_once(g_tune_once, tune_init);
    const int i = tune_index(key);
    return i < 0 ? 0 : g_tune_values[i].load(std::memory_order_relaxed);
}

}  // namespace rl

extern "C" {

const char *rl_status_string(rl_status s) {
    switch (s) {
        case RL_OK: return "ok";
        case RL_ERR_INVALID_ARG: return "invalid argument";
        case RL_ERR_DECOMP_FAILURE: return "decomposition failure";
        case RL_ERR_ALGEBRA_FAILURE: return "algebra failure";
        case RL_ERR_DIV_BY_ZERO: return "division by zero (singular to working precision)";
        case RL_ERR_SCALAR_CONVERSION: return "scalar conversion failure";
        case RL_ERR_INVALID_PERMUTATION: return "invalid permutation";
        case RL_ERR_SHAPE: return "dimension mismatch";
        case RL_ERR_CUDA: return "CUDA error";
        case RL_ERR_NO_DEVICE: return "no usable sm_103 GPU";
        case RL_ERR_OUT_OF_MEMORY: return "out of device memory";
        case RL_ERR_TIMEOUT: return "device wait timed out";
        case RL_ERR_NOT_CONVERGED: return "iterative refinement did not converge";
        case RL_ERR_BUSY: return "server queue full (backpressure)";
        default: return "unknown status";
    }
}

int rl_version(void) { return 100; }

rl_status rl_device_check(void) { return rl::ensure_device(); }

uint64_t rl_launch_count(void) { return rl::g_launches.load(std::memory_order_relaxed); }

rl_status rl_tune_set(int key, int64_t value) {
    std::call_once(rl::g_tune_once, rl::tune_init);
    const int i = rl::tune_index(key);
    if (i < 0 || value < rl::g_tune_keys[i].lo || value > rl::g_tune_keys[i].hi) return RL_ERR_INVALID_ARG;
    rl::g_tune_values[i].store(value);
    return RL_OK;
}

rl_status rl_tune_get(int key, int64_t *value) {
    const int i = rl::tune_index(key);
    if (i < 0 || !value) return RL_ERR_INVALID_ARG;
    *value = rl::tune(key);
    return RL_OK;
}

}  // extern "C"
