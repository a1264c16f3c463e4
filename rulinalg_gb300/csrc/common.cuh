// Shared runtime pieces of the rulinalg_gb300 CUDA library: status mapping, the
// launch counter, device checks, stream resolution and stream-ordered device buffers.
#pragma once

#include <cuda_runtime.h>
#include <nvtx3/nvToolsExt.h>

#include <atomic>
#include <cstddef>
#include <cstdint>
#include <cstring>

#include "../../include/rulinalg_gb300.h"

namespace rl {

// Number of kernel launches issued by this library (reported by rl_launch_count()).
extern std::atomic<uint64_t> g_launches;
inline void count_launch(uint64_t k = 1) { g_launches.fetch_add(k, std::memory_order_relaxed); }

// Map a CUDA error to an rl_status and remember it for diagnostics.
rl_status from_cuda(cudaError_t e);

// RL_OK when a compute capability 10.3 device is usable; cached after the first call.
rl_status ensure_device();

// Host-pointer entry points run on the calling thread's default stream.
inline cudaStream_t resolve_stream(void *s) { return s ? static_cast<cudaStream_t>(s) : cudaStreamPerThread; }

#define RL_TRY_CUDA(expr)                                   \
    do {                                                    \
        cudaError_t rl_e_ = (expr);                         \
        if (rl_e_ != cudaSuccess) return rl::from_cuda(rl_e_); \
    } while (0)

#define RL_TRY(expr)                          \
    do {                                      \
        rl_status rl_s_ = (expr);             \
        if (rl_s_ != RL_OK) return rl_s_;     \
    } while (0)

// Launch bookkeeping: every kernel launch in the library goes through this macro so
// that rl_launch_count() and the launch-error check stay exact.
#define RL_LAUNCH(kernel, grid, block, smem, stream, ...)                  \
    do {                                                                   \
        kernel<<<(grid), (block), (smem), (stream)>>>(__VA_ARGS__);        \
        rl::count_launch();                                                \
        cudaError_t rl_le_ = cudaGetLastError();                           \
        if (rl_le_ != cudaSuccess) return rl::from_cuda(rl_le_);           \
    } while (0)

// A stream-ordered device buffer (cudaMallocAsync from the device's default pool, whose
// release threshold is raised at start-up so that repeated calls reuse memory).
template <class T>
struct DevBuf {
    T *p = nullptr;
    size_t n = 0;
    cudaStream_t s = nullptr;
    DevBuf() = default;
    DevBuf(const DevBuf &) = delete;
    DevBuf &operator=(const DevBuf &) = delete;
    rl_status alloc(size_t count, cudaStream_t stream) {
        s = stream;
        n = count;
        if (count == 0) return RL_OK;
        cudaError_t e = cudaMallocAsync(reinterpret_cast<void **>(&p), count * sizeof(T), stream);
        if (e != cudaSuccess) {
            p = nullptr;
            return from_cuda(e);
        }
        return RL_OK;
    }
    ~DevBuf() {
        if (p) cudaFreeAsync(p, s);
    }
};

// Row-major strided copies between host and device (a MatrixSlice with row_stride).
template <class T>
inline rl_status copy_h2d(T *dst, size_t ldd, const T *src, size_t lds, size_t rows, size_t cols,
                          cudaStream_t s) {
    if (rows == 0 || cols == 0) return RL_OK;
    RL_TRY_CUDA(cudaMemcpy2DAsync(dst, ldd * sizeof(T), src, lds * sizeof(T), cols * sizeof(T), rows,
                                  cudaMemcpyHostToDevice, s));
    return RL_OK;
}
template <class T>
inline rl_status copy_d2h(T *dst, size_t ldd, const T *src, size_t lds, size_t rows, size_t cols,
                          cudaStream_t s) {
    if (rows == 0 || cols == 0) return RL_OK;
    RL_TRY_CUDA(cudaMemcpy2DAsync(dst, ldd * sizeof(T), src, lds * sizeof(T), cols * sizeof(T), rows,
                                  cudaMemcpyDeviceToHost, s));
    return RL_OK;
}

// A named NVTX range around a phase of the library's work (a factorisation, a refinement
// loop, a batched solve): profilers attached to the process (ncu --nvtx, nsys) show and
// filter by it; without one the calls return at once.
struct NvtxRange {
    explicit NvtxRange(const char *name) { nvtxRangePushA(name); }
    ~NvtxRange() { nvtxRangePop(); }
    NvtxRange(const NvtxRange &) = delete;
    NvtxRange &operator=(const NvtxRange &) = delete;
};

template <class T>
struct Eps;
template <>
struct Eps<float> {
    static constexpr float value = 1.1920928955078125e-07f;
};
template <>
struct Eps<double> {
    static constexpr double value = 2.220446049250313e-16;
};

inline int ceil_div(long long a, long long b) { return static_cast<int>((a + b - 1) / b); }

int num_sms();

// The current value of a process-wide tunable (RL_TUNE_* in rulinalg_gb300.h).
int64_t tune(int key);
inline unsigned long long wait_ns() { return (unsigned long long)tune(RL_TUNE_WAIT_TIMEOUT_NS); }

// Set on threads that share the GPU with other streams of this library (the serving
// loop's workers): kernels whose CTAs wait on other CTAs of the same launch, holding
// their SMs meanwhile, are replaced there by chains of short launches. Measured on the
// served stream: the one-launch triangular sweep next to the other workers' panels and
// batched launches cut throughput from ~870 to ~390 requests/s.
extern thread_local bool g_shared_gpu;

}  // namespace rl
