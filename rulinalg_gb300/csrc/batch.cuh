// Batched solve kernels (thousands of independent systems, n <= 512, one launch) and
// the one-CTA kernels used by the single-matrix entry points for n <= 512.
#pragma once

#include <cfloat>

#include "factor_cta.cuh"

namespace rl {

// Where a batch lives and where each CTA finds its work.
struct BatchDesc {
    int count;               // systems in `order`
    const int *count_dev;    // if set, the count is read from device memory instead
    const int *order;        // system indices in scheduling order (largest first)
    const int *n;            // per-system order
    const uint8_t *kind;     // 0 = PartialPivLu, 1 = Cholesky
    const long long *a_off;  // matrix start (elements), row stride = n
    const long long *b_off;  // vector start (elements)
    int *next;               // work counter, zero before the launch
    int *fb_list;            // mixed precision: systems handed to the FP64 pass
    int *fb_count;
    void *work;              // per-CTA factor workspace slots
    long long work_stride;   // elements per slot (>= ldw * n, ldw = n rounded up to 4)
    int *info;               // per-system status
    int *iters;              // refinement steps (-1: solved by the FP64 fallback pass)
    double *berr;            // normwise backward error ||b - Ax|| / (||A|| ||x|| + ||b||), inf-norms
    int iters_tag;           // value written to iters by a plain pass (0, or -1 for fallback)
    int max_iters;           // refinement limit (mixed)
    int warp_small;          // 1: `order` is largest-cost first (n^3, x2 for LU) from position
                             // warp_from on, so that small tail may go to the warp-per-system path
    int warp_from;
    // Host path, one launch for all chunks: chunk c owns the order positions
    // [gate_pos[c], gate_pos[c + 1]) and its inputs are on the device once gate[c] != 0
    // (written by the copy stream after the chunk's copies). gate_n = 0: no gating.
    const int *gate;
    const int *gate_pos;
    int gate_n;
    int *gate_err;           // set when a wait for a chunk ran out; the CTA then stops
    unsigned long long wait_ns;  // limit of a chunk wait (RL_TUNE_WAIT_TIMEOUT_NS)
    int warp_cost;           // systems of cost n^3 (x2 for LU) up to this go one per warp (<= kWarpCost)
};

// Systems of cost n^3 (x2 for LU) at most this go one per warp: a Cholesky n <= 32 or an
// LU n <= 25, so that everything after such a system in a largest-first order fits a warp.
constexpr double kWarpCost = 32.0 * 32.0 * 32.0;

constexpr double kU64 = 1.1102230246251565e-16;  // 2^-53

}  // namespace rl

#include "warp_small.cuh"

namespace rl {

template <class TI, class TF>
__device__ void store_solution(const BatchDesc &d, int sys, int n, TI *xi, CtaSmem<TF> &S, int st, int iters,
                               double berr) {
    if (st == RL_OK)
        for (int i = threadIdx.x; i < n; i += CTA_THREADS) xi[i] = (TI)S.x()[i];
    if (threadIdx.x == 0) {
        d.info[sys] = st;
        if (d.iters) d.iters[sys] = iters;
        if (d.berr) d.berr[sys] = berr;
    }
}

template <class TF>
__device__ void push_fallback(const BatchDesc &d, int sys) {
    if (threadIdx.x == 0) {
        const int k = atomicAdd(d.fb_count, 1);
        d.fb_list[k] = sys;
    }
}

// One system. MIXED: factor a TF copy, refine in FP64 against the TI matrix; failures
// and stagnation go to the fallback list. Plain: factor and solve in TF, report berr.
template <class TI, class TF, bool MIXED>
__device__ void batch_solve_one(const BatchDesc &d, int sys, const TI *__restrict__ A, const TI *__restrict__ B,
                                TI *__restrict__ X, TF *__restrict__ W, CtaSmem<TF> &S) {
    const int tid = threadIdx.x;
    const int n = d.n[sys];
    const int kind = d.kind[sys];
    const TI *Ai = A + d.a_off[sys];
    const TI *bi = B + d.b_off[sys];
    TI *xi = X + d.b_off[sys];
    if (n == 0) {
        store_solution<TI, TF>(d, sys, 0, xi, S, RL_OK, 0, 0.0);
        __syncthreads();
        return;
    }
    // Working copy in the factor type (row stride rounded up to 4 elements so that the
    // trailing updates use 128-bit accesses); ||A||_inf from the same pass.
    const int ldw = (n + 3) & ~3;
    const double anorm = cta_copy_convert<TI, TF>(Ai, n, n, W, ldw, S);
    double bm = 0.0;
    for (int i = tid; i < n; i += CTA_THREADS) bm = fmax(bm, fabs((double)bi[i]));
    const double bnorm = block_max(bm, S);

    const TF tiny = MIXED ? TF(FLT_MIN) : Eps<TF>::value;
    int st = kind ? cta_chol_factor<TF>(W, ldw, n, S, tiny) : cta_lu_factor<TF>(W, ldw, n, S, tiny);
    if (st == RL_OK && !kind) cta_build_rowperm(n, S);
    if (st == RL_OK) {
        for (int i = tid; i < n; i += CTA_THREADS) S.w[i] = (TF)bi[i];
        __syncthreads();
        st = cta_factor_solve<TF>(W, ldw, n, kind, S, tiny);
    }
    if (st != RL_OK) {
        if (MIXED)
            push_fallback<TF>(d, sys);
        else
            store_solution<TI, TF>(d, sys, n, xi, S, st, d.iters_tag, 0.0);
        __syncthreads();
        return;
    }
    for (int i = tid; i < n; i += CTA_THREADS) S.x()[i] = (double)S.w[i];
    __syncthreads();

    if (!MIXED) {
        const double rn = cta_residual<TI, TF>(Ai, n, bi, n, S);
        double xm = 0.0;
        for (int i = tid; i < n; i += CTA_THREADS) xm = fmax(xm, fabs(S.x()[i]));
        const double xn = block_max(xm, S);
        const double den = anorm * xn + bnorm;
        store_solution<TI, TF>(d, sys, n, xi, S, RL_OK, d.iters_tag, den > 0 ? rn / den : 0.0);
        __syncthreads();
        return;
    }

    // FP64 iterative refinement: r = b - A x in FP64, d = A_f^-1 r in the factor type,
    // x += d in FP64. Stop when ||r|| <= sqrt(n) u ||A|| ||x|| (LAPACK dsgesv's test).
    const double stop = sqrt((double)n) * kU64;
    double prev = INFINITY, rn = 0.0, xn = 0.0;
    bool ok = false;
    int it = 0;
    for (;; it++) {
        rn = cta_residual<TI, TF>(Ai, n, bi, n, S);
        double xm = 0.0;
        for (int i = tid; i < n; i += CTA_THREADS) xm = fmax(xm, fabs(S.x()[i]));
        xn = block_max(xm, S);
        if (rn <= stop * anorm * xn) {
            ok = true;
            break;
        }
        if (it >= d.max_iters) break;
        if (it >= 2 && rn > 0.5 * prev) {  // stagnation: accept only within 10 n u
            ok = rn <= 10.0 * n * kU64 * (anorm * xn + bnorm);
            break;
        }
        prev = rn;
        const double scale = 1.0 / rn;
        for (int i = tid; i < n; i += CTA_THREADS) S.w[i] = (TF)(S.r()[i] * scale);
        __syncthreads();
        if (cta_factor_solve<TF>(W, ldw, n, kind, S, tiny) != RL_OK) break;
        for (int i = tid; i < n; i += CTA_THREADS) S.x()[i] = fma(rn, (double)S.w[i], S.x()[i]);
        __syncthreads();
    }
    if (ok) {
        const double den = anorm * xn + bnorm;
        store_solution<TI, TF>(d, sys, n, xi, S, RL_OK, it, den > 0 ? rn / den : 0.0);
    } else {
        push_fallback<TF>(d, sys);
    }
    __syncthreads();
}

// Waits (one thread) until *flag != 0, sleeping between polls, at most `limit` ns of wall
// time; false if it ran out. The flag is written by a copy after the chunk's data copies
// on the same stream, so the data is in device memory once the flag is seen.
__device__ __forceinline__ bool gate_wait(const int *flag, unsigned long long limit) {
    unsigned long long t0, t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t0));
    for (;;) {
        int v;
        asm volatile("ld.acquire.gpu.global.b32 %0, [%1];" : "=r"(v) : "l"(flag) : "memory");
        if (v != 0) return true;
        asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
        if (t - t0 > limit) return false;
        __nanosleep(256);
    }
}

// The next position of the queue (one thread); with gating, waits until the position's
// chunk is on the device (gate_ok = 0 if the wait ran out). Out of line: it keeps the
// gate bookkeeping out of the solver's registers.
static __device__ __noinline__ int dequeue(const BatchDesc &d, int count, int &gate, int &gate_ok) {
    const int it = atomicAdd(d.next, 1);
    gate_ok = 1;
    if (d.gate_n > 0 && it < count) {
        int c = 0;
        while (c + 1 < d.gate_n && it >= d.gate_pos[c + 1]) c++;
        if (c > gate) {
            gate_ok = gate_wait(d.gate + c, d.wait_ns);
            if (gate_ok)
                gate = c;  // chunks arrive in order: every chunk up to c is in
            else
                atomicExch(d.gate_err, 1);
        }
    }
    return it;
}

// GATED: the host path's single launch over chunks that are still arriving (dequeue()
// waits on the chunk flags); a separate instantiation, so the device path's kernel
// carries none of it.
template <class TI, class TF, bool MIXED, bool GATED = false>
__global__ void __launch_bounds__(CTA_THREADS, CtaOcc<TF>::value) batch_solve_kernel(BatchDesc d, const TI *A, const TI *B, TI *X) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    CtaSmem<TF> &S = *reinterpret_cast<CtaSmem<TF> *>(smem_raw);
    TF *W = static_cast<TF *>(d.work) + (long long)blockIdx.x * d.work_stride;
    const int count = d.count_dev ? *d.count_dev : d.count;
    __shared__ int s_gate, s_gate_ok;  // highest chunk seen on the device; this item's chunk arrived
    if (GATED && threadIdx.x == 0) s_gate = -1;
    for (;;) {
        if (threadIdx.x == 0) {
            if (GATED)
                S.item = dequeue(d, count, s_gate, s_gate_ok);
            else
                S.item = atomicAdd(d.next, 1);
        }
        __syncthreads();
        const int it = S.item;
        const bool gate_ok = !GATED || s_gate_ok != 0;
        __syncthreads();
        if (it >= count || !gate_ok) return;  // done, or a chunk never arrived (gate_err is set)
        const int sys0 = d.order[it], n0 = d.n[sys0];
        const bool small = (double)n0 * n0 * n0 * (d.kind[sys0] ? 1.0 : 2.0) <= (double)d.warp_cost;
        if (small && (!d.warp_small || (GATED && it < d.warp_from))) {
            // an unordered list (the fallback pass): the small system still takes the
            // warp path, so its arithmetic is the same in every pass
            if (threadIdx.x < 32) warp_solve_small<TI, TF, MIXED>(d, sys0, A, B, X, S.P);
            __syncthreads();
            continue;
        }
        if (small) {
            // Largest first: everything left is this small. From here each warp takes its
            // own systems (warp 0 starts with this one); no CTA barrier follows.
            const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
            TF *tile = S.P + warp * WARP_NMAX * WARP_LDT;
            int item = warp == 0 ? it : -1;
            for (;;) {
                if (item < 0) {
                    if (lane == 0) item = atomicAdd(d.next, 1);
                    item = __shfl_sync(0xffffffffu, item, 0);
                }
                if (item >= count) return;
                warp_solve_small<TI, TF, MIXED>(d, d.order[item], A, B, X, tile);
                item = -1;
            }
        }
        batch_solve_one<TI, TF, MIXED>(d, d.order[it], A, B, X, W, S);
    }
}

// ------------------------------------------------ single matrices with n <= 512 --

// Factor one matrix in place. kind 0: LU (ipiv receives LAPACK-style pivots),
// 1: Cholesky. status[0] receives the result.
template <class T>
__global__ void __launch_bounds__(CTA_THREADS, 2)
    factor_one_kernel(T *A, int lda, int n, int kind, int *ipiv, int *status, T tiny) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    CtaSmem<T> &S = *reinterpret_cast<CtaSmem<T> *>(smem_raw);
    const int st = kind ? cta_chol_factor<T>(A, lda, n, S, tiny) : cta_lu_factor<T>(A, lda, n, S, tiny);
    if (kind == 0 && ipiv)
        for (int i = threadIdx.x; i < n; i += CTA_THREADS) ipiv[i] = S.piv[i];
    if (threadIdx.x == 0) status[0] = st;
}

// Solve with a factor for nrhs columns of B (row-major n x nrhs, stride ldb); one CTA
// per column. LU: perm is the stored permutation (y[perm[i]] = b[i], the reference's
// P * b); Cholesky: perm is null. The first failing status is kept in status[0].
template <class T>
__global__ void __launch_bounds__(CTA_THREADS) solve_one_kernel(const T *F, int lda, int n, int kind,
                                                                 const uint64_t *perm, T *B, long long ldb,
                                                                 int *status, T tiny) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    CtaSmem<T> &S = *reinterpret_cast<CtaSmem<T> *>(smem_raw);
    const int c = blockIdx.x;
    for (int i = threadIdx.x; i < n; i += CTA_THREADS) {
        const T v = B[(long long)i * ldb + c];
        if (perm)
            S.w[perm[i]] = v;
        else
            S.w[i] = v;
    }
    __syncthreads();
    int st;
    if (kind == 1) {
        st = cta_lower_solve<T>(F, lda, n, S, tiny);
        if (st == RL_OK) st = cta_lower_t_solve<T>(F, lda, n, S, tiny);
    } else {
        cta_unit_lower_solve<T>(F, lda, n, S);
        st = cta_upper_solve<T>(F, lda, n, S, tiny);
    }
    if (st == RL_OK)
        for (int i = threadIdx.x; i < n; i += CTA_THREADS) B[(long long)i * ldb + c] = S.w[i];
    if (threadIdx.x == 0 && st != RL_OK) atomicCAS(status, 0, st);
}

template <class T>
inline size_t cta_smem_bytes() {
    return sizeof(CtaSmem<T>);
}

}  // namespace rl
