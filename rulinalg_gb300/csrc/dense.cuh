// Kernels of the blocked (multi-CTA) factorisations used for n > 512 and for every
// HouseholderQr: cooperative panel kernels with a bounded grid barrier, row swaps,
// diagonal-block triangular solves and the compact-WY T factor. Trailing updates are
// GEMMs (gemm.cuh).
#pragma once

#include <climits>

#include <cooperative_groups.h>

#include "factor_cta.cuh"

namespace rl {

// Largest panel width of the blocked paths.
template <class T>
struct PanelNB {
    static constexpr int value = 64;
};

// ------------------------------------------------------------------ grid barrier --
// All CTAs of a cooperative launch arrive on `ctr`; thread 0 spins (bounded by
// `limit` ns of wall time, RL_TUNE_WAIT_TIMEOUT_NS) until the count reaches `target`.
// On timeout the error word is set and every CTA leaves the kernel at its next barrier.

__device__ __forceinline__ unsigned long long global_ns() {
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

__device__ __forceinline__ unsigned ld_acquire_u32(const unsigned *p) {
    unsigned v;
    asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}
__device__ __forceinline__ int ld_acquire(const int *p) { return (int)ld_acquire_u32(reinterpret_cast<const unsigned *>(p)); }
__device__ __forceinline__ void st_release(int *p, int v) {
    asm volatile("st.release.gpu.global.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}

static __device__ bool grid_barrier(unsigned *ctr, unsigned target, int *err, unsigned long long limit) {
    __shared__ int s_ok;
    __syncthreads();
    if (threadIdx.x == 0) {
        __threadfence();
        atomicAdd(ctr, 1u);
        const unsigned long long t0 = global_ns();
        int ok = 1;
        for (;;) {
            if (ld_acquire_u32(ctr) >= target) break;
            if (*(volatile int *)err != 0) {
                ok = 0;
                break;
            }
            if (global_ns() - t0 > limit) {
                atomicCAS(err, 0, RL_ERR_TIMEOUT);
                ok = 0;
                break;
            }
            __nanosleep(64);
        }
        __threadfence();
        s_ok = ok && (*(volatile int *)err == 0);
    }
    __syncthreads();
    return s_ok != 0;
}

// Shared state of one cooperative panel launch (global memory, zeroed per launch).
struct PanelSync {
    unsigned ctr;
    int err;     // RL_ERR_TIMEOUT or a numerical status, first writer wins
    int pad[2];
};

// ------------------------------------------------------------------- LU panel --
// Factors the panel rows [0, mrows) x cols [0, kb) of `P` (row stride lda; P points at
// A[k0][k0]) with partial pivoting. CTA g owns rows [g*rows_per, ...) staged in shared
// memory row-major (stride NB + 1). Per column: local argmax -> publish candidate row
// -> one grid barrier -> every CTA picks the same winner (largest |v|, smallest row on
// ties), swaps, scales and updates its rows. ipiv receives k0-based global pivots.
// cand: 2 slots x G x (2 + NB) values, rowj: 2 slots x NB values.
template <class T>
static __global__ void __launch_bounds__(256) lu_panel_kernel(T *P, long long lda, int mrows, int kb, int k0, int rows_per,
                                                       int *ipiv, T *cand, T *rowj, PanelSync *sync, T tiny,
                                                       unsigned long long wait_ns) {
    constexpr int NB = PanelNB<T>::value;
    constexpr int LDR = NB + 1;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    T *R = reinterpret_cast<T *>(smem_raw);  // rows_per x LDR
    T *prow = R + (size_t)rows_per * LDR;    // pivot row copy (NB)
    __shared__ T s_v[8];
    __shared__ int s_i[8];
    const int G = gridDim.x, g = blockIdx.x, tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int r0 = g * rows_per, r1 = min(mrows, r0 + rows_per), nr = max(0, r1 - r0);
    const int CS = 2 + NB;  // candidate record: |v|, row, then the row's values

    // Identity pivots first: a launch that stops early (error or timeout) still leaves
    // in-range pivots for the row swaps that follow it on the stream.
    if (g == 0)
        for (int j = tid; j < kb; j += blockDim.x) ipiv[j] = k0 + j;
    for (int idx = tid; idx < nr * kb; idx += blockDim.x) {
        const int r = idx / kb, c = idx - r * kb;
        R[r * LDR + c] = P[(long long)(r0 + r) * lda + c];
    }
    __syncthreads();
    __shared__ int s_q[8];
    for (int j = 0; j < kb; j++) {
        const int slot = j & 1;
        T bv = T(-1);
        int bi = INT_MAX;
        for (int r = max(j - r0, 0) + tid; r < nr; r += blockDim.x) {
            const T v = absT(R[r * LDR + j]);
            if (v > bv) {
                bv = v;
                bi = r0 + r;
            }
        }
        warp_amax(bv, bi);
        if (lane == 0) {
            s_v[warp] = bv;
            s_i[warp] = bi;
        }
        __syncthreads();
        bv = s_v[0];
        bi = s_i[0];
        for (int w = 1; w < (int)(blockDim.x >> 5); w++) amax_combine(bv, bi, s_v[w], s_i[w]);
        T *mine = cand + ((size_t)slot * G + g) * CS;
        if (tid == 0) {
            mine[0] = bv;
            mine[1] = (T)(bi == INT_MAX ? -1 : bi);
        }
        if (bi != INT_MAX && tid < kb) mine[2 + tid] = R[(bi - r0) * LDR + tid];
        if (j >= r0 && j < r1 && tid < kb) rowj[slot * NB + tid] = R[(j - r0) * LDR + tid];
        if (!grid_barrier(&sync->ctr, (unsigned)(G * (j + 1)), &sync->err, wait_ns)) return;
        // Winner over all CTAs, identical in every CTA: thread q reads CTA q's candidate,
        // then a block argmax (largest |v|, smallest row on ties).
        T wv = T(-1);
        int wi = INT_MAX, wg = -1;
        for (int q = tid; q < G; q += blockDim.x) {
            const volatile T *c = cand + ((size_t)slot * G + q) * CS;
            const T v = c[0];
            const int i = (int)c[1];
            if (i >= 0 && (v > wv || (v == wv && i < wi))) {
                wv = v;
                wi = i;
                wg = q;
            }
        }
        warp_amax3(wv, wi, wg);
        __syncthreads();  // s_v / s_i of the local argmax are read no more
        if (lane == 0) {
            s_v[warp] = wv;
            s_i[warp] = wi;
            s_q[warp] = wg;
        }
        __syncthreads();
        wv = s_v[0];
        wi = s_i[0];
        wg = s_q[0];
        for (int w = 1; w < (int)(blockDim.x >> 5); w++)
            if (s_v[w] > wv || (s_v[w] == wv && s_i[w] < wi)) {
                wv = s_v[w];
                wi = s_i[w];
                wg = s_q[w];
            }
        if (wi == INT_MAX) {  // no finite candidate (NaN column): keep the diagonal
            wi = j;
            wg = -1;
        }
        if (wg >= 0 && wv < tiny) {
            if (g == 0 && tid == 0) atomicCAS(&sync->err, 0, RL_ERR_DIV_BY_ZERO);
            return;
        }
        if (tid < kb) {
            T v;
            if (wg >= 0)
                v = ((volatile T *)(cand + ((size_t)slot * G + wg) * CS))[2 + tid];
            else
                v = ((volatile T *)rowj)[slot * NB + tid];
            prow[tid] = v;
        }
        __syncthreads();
        if (wi != j) {
            if (j >= r0 && j < r1 && tid < kb) R[(j - r0) * LDR + tid] = prow[tid];
            if (wi >= r0 && wi < r1 && tid < kb) R[(wi - r0) * LDR + tid] = ((volatile T *)rowj)[slot * NB + tid];
        }
        if (g == 0 && tid == 0) ipiv[j] = k0 + wi;
        __syncthreads();
        const T inv_p = T(1) / prow[j];  // multipliers by the reciprocal: one division per column
        for (int r = max(j + 1 - r0, 0) + tid; r < nr; r += blockDim.x) {
            T *row = R + r * LDR;
            const T l = row[j] * inv_p;
            row[j] = l;
            for (int c = j + 1; c < kb; c++) row[c] = fma(-l, prow[c], row[c]);
        }
        __syncthreads();
    }
    for (int idx = tid; idx < nr * kb; idx += blockDim.x) {
        const int r = idx / kb, c = idx - r * kb;
        P[(long long)(r0 + r) * lda + c] = R[r * LDR + c];
    }
}

// |v| as an unsigned key that orders like |v| (non-negative IEEE values order like
// their bits), 0 for NaN, which never wins: the pivot search compares keys on the
// integer pipe. On GB300 an FP64 comparison issues on the FP64 pipe, which a warp
// occupies for tens of cycles; the integer form also keeps FP32 and FP64 alike.
__device__ __forceinline__ unsigned long long amax_key(float v) {
    const unsigned u = __float_as_uint(v) & 0x7fffffffu;
    return u > 0x7f800000u ? 0ull : (unsigned long long)u + 1ull;
}
__device__ __forceinline__ unsigned long long amax_key(double v) {
    const unsigned long long u = (unsigned long long)__double_as_longlong(v) & 0x7fffffffffffffffull;
    return u > 0x7ff0000000000000ull ? 0ull : u + 1ull;
}

// Largest key over the warp and the smallest index among the lanes holding it, in every
// lane, on the redux instructions (keys of FP32 values fit in 32 bits; FP64 keys are
// reduced high word first). Lanes without a candidate hold key 0 and index INT_MAX.
template <class T>
__device__ __forceinline__ void warp_amax_key(unsigned long long &k, int &i) {
    bool top;
    if (sizeof(T) == 4) {
        const unsigned k32 = (unsigned)k;
        const unsigned kmax = __reduce_max_sync(0xffffffffu, k32);
        top = k32 == kmax;
        k = kmax;
    } else {
        const unsigned hi = (unsigned)(k >> 32), lo = (unsigned)k;
        const unsigned hmax = __reduce_max_sync(0xffffffffu, hi);
        const unsigned lmax = __reduce_max_sync(0xffffffffu, hi == hmax ? lo : 0u);
        top = hi == hmax && lo == lmax;
        k = ((unsigned long long)hmax << 32) | lmax;
    }
    i = (int)__reduce_min_sync(0xffffffffu, top ? (unsigned)i : 0xffffffffu);
}

// LU panel on one thread-block cluster (up to 16 CTAs): the same algorithm as
// lu_panel_kernel with the cross-CTA exchange moved on chip. CTA g owns rows
// [g * rows_per, ...) in shared memory; inside a CTA, `tpr` consecutive threads (1, 2, 4
// or 8) share each row, thread q of a row owning the columns c = q (mod tpr), and thread
// group t the rows t, t + 256 / tpr, ... The panel's row updates run at the SM's FP64
// rate, so spreading a few rows over all four schedulers of every SM of the cluster is
// what shortens a column. Per column:
//   1. each thread searches column j of its rows (the thread that wrote them), the warps
//      reduce on integer keys, one CTA barrier, every thread combines the warps' maxima;
//   2. the CTA pushes its candidate row (and row j, if it holds it) into every CTA's
//      tables with 16-byte remote shared-memory stores, and its record (key, row,
//      1 / pivot);
//   3. one cluster barrier (release / acquire); every warp picks the same winner from
//      its own CTA's table, where the winning row and row j already are;
//   4. the swap and the update run at once, each element stored by one thread: thread
//      c < kb stores column c of the new row j and, for c < j, of row wi; the threads of
//      row wi compute its columns >= j from the old row j; every other row below j
//      updates itself, the multiplier broadcast within the row's threads by a shuffle.
// Tables and records are double-buffered by column parity: a CTA writes slot s again
// only after the next cluster barrier, which every CTA reaches after it has read slot s.
// Every CTA runs the same barrier sequence (a failing pivot is seen by all at the same
// column).
template <class T>
static __global__ void __launch_bounds__(256) lu_panel_cluster_kernel(T *P, long long lda, int mrows, int kb, int k0,
                                                              int rows_per, int tpr, int *ipiv, int *err, T tiny) {
    namespace cg = cooperative_groups;
    constexpr int NB = PanelNB<T>::value;
    constexpr int LDR = NB + 1;
    constexpr int CMAX = 16;
    constexpr int VW = 16 / (int)sizeof(T);  // elements per 16-byte chunk of a row
    extern __shared__ __align__(16) unsigned char smem_raw[];
    T *tab = reinterpret_cast<T *>(smem_raw);  // 2 x CMAX x NB: every CTA's candidate row
    T *rowj = tab + 2 * CMAX * NB;             // 2 x NB: row j (pushed by the CTA holding it)
    T *R = rowj + 2 * NB;                      // rows_per x LDR
    __shared__ unsigned long long s_k[8], rec_k[2 * CMAX];
    __shared__ int s_i[8], rec_i[2 * CMAX];
    __shared__ T rec_inv[2 * CMAX];
    cg::cluster_group cluster = cg::this_cluster();
    const int C = (int)cluster.num_blocks(), g = (int)cluster.block_rank();
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int r0 = g * rows_per, r1 = min(mrows, r0 + rows_per), nr = max(0, r1 - r0);
    const int q = tid & (tpr - 1), grp = tid / tpr, G = (int)blockDim.x / tpr;
    const int rpt = (rows_per + G - 1) / G;  // rows per thread group, the same in every thread
    const unsigned long long ktiny = amax_key(tiny);
    if (g == 0)
        for (int j = tid; j < kb; j += blockDim.x) ipiv[j] = k0 + j;
    for (int idx = tid; idx < nr * kb; idx += blockDim.x) {
        const int r = idx / kb, c = idx - r * kb;
        R[r * LDR + c] = P[(long long)(r0 + r) * lda + c];
    }
    __syncthreads();
    for (int j = 0; j < kb; j++) {
        const int slot = j & 1, qj = j & (tpr - 1);
        // 1. local candidate
        unsigned long long bk = 0ull;
        int bi = INT_MAX;
        if (q == qj)
            for (int k = 0; k < rpt; k++) {
                const int r = grp + k * G;
                if (r < nr && r0 + r >= j) {
                    const unsigned long long key = amax_key(R[r * LDR + j]);
                    if (key > bk) {
                        bk = key;
                        bi = r0 + r;
                    }
                }
            }
        warp_amax_key<T>(bk, bi);
        if (lane == 0) {
            s_k[warp] = bk;
            s_i[warp] = bi;
        }
        __syncthreads();  // also: every row's update for the previous column is done
        bk = s_k[0];
        bi = s_i[0];
        for (int w = 1; w < (int)(blockDim.x >> 5); w++) {
            const unsigned long long k2 = s_k[w];
            const int i2 = s_i[w];
            if (k2 > bk || (k2 == bk && i2 < bi)) {
                bk = k2;
                bi = i2;
            }
        }
        // 2. push the candidate row (and row j, from the CTA holding it) into every CTA's
        // tables in 16-byte stores, and the record
        const int nch = (kb + VW - 1) / VW;
        if (bk != 0ull)
            for (int idx = tid; idx < C * nch; idx += blockDim.x) {
                const int dst = idx / nch, ch = idx - dst * nch;
                const T *src = R + (size_t)(bi - r0) * LDR + ch * VW;
                uint4 v;
                T *vt = reinterpret_cast<T *>(&v);
#pragma unroll
                for (int e = 0; e < VW; e++) vt[e] = src[e];
                *reinterpret_cast<uint4 *>(cluster.map_shared_rank(tab + (slot * CMAX + g) * NB + ch * VW, dst)) = v;
            }
        if (j >= r0 && j < r1)
            for (int idx = tid; idx < C * nch; idx += blockDim.x) {
                const int dst = idx / nch, ch = idx - dst * nch;
                const T *src = R + (size_t)(j - r0) * LDR + ch * VW;
                uint4 v;
                T *vt = reinterpret_cast<T *>(&v);
#pragma unroll
                for (int e = 0; e < VW; e++) vt[e] = src[e];
                *reinterpret_cast<uint4 *>(cluster.map_shared_rank(rowj + slot * NB + ch * VW, dst)) = v;
            }
        if (warp == 0) {
            const T inv = bk != 0ull ? T(1) / R[(bi - r0) * LDR + j] : T(0);
            if (lane < C) {
                const int e = slot * CMAX + g;
                *cluster.map_shared_rank(rec_k + e, lane) = bk;
                *cluster.map_shared_rank(rec_i + e, lane) = bk != 0ull ? bi : INT_MAX;
                *cluster.map_shared_rank(rec_inv + e, lane) = inv;
            }
        }
        cluster.sync();
        // 3. the winner, the same in every warp of every CTA
        unsigned long long wk = lane < C ? rec_k[slot * CMAX + lane] : 0ull;
        int wi = lane < C ? rec_i[slot * CMAX + lane] : INT_MAX;
        warp_amax_key<T>(wk, wi);
        int wg = -1;
        if (wk != 0ull) {
            if (wk < ktiny) {  // the same decision in every CTA
                if (g == 0 && tid == 0) atomicCAS(err, 0, RL_ERR_DIV_BY_ZERO);
                break;
            }
            wg = wi / rows_per;
        } else {  // no finite candidate (NaN column): keep the diagonal
            wi = j;
        }
        const T *oldj = rowj + slot * NB;                                // the old row j
        const T *prow = wg >= 0 ? tab + (slot * CMAX + wg) * NB : oldj;  // the pivot row
        if (g == 0 && tid == 0) ipiv[j] = k0 + wi;
        const T inv_p = wg >= 0 ? rec_inv[slot * CMAX + wg] : T(1) / oldj[j];
        // 4. swap and update
        if (wi != j && tid < kb) {
            if (j >= r0 && j < r1) R[(j - r0) * LDR + tid] = prow[tid];
            if (wi >= r0 && wi < r1 && tid < j) R[(wi - r0) * LDR + tid] = oldj[tid];
        }
        const int cfirst = j + 1 + ((q - j - 1) & (tpr - 1));  // this thread's first column > j
        for (int k = 0; k < rpt; k++) {
            const int r = grp + k * G, gr = r0 + r;
            const bool valid = r < nr && gr > j;
            T *row = R + (size_t)(valid ? r : 0) * LDR;
            const T *src = gr == wi ? oldj : row;
            T l = T(0);
            if (valid && q == qj) l = src[j] * inv_p;
            if (tpr > 1) l = __shfl_sync(0xffffffffu, l, qj, tpr);
            if (valid) {
                if (q == qj) row[j] = l;
#pragma unroll 4
                for (int c = cfirst; c < kb; c += tpr) row[c] = fma(-l, prow[c], src[c]);
            }
        }
    }
    __syncthreads();
    for (int idx = tid; idx < nr * kb; idx += blockDim.x) {
        const int r = idx / kb, c = idx - r * kb;
        P[(long long)(r0 + r) * lda + c] = R[r * LDR + c];
    }
    cluster.sync();  // no CTA leaves while another may still read its shared memory
}

// The same panel with look-ahead across columns. After column j's winner is known a CTA
// updates only column j + 1 of its rows, finds its candidate for column j + 1, completes
// that candidate row (and row j + 1, if it holds it), pushes them and ARRIVES at the
// cluster barrier; the rest of column j's elimination (columns j + 2 .. kb - 1 of its
// other rows) runs while the barrier completes, and the CTA WAITS only before reading
// column j + 1's records. Every element gets the same fma(-l, u, a) as in
// lu_panel_cluster_kernel, so the factors and pivots are identical. The tables have three
// slots: a CTA may push column j + 1 while another still eliminates with column j - 1's
// pivot row.
__device__ __forceinline__ void cluster_arrive() { asm volatile("barrier.cluster.arrive.release.aligned;" ::: "memory"); }
__device__ __forceinline__ void cluster_wait() { asm volatile("barrier.cluster.wait.acquire.aligned;" ::: "memory"); }

template <class T>
static __global__ void __launch_bounds__(256) lu_panel_cluster_la_kernel(T *P, long long lda, int mrows, int kb, int k0,
                                                                  int rows_per, int tpr, int *ipiv, int *err, T tiny) {
    namespace cg = cooperative_groups;
    constexpr int NB = PanelNB<T>::value;
    constexpr int LDR = NB + 1;
    constexpr int CMAX = 16, NS = 3;
    constexpr int VW = 16 / (int)sizeof(T);
    extern __shared__ __align__(16) unsigned char smem_raw[];
    T *tab = reinterpret_cast<T *>(smem_raw);  // NS x CMAX x NB: every CTA's candidate row
    T *rowj = tab + NS * CMAX * NB;            // NS x NB: row j (pushed by the CTA holding it)
    T *R = rowj + NS * NB;                     // rows_per x LDR
    __shared__ unsigned long long s_k[8], rec_k[NS * CMAX];
    __shared__ int s_i[8], rec_i[NS * CMAX];
    __shared__ T rec_inv[NS * CMAX];
    cg::cluster_group cluster = cg::this_cluster();
    const int C = (int)cluster.num_blocks(), g = (int)cluster.block_rank();
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int r0 = g * rows_per, r1 = min(mrows, r0 + rows_per), nr = max(0, r1 - r0);
    const int q = tid & (tpr - 1), grp = tid / tpr, G = (int)blockDim.x / tpr;
    const int rpt = (rows_per + G - 1) / G;
    const unsigned long long ktiny = amax_key(tiny);
    const int nch = (kb + VW - 1) / VW;
    if (g == 0)
        for (int j = tid; j < kb; j += blockDim.x) ipiv[j] = k0 + j;
    for (int idx = tid; idx < nr * kb; idx += blockDim.x) {
        const int r = idx / kb, c = idx - r * kb;
        R[r * LDR + c] = P[(long long)(r0 + r) * lda + c];
    }
    __syncthreads();
    // candidate of this CTA for column c (rows >= c; thread group q == c mod tpr scans)
    auto candidate = [&](int c, unsigned long long &bk, int &bi) {
        bk = 0ull;
        bi = INT_MAX;
        if (q == (c & (tpr - 1)))
            for (int k = 0; k < rpt; k++) {
                const int r = grp + k * G;
                if (r < nr && r0 + r >= c) {
                    const unsigned long long key = amax_key(R[r * LDR + c]);
                    if (key > bk) {
                        bk = key;
                        bi = r0 + r;
                    }
                }
            }
        warp_amax_key<T>(bk, bi);
        if (lane == 0) {
            s_k[warp] = bk;
            s_i[warp] = bi;
        }
        __syncthreads();
        bk = s_k[0];
        bi = s_i[0];
        for (int w = 1; w < (int)(blockDim.x >> 5); w++) {
            const unsigned long long k2 = s_k[w];
            const int i2 = s_i[w];
            if (k2 > bk || (k2 == bk && i2 < bi)) {
                bk = k2;
                bi = i2;
            }
        }
    };
    // push the candidate row bi (complete) and row c (if held) into every CTA's slot for
    // column c, with the record; then arrive
    auto push = [&](int c, unsigned long long bk, int bi) {
        const int slot = c % NS;
        if (bk != 0ull)
            for (int idx = tid; idx < C * nch; idx += blockDim.x) {
                const int dst = idx / nch, ch = idx - dst * nch;
                const T *src = R + (size_t)(bi - r0) * LDR + ch * VW;
                uint4 v;
                T *vt = reinterpret_cast<T *>(&v);
#pragma unroll
                for (int e = 0; e < VW; e++) vt[e] = src[e];
                *reinterpret_cast<uint4 *>(cluster.map_shared_rank(tab + (slot * CMAX + g) * NB + ch * VW, dst)) = v;
            }
        if (c >= r0 && c < r1)
            for (int idx = tid; idx < C * nch; idx += blockDim.x) {
                const int dst = idx / nch, ch = idx - dst * nch;
                const T *src = R + (size_t)(c - r0) * LDR + ch * VW;
                uint4 v;
                T *vt = reinterpret_cast<T *>(&v);
#pragma unroll
                for (int e = 0; e < VW; e++) vt[e] = src[e];
                *reinterpret_cast<uint4 *>(cluster.map_shared_rank(rowj + slot * NB + ch * VW, dst)) = v;
            }
        if (warp == 0) {
            const T inv = bk != 0ull ? T(1) / R[(bi - r0) * LDR + c] : T(0);
            if (lane < C) {
                const int e = slot * CMAX + g;
                *cluster.map_shared_rank(rec_k + e, lane) = bk;
                *cluster.map_shared_rank(rec_i + e, lane) = bk != 0ull ? bi : INT_MAX;
                *cluster.map_shared_rank(rec_inv + e, lane) = inv;
            }
        }
        cluster_arrive();
    };
    {
        unsigned long long bk;
        int bi;
        candidate(0, bk, bi);
        push(0, bk, bi);
    }
    int skip0 = -1, skip1 = -1;  // rows completed before their push (not eliminated again)
    for (int j = 0; j < kb; j++) {
        const int slot = j % NS, qj = j & (tpr - 1);
        cluster_wait();  // column j's records and rows are in every CTA's tables
        unsigned long long wk = lane < C ? rec_k[slot * CMAX + lane] : 0ull;
        int wi = lane < C ? rec_i[slot * CMAX + lane] : INT_MAX;
        warp_amax_key<T>(wk, wi);
        int wg = -1;
        if (wk != 0ull) {
            if (wk < ktiny) {
                if (g == 0 && tid == 0) atomicCAS(err, 0, RL_ERR_DIV_BY_ZERO);
                break;
            }
            wg = wi / rows_per;
        } else {
            wi = j;
        }
        const T *oldj = rowj + slot * NB;
        const T *prow = wg >= 0 ? tab + (slot * CMAX + wg) * NB : oldj;
        if (g == 0 && tid == 0) ipiv[j] = k0 + wi;
        const T inv_p = wg >= 0 ? rec_inv[slot * CMAX + wg] : T(1) / oldj[j];
        if (wi != j && tid < kb) {
            if (j >= r0 && j < r1) R[(j - r0) * LDR + tid] = prow[tid];
            if (wi >= r0 && wi < r1 && tid < j) R[(wi - r0) * LDR + tid] = oldj[tid];
        }
        // (a) multipliers and column j + 1 of every row below j
        const int q1 = (j + 1) & (tpr - 1);
        for (int k = 0; k < rpt; k++) {
            const int r = grp + k * G, gr = r0 + r;
            const bool valid = r < nr && gr > j;
            T *row = R + (size_t)(valid ? r : 0) * LDR;
            const T *src = gr == wi ? oldj : row;
            T l = T(0);
            if (valid && q == qj) l = src[j] * inv_p;
            if (tpr > 1) l = __shfl_sync(0xffffffffu, l, qj, tpr);
            if (valid) {
                if (q == qj) row[j] = l;
                if (j + 1 < kb && q == q1) row[j + 1] = fma(-l, prow[j + 1], src[j + 1]);
            }
        }
        if (j + 1 >= kb) break;
        // (b) the candidate for column j + 1 (the barrier inside also orders (a))
        unsigned long long bk;
        int bi;
        candidate(j + 1, bk, bi);
        // (c) complete the rows pushed for column j + 1: the candidate and row j + 1
        skip0 = bk != 0ull ? bi : -1;
        skip1 = (j + 1 >= r0 && j + 1 < r1) ? j + 1 : -1;
        for (int t = 0; t < 2; t++) {
            const int gr = t == 0 ? skip0 : skip1;
            if (gr < 0 || (t == 1 && gr == skip0)) continue;
            T *row = R + (size_t)(gr - r0) * LDR;
            const T *src = gr == wi ? oldj : row;
            const T l = row[j];
            for (int c = j + 2 + tid; c < kb; c += blockDim.x) row[c] = fma(-l, prow[c], src[c]);
        }
        __syncthreads();
        push(j + 1, bk, bi);
        // (d) the rest of column j's elimination, while the barrier completes
        const int cfirst = j + 2 + ((q - j - 2) & (tpr - 1));
        for (int k = 0; k < rpt; k++) {
            const int r = grp + k * G, gr = r0 + r;
            if (r >= nr || gr <= j || gr == skip0 || gr == skip1) continue;
            T *row = R + (size_t)r * LDR;
            const T *src = gr == wi ? oldj : row;
            const T l = row[j];
#pragma unroll 4
            for (int c = cfirst; c < kb; c += tpr) row[c] = fma(-l, prow[c], src[c]);
        }
    }
    __syncthreads();
    for (int idx = tid; idx < nr * kb; idx += blockDim.x) {
        const int r = idx / kb, c = idx - r * kb;
        P[(long long)(r0 + r) * lda + c] = R[r * LDR + c];
    }
    cluster.sync();  // no CTA leaves while another may still read its shared memory
}

// ------------------------------------------------------------ Householder panel --
// Unblocked Householder QR of the panel rows [0, mrows) x cols [0, kb) (P points at
// A[k0][k0]), reflector by reflector exactly as HouseholderReflection::compute and
// buffered_left_multiply_into (householder.rs:32-130) but with the reductions split
// over CTAs: sigma = dot(x[1..], x[1..]) and u = A^T v are summed from per-CTA partials
// in CTA order after a grid barrier. Two barriers per column. tau receives kb values.
// part: 2 slots x G x (1 + NB) partial sums; x0buf: 2 slots.
template <class T>
static __global__ void __launch_bounds__(256) qr_panel_kernel(T *P, long long lda, int mrows, int kb, int rows_per, T *tau,
                                                       T *part, T *x0buf, PanelSync *sync,
                                                       unsigned long long wait_ns) {
    constexpr int NB = PanelNB<T>::value;
    constexpr int LDR = NB + 1;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    T *R = reinterpret_cast<T *>(smem_raw);  // rows_per x LDR
    T *u = R + (size_t)rows_per * LDR;       // NB
    __shared__ T s_red[8][NB + 1];
    const int G = gridDim.x, g = blockIdx.x, tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int nw = blockDim.x >> 5;
    const int r0 = g * rows_per, r1 = min(mrows, r0 + rows_per), nr = max(0, r1 - r0);
    const int PS = 1 + NB;
    for (int idx = tid; idx < nr * kb; idx += blockDim.x) {
        const int r = idx / kb, c = idx - r * kb;
        R[r * LDR + c] = P[(long long)(r0 + r) * lda + c];
    }
    __syncthreads();
    unsigned phase = 0;
    for (int j = 0; j < kb; j++) {
        const int slot = j & 1;
        // (1) sigma partial over rows > j, in row order per thread then tree order.
        T s = T(0);
        for (int r = max(j + 1 - r0, 0) + tid; r < nr; r += blockDim.x) {
            const T v = R[r * LDR + j];
            s = fma(v, v, s);
        }
        s = warp_sum(s);
        if (lane == 0) s_red[warp][0] = s;
        __syncthreads();
        if (tid == 0) {
            T t = T(0);
            for (int w = 0; w < nw; w++) t += s_red[w][0];
            part[((size_t)slot * G + g) * PS] = t;
            if (j >= r0 && j < r1) x0buf[slot] = R[(j - r0) * LDR + j];
        }
        if (!grid_barrier(&sync->ctr, (unsigned)(G * (++phase)), &sync->err, wait_ns)) return;
        // sigma = sum of the CTAs' partials, a fixed tree over q (thread q, then warps)
        T sigma = T(0);
        for (int q = tid; q < G; q += blockDim.x) sigma += ((volatile T *)part)[((size_t)slot * G + q) * PS];
        sigma = warp_sum(sigma);
        __syncthreads();  // s_red from step (1) is read no more
        if (lane == 0) s_red[warp][0] = sigma;
        __syncthreads();
        sigma = T(0);
        for (int w = 0; w < nw; w++) sigma += s_red[w][0];
        const T x0 = ((volatile T *)x0buf)[slot];
        if (sigma == T(0)) {  // already a multiple of e1: tau = 0, nothing changes
            if (g == 0 && tid == 0) tau[j] = T(0);
            if (!grid_barrier(&sync->ctr, (unsigned)(G * (++phase)), &sync->err, wait_ns)) return;
            continue;
        }
        const T x_norm = sqrt(x0 * x0 + sigma);
        const T v0 = x0 > T(0) ? x0 + x_norm : x0 - x_norm;
        const T two = T(2);
        const T t = two * v0 * v0 / (v0 * v0 + sigma);
        if (g == 0 && tid == 0) tau[j] = t;
        // (2) u_c = sum_r v_r a[r][c] for c >= j over owned rows r >= j, with
        // v_r = x_r / v0 (v_j = 1) formed on the fly so that column j still holds x.
        for (int c = j + warp; c < kb; c += nw) {
            T acc = T(0);
            for (int r = max(j - r0, 0) + lane; r < nr; r += 32) {
                const T vr = (r0 + r == j) ? T(1) : R[r * LDR + j] / v0;
                acc = fma(vr, R[r * LDR + c], acc);
            }
            acc = warp_sum(acc);
            if (lane == 0) part[((size_t)slot * G + g) * PS + 1 + c] = acc;
        }
        if (!grid_barrier(&sync->ctr, (unsigned)(G * (++phase)), &sync->err, wait_ns)) return;
        // u_c = sum over CTAs of the partials: warp per column, lanes over CTAs
        for (int c = j + warp; c < kb; c += nw) {
            T a = T(0);
            for (int q = lane; q < G; q += 32) a += ((volatile T *)part)[((size_t)slot * G + q) * PS + 1 + c];
            a = warp_sum(a);
            if (lane == 0) u[c] = a;
        }
        __syncthreads();
        // (3) a[r][c] += (-tau v_r) u_c for c > j (ger, internal_utils.rs:67-83); the
        // diagonal becomes x0 - tau u_j and v[1..] is stored below it (store_in_col).
        for (int r = max(j - r0, 0) + tid; r < nr; r += blockDim.x) {
            T *row = R + r * LDR;
            const bool diag = (r0 + r == j);
            const T vr = diag ? T(1) : row[j] / v0;
            const T sc = -t * vr;
            for (int c = j + 1; c < kb; c++) row[c] = fma(sc, u[c], row[c]);
            row[j] = diag ? x0 - t * u[j] : vr;
        }
        __syncthreads();
    }
    for (int idx = tid; idx < nr * kb; idx += blockDim.x) {
        const int r = idx / kb, c = idx - r * kb;
        P[(long long)(r0 + r) * lda + c] = R[r * LDR + c];
    }
}

// Householder panel on one thread-block cluster (up to 16 CTAs): qr_panel_kernel's
// algorithm with the two cross-CTA sums per column (sigma, then u = A^T v) exchanged on
// chip. Each CTA pushes its partial sums (and x0, from the CTA holding row j) into every
// CTA's tables by remote shared-memory stores before a cluster barrier; after it every
// CTA adds the C partials from its own tables in rank order, so all compute the same tau
// and u with no remote read on the critical path. v_r = a_rj / v0 is formed once per
// row (it was formed again for every column of the u sums). The tables are written for
// column j + 1 only after the barrier that every CTA reaches once it has read them for
// column j. A column with sigma = 0 still passes the second barrier, so every CTA runs
// the same barrier sequence.
template <class T>
static __global__ void __launch_bounds__(256) qr_panel_cluster_kernel(T *P, long long lda, int mrows, int kb,
                                                              int rows_per, T *tau) {
    namespace cg = cooperative_groups;
    constexpr int NB = PanelNB<T>::value;
    constexpr int LDR = NB + 1;
    constexpr int CMAX = 16;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    T *R = reinterpret_cast<T *>(smem_raw);  // rows_per x LDR
    T *vb = R + (size_t)rows_per * LDR;      // rows_per: this column's v for the owned rows
    T *u = vb + rows_per;                    // NB: this column's u
    T *up_tab = u + NB;                      // CMAX x NB: every CTA's partial of u
    T *sig_tab = up_tab + CMAX * NB;         // CMAX: every CTA's partial of sigma
    T *x0_slot = sig_tab + CMAX;             // 1: x0 = a_jj from the CTA holding row j
    __shared__ T s_red[8];
    cg::cluster_group cluster = cg::this_cluster();
    const int C = (int)cluster.num_blocks(), g = (int)cluster.block_rank();
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int nw = blockDim.x >> 5;
    const int r0 = g * rows_per, r1 = min(mrows, r0 + rows_per), nr = max(0, r1 - r0);
    for (int idx = tid; idx < nr * kb; idx += blockDim.x) {
        const int r = idx / kb, c = idx - r * kb;
        R[r * LDR + c] = P[(long long)(r0 + r) * lda + c];
    }
    __syncthreads();
    for (int j = 0; j < kb; j++) {
        // (1) sigma partial over rows > j, pushed (with x0) to every CTA
        T sp = T(0);
        for (int r = max(j + 1 - r0, 0) + tid; r < nr; r += blockDim.x) {
            const T v = R[r * LDR + j];
            sp = fma(v, v, sp);
        }
        sp = warp_sum(sp);
        if (lane == 0) s_red[warp] = sp;
        __syncthreads();
        if (tid < C) {
            T t = T(0);
            for (int w = 0; w < nw; w++) t += s_red[w];
            *cluster.map_shared_rank(sig_tab + g, tid) = t;
            if (j >= r0 && j < r1) *cluster.map_shared_rank(x0_slot, tid) = R[(j - r0) * LDR + j];
        }
        cluster.sync();
        // sigma over the CTAs in rank order (lane q holds CTA q's partial)
        if (warp == 0) {
            T sigma = lane < C ? sig_tab[lane] : T(0);
            sigma = warp_sum(sigma);
            if (lane == 0) s_red[0] = sigma;
        }
        __syncthreads();
        const T sigma = s_red[0];
        const T x0 = *x0_slot;
        if (sigma == T(0)) {  // already a multiple of e1: tau = 0, nothing changes
            if (g == 0 && tid == 0) tau[j] = T(0);
            cluster.sync();
            continue;
        }
        const T x_norm = sqrt(x0 * x0 + sigma);
        const T v0 = x0 > T(0) ? x0 + x_norm : x0 - x_norm;
        const T two = T(2);
        const T t = two * v0 * v0 / (v0 * v0 + sigma);
        if (g == 0 && tid == 0) tau[j] = t;
        // v of the owned rows below the diagonal (stored into the panel by the update)
        for (int r = max(j + 1 - r0, 0) + tid; r < nr; r += blockDim.x) vb[r] = R[r * LDR + j] / v0;
        __syncthreads();
        // (2) u_c partial = sum_r v_r a[r][c] for c >= j over owned rows r >= j, pushed
        for (int c = j + warp; c < kb; c += nw) {
            T acc = T(0);
            for (int r = max(j - r0, 0) + lane; r < nr; r += 32) {
                const T vr = (r0 + r == j) ? T(1) : vb[r];
                acc = fma(vr, R[r * LDR + c], acc);
            }
            acc = __shfl_sync(0xffffffffu, warp_sum(acc), 0);  // lane 0's sum, in every lane
            if (lane < C) *cluster.map_shared_rank(up_tab + g * NB + c, lane) = acc;
        }
        cluster.sync();
        if (tid >= j && tid < kb) {
            T a = T(0);
            for (int q = 0; q < C; q++) a += up_tab[q * NB + tid];
            u[tid] = a;
        }
        __syncthreads();
        // (3) a[r][c] += (-tau v_r) u_c for c > j; the diagonal becomes x0 - tau u_j and
        // v[1..] stays below it
        for (int r = max(j - r0, 0) + tid; r < nr; r += blockDim.x) {
            T *row = R + r * LDR;
            const bool diag = (r0 + r == j);
            const T vr = diag ? T(1) : vb[r];
            const T sc = -t * vr;
            for (int c = j + 1; c < kb; c++) row[c] = fma(sc, u[c], row[c]);
            row[j] = diag ? x0 - t * u[j] : vr;
        }
        __syncthreads();
    }
    for (int idx = tid; idx < nr * kb; idx += blockDim.x) {
        const int r = idx / kb, c = idx - r * kb;
        P[(long long)(r0 + r) * lda + c] = R[r * LDR + c];
    }
    cluster.sync();  // no CTA leaves while another may still store into its shared memory
}

// ------------------------------------------------------------------- row swaps --
// Applies ipiv[j0..j1) (global rows; step j swaps rows j and ipiv[j]) to the columns
// [0, c_skip0) and [c_skip1, ncols) of A, 64 columns per CTA, in blocks of 64 pivots:
// the rows a block touches (its own 64 rows and the pivot rows outside them, at most
// 128) are staged in shared memory with all loads in flight at once, the block's swaps
// run there in order (thread per column), and the rows are written back. A swap chain
// applied straight to global memory would wait one memory round trip per pivot.
constexpr int kSwapCols = 64, kSwapBlock = 64;
template <class T>
static __global__ void __launch_bounds__(256) laswp_kernel(T *A, long long lda, int ncols, int c_skip0, int c_skip1,
                                                    const int *ipiv, int j0, int j1) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    T *S = reinterpret_cast<T *>(smem_raw);  // 2 * kSwapBlock slots x kSwapCols columns
    __shared__ int s_piv[kSwapBlock], s_slot[kSwapBlock], s_row[2 * kSwapBlock];
    const int tid = threadIdx.x, t = tid & (kSwapCols - 1), quarter = tid / kSwapCols;
    const int nother = ncols - (c_skip1 - c_skip0);
    const int c = blockIdx.x * kSwapCols + t;
    const bool act = c < nother;
    const int gc = c < c_skip0 ? c : c + (c_skip1 - c_skip0);
    for (int b = j0; b < j1; b += kSwapBlock) {
        const int kb = min(kSwapBlock, j1 - b);
        if (tid < kb) s_piv[tid] = ipiv[b + tid];
        __syncthreads();
        // slot of each pivot row: its place in [b, b + kb), else an outside slot named
        // by the first step that swaps it in (the slot that stages it)
        if (tid < kb) {
            const int p = s_piv[tid];
            int sl;
            if (p >= b && p < b + kb) {
                sl = p - b;
            } else {
                int first = tid;
                for (int u = 0; u < tid; u++)
                    if (s_piv[u] == p) {
                        first = u;
                        break;
                    }
                sl = kSwapBlock + first;
            }
            s_slot[tid] = sl;
            s_row[tid] = b + tid;
            s_row[kSwapBlock + tid] = sl == kSwapBlock + tid ? p : -1;
        } else if (tid < kSwapBlock) {
            s_row[tid] = -1;
            s_row[kSwapBlock + tid] = -1;
        }
        __syncthreads();
        if (act) {
            T v[2 * kSwapBlock / 4];
#pragma unroll
            for (int i = 0; i < 2 * kSwapBlock / 4; i++) {
                const int r = s_row[quarter + 4 * i];
                v[i] = r >= 0 ? A[(long long)r * lda + gc] : T(0);
            }
#pragma unroll
            for (int i = 0; i < 2 * kSwapBlock / 4; i++) S[(quarter + 4 * i) * kSwapCols + t] = v[i];
        }
        __syncthreads();
        if (act && quarter == 0)
            for (int u = 0; u < kb; u++) {
                const int sl = s_slot[u];
                if (sl != u) {
                    const T x = S[u * kSwapCols + t];
                    S[u * kSwapCols + t] = S[sl * kSwapCols + t];
                    S[sl * kSwapCols + t] = x;
                }
            }
        __syncthreads();
        if (act)
#pragma unroll 4
            for (int i = 0; i < 2 * kSwapBlock / 4; i++) {
                const int sl = quarter + 4 * i, r = s_row[sl];
                if (r >= 0) A[(long long)r * lda + gc] = S[sl * kSwapCols + t];
            }
        __syncthreads();  // the staging area and slot map are reused by the next block
    }
}

// Launch of laswp_kernel over the columns outside [c_skip0, c_skip1).
template <class T>
rl_status laswp(T *A, long long lda, int ncols, int c_skip0, int c_skip1, const int *ipiv, int j0, int j1,
                cudaStream_t s) {
    const int nother = ncols - (c_skip1 - c_skip0);
    if (nother <= 0 || j1 <= j0) return RL_OK;
    const size_t smem = sizeof(T) * 2 * kSwapBlock * kSwapCols;
    static const cudaError_t attr =
        cudaFuncSetAttribute(laswp_kernel<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    RL_TRY_CUDA(attr);
    RL_LAUNCH(laswp_kernel<T>, ceil_div(nother, kSwapCols), 256, smem, s, A, lda, ncols, c_skip0, c_skip1, ipiv, j0, j1);
    return RL_OK;
}

// ------------------------------------------------------- diagonal-block solves --
// Solves op(D) X = Y in place for the bs x bs diagonal block D (bs <= 64, row stride
// ldd) and Y = bs x nrhs (row stride ldy). mode 0: D unit lower; 1: D lower; 2: D upper;
// 3: D^T with D lower (L^T). |d_ii| < tiny (modes 1-3) records RL_ERR_DIV_BY_ZERO in
// status and leaves Y unchanged. CTA per 8 columns, warp per 2 columns, 16 lanes per
// column each holding 4 of its rows in registers: step j broadcasts x_j within the
// column's lanes by a shuffle and every lane updates its rows, y_i -= d_ij x_j in
// increasing j (the order of the reference's substitution). The FP64 work of a U12
// solve is spread over every scheduler of every SM instead of a few CTAs' threads.
constexpr int kTrsmCols = 8;
template <class T>
static __global__ void __launch_bounds__(128) trsm_diag_kernel(const T *D, long long ldd, int bs, T *Y, long long ldy,
                                                        int nrhs, int mode, int *status, T tiny) {
    __shared__ T Ds[64][65];
    __shared__ T Ys[64][kTrsmCols];
    __shared__ int s_bad;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int c0 = blockIdx.x * kTrsmCols;
    if (tid == 0) s_bad = 0;
    for (int idx = tid; idx < bs * bs; idx += blockDim.x) {
        const int i = idx / bs, j = idx - i * bs;
        Ds[i][j] = D[(long long)i * ldd + j];
    }
    for (int idx = tid; idx < 64 * kTrsmCols; idx += blockDim.x) {
        const int i = idx / kTrsmCols, cc = idx - i * kTrsmCols;
        Ys[i][cc] = (i < bs && c0 + cc < nrhs) ? Y[(long long)i * ldy + c0 + cc] : T(0);
    }
    __syncthreads();
    if (mode != 0 && tid < bs && absT(Ds[tid][tid]) < tiny) s_bad = 1;
    __syncthreads();
    if (s_bad) {
        if (tid == 0) atomicCAS(status, 0, RL_ERR_DIV_BY_ZERO);
        return;
    }
    const int col = 2 * warp + (lane >> 4), r16 = lane & 15;
    T y[4];
#pragma unroll
    for (int sl = 0; sl < 4; sl++) y[sl] = Ys[16 * sl + r16][col];
    if (mode <= 1) {
#pragma unroll
        for (int j = 0; j < 64; j++) {
            if (j < bs) {
                if (mode == 1 && r16 == (j & 15)) y[j >> 4] = y[j >> 4] / Ds[j][j];
                const T xj = __shfl_sync(0xffffffffu, y[j >> 4], j & 15, 16);
#pragma unroll
                for (int sl = j >> 4; sl < 4; sl++) {
                    const int i = 16 * sl + r16;
                    if (i > j && i < bs) y[sl] = fma(-Ds[i][j], xj, y[sl]);
                }
            }
        }
    } else {
#pragma unroll
        for (int j = 63; j >= 0; j--) {
            if (j < bs) {
                if (r16 == (j & 15)) y[j >> 4] = y[j >> 4] / Ds[j][j];
                const T xj = __shfl_sync(0xffffffffu, y[j >> 4], j & 15, 16);
#pragma unroll
                for (int sl = 0; sl <= (j >> 4); sl++) {
                    const int i = 16 * sl + r16;
                    if (i < j) y[sl] = fma(-(mode == 2 ? Ds[i][j] : Ds[j][i]), xj, y[sl]);
                }
            }
        }
    }
    __syncthreads();
#pragma unroll
    for (int sl = 0; sl < 4; sl++) Ys[16 * sl + r16][col] = y[sl];
    __syncthreads();
    for (int idx = tid; idx < bs * kTrsmCols; idx += blockDim.x) {
        const int i = idx / kTrsmCols, cc = idx - i * kTrsmCols;
        if (c0 + cc < nrhs) Y[(long long)i * ldy + c0 + cc] = Ys[i][cc];
    }
}

// ------------------------------------------- few-right-hand-side triangular sweep --
// op(A) X = Y in place for nrhs <= 8 right-hand sides in ONE launch of at most
// kSweepCtas CTAs: each CTA takes 64-row blocks of the solution in solve order by an
// atomic ticket (forward for modes 0 / 1, backward for modes 2 / 3; the modes are those
// of tri_solve_dev), one after another. A block folds in the contribution of every block
// solved before it as each one is published (its flag in ctl), overlapping that GEMV
// work with the blocks still being solved, then solves its diagonal block by
// substitution (one warp per right-hand side, the multipliers by the diagonal's
// reciprocals) and publishes its rows. A CTA waits only on tickets taken before its own,
// by CTAs that are running, so the sweep always progresses; a waiting thread sleeps
// between polls (other streams' kernels share the SMs), and every wait is bounded by
// wait_ns (RL_TUNE_WAIT_TIMEOUT_NS; RL_ERR_TIMEOUT). withhold >= 0 is a test setting
// (RL_TUNE_TEST_WITHHOLD_SWEEP_BLOCK): that block is solved but never published, so the
// waits for it run out. With Dinv (the inverses of the operated diagonal blocks, 64 x 64
// row-major per block, from diag_inverse_kernel) a block's solve is the product
// x_b = Dinv_b (y_b - folded sums), 16-term dot products over all 256 threads, instead
// of the 64-step substitution chain: in FP64 that chain's dependent DFMAs cost ~20 us
// per block on this part.
// More than kSweepRhs right-hand sides run as groups of kSweepRhs columns side by side:
// blockIdx.y is the group, with its own ticket and block flags; groups never wait on one
// another.
// Per-launch state, per group g: ctl[g (1 + nb)] = ticket, ctl[g (1 + nb) + 1 + b] =
// block b published, zeroed by the host.
constexpr int kSweepRows = 64, kSweepRhs = 8, kSweepCtas = 32, kSweepGroups = 16;

// Right-hand-side groups of a sweep over nrhs columns, 0 when the sweep does not take
// them (more than kSweepGroups groups); ctl words it needs for n rows.
inline int sweep_groups(int nrhs) {
    const int g = (nrhs + kSweepRhs - 1) / kSweepRhs;
    return g <= kSweepGroups ? g : 0;
}
inline int sweep_ctl_words(int n, int nrhs) {
    return sweep_groups(nrhs) * (1 + (n + kSweepRows - 1) / kSweepRows);
}
template <class T, class TA = T, int RW = kSweepRhs>
static __global__ void __launch_bounds__(256) trsv_sweep_kernel(const TA *__restrict__ A, long long lda, int n,
                                                             T *__restrict__ Y, long long ldy, int nrhs, int mode,
                                                             int *ctl, int *status, T tiny,
                                                             unsigned long long wait_ns, int withhold,
                                                             const T *__restrict__ Dinv) {
    constexpr int BR = kSweepRows, LDD = BR + 1;
    constexpr int FB = sizeof(T) == 4 ? 8 : 2;  // published blocks folded per barrier round
    __shared__ T Ds[BR * LDD];                  // the diagonal block
    __shared__ T inv[BR];                        // 1 / d_ii
    __shared__ T xs[FB * BR * kSweepRhs];        // a round's published solutions, then the folded sums
    __shared__ int s_t, s_fail, s_m;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int nb = (n + BR - 1) / BR;
    const bool fwd = mode <= 1, trans = mode == 3;
    // this CTA's group of right-hand sides
    Y += (long long)blockIdx.y * kSweepRhs;
    nrhs = min(kSweepRhs, nrhs - (int)blockIdx.y * kSweepRhs);
    ctl += (long long)blockIdx.y * (1 + nb);
    if (tid == 0) s_fail = 0;
    for (;;) {
        __syncthreads();  // the previous block's shared state is no longer read
        if (tid == 0) s_t = atomicAdd(ctl, 1);
        __syncthreads();
        if (s_t >= nb) break;
        const int b = fwd ? s_t : nb - 1 - s_t, r0 = b * BR, bs = min(BR, n - r0);
        // Loads that do not wait on other blocks, issued before the fold: this block's
        // right-hand-side rows (only this block writes them) and, with Dinv, its row of
        // the inverted diagonal block; first read after the fold, off the chain.
        const int rr = tid >> 2, qq = tid & 3;
        T dpre[16], ypre[2];
        if (Dinv) {
            const T *Db = Dinv + (long long)b * BR * BR + (long long)rr * BR + qq * 16;
    #pragma unroll
            for (int jj = 0; jj < 16; jj++) dpre[jj] = (rr < bs && qq * 16 + jj < bs) ? Db[jj] : T(0);
    #pragma unroll
            for (int h = 0; h < 2; h++) {
                const int idx = tid + h * 256, i = idx / nrhs, c = idx - i * nrhs;
                ypre[h] = idx < bs * nrhs ? __ldcg(Y + (long long)(r0 + i) * ldy + c) : T(0);
            }
        } else {
    #pragma unroll
            for (int h = 0; h < 2; h++) {
                const int i = lane + 32 * h;
                ypre[h] = (warp < nrhs && i < bs) ? __ldcg(Y + (long long)(r0 + i) * ldy + warp) : T(0);
            }
        }
        // the diagonal block and its reciprocal diagonal: no dependence on other blocks
        if (!Dinv)
            for (int idx = tid; idx < bs * bs; idx += blockDim.x) {
                const int i = idx / bs, j = idx - i * bs;
                Ds[i * LDD + j] = T(A[(long long)(r0 + i) * lda + r0 + j]);
            }
        __syncthreads();
        if (tid < bs && !Dinv) {
            const T d = Ds[tid * LDD + tid];
            if (mode != 0 && absT(d) < tiny) atomicCAS(status, 0, RL_ERR_DIV_BY_ZERO);
            inv[tid] = mode == 0 ? T(1) : T(1) / d;
        }
        // thread (row r, quarter q): non-transposed reads A[r][q * 16 + jj] (a thread's 16
        // columns contiguous), transposed reads A[q * 16 + jj][r] (a warp's rows contiguous)
        const int r = trans ? (tid & (BR - 1)) : (tid >> 2), q = trans ? (tid >> 6) : (tid & 3);
        T acc[RW];
    #pragma unroll
        for (int c = 0; c < RW; c++) acc[c] = T(0);
        const int nk = fwd ? b : nb - 1 - b;  // blocks solved before this one
        // The fold, in rounds of up to FB published blocks: thread 0 waits (bounded) for the
        // round's first block and takes the consecutive published ones after it; their
        // solutions go to shared memory under one barrier, and the round's products run
        // without barriers between blocks. (One block per round cost three barriers and a
        // dependent memory round trip per earlier block: O(b) latencies for block b.) Each
        // thread adds the blocks in the same order as before, so the sums are unchanged.
        for (int kk0 = 0; kk0 < nk;) {
            // FP32, one right-hand side: the A tile of the block about to be waited for is
            // loaded before the wait (with 8 right-hand sides the extra registers cost more)
            constexpr bool PRE = sizeof(T) == 4 && RW == 1;
            T apre[PRE ? 16 : 1];
            if (PRE) {
                const int k = fwd ? kk0 : nb - 1 - kk0, c0 = k * BR, ks = min(BR, n - c0);
    #pragma unroll
                for (int jj = 0; jj < (PRE ? 16 : 1); jj++) {
                    const int j = q * 16 + jj;
                    apre[jj] = (r < bs && j < ks)
                                   ? T(trans ? A[(long long)(c0 + j) * lda + r0 + r] : A[(long long)(r0 + r) * lda + c0 + j])
                                   : T(0);
                }
            }
            if (tid == 0 && !s_fail) {
                const int k = fwd ? kk0 : nb - 1 - kk0;
                const unsigned long long t0 = global_ns();
                while (ld_acquire(ctl + 1 + k) == 0) {
                    if (global_ns() - t0 > wait_ns) {
                        s_fail = 1;
                        break;
                    }
                    __nanosleep(100);
                }
                int m = 1;
                while (!s_fail && m < FB && kk0 + m < nk &&
                       ld_acquire(ctl + 1 + (fwd ? kk0 + m : nb - 1 - (kk0 + m))) != 0)
                    m++;
                s_m = m;
            }
            __syncthreads();
            if (s_fail) break;
            const int m = s_m;
            // rows ks..BR-1 of a short last block are zeroed: they meet a[jj] = 0, and a
            // stale shared value there could be a NaN (0 * NaN = NaN)
            for (int idx = tid; idx < m * BR * nrhs; idx += blockDim.x) {
                const int u = idx / (BR * nrhs), rem = idx - u * (BR * nrhs), i = rem / nrhs, c = rem - i * nrhs;
                const int k = fwd ? kk0 + u : nb - 1 - (kk0 + u), c0 = k * BR, ks = min(BR, n - c0);
                xs[(u * BR + i) * kSweepRhs + c] = i < ks ? __ldcg(Y + (long long)(c0 + i) * ldy + c) : T(0);
            }
            __syncthreads();
    #pragma unroll 2
            for (int u = 0; u < m; u++) {
                const int k = fwd ? kk0 + u : nb - 1 - (kk0 + u), c0 = k * BR, ks = min(BR, n - c0);
                T a[16];
    #pragma unroll
                for (int jj = 0; jj < 16; jj++) {
                    const int j = q * 16 + jj;
                    if (PRE && u == 0)
                        a[jj] = apre[PRE ? jj : 0];
                    else
                        a[jj] = (r < bs && j < ks)
                                    ? T(trans ? A[(long long)(c0 + j) * lda + r0 + r] : A[(long long)(r0 + r) * lda + c0 + j])
                                    : T(0);
                }
    #pragma unroll
                for (int jj = 0; jj < 16; jj++) {
                    const int j = q * 16 + jj;
    #pragma unroll
                    for (int c = 0; c < RW; c++)
                        if (c < nrhs) acc[c] = fma(a[jj], xs[(u * BR + j) * kSweepRhs + c], acc[c]);
                }
            }
            __syncthreads();  // xs is refilled by the next round
            kk0 += m;
        }
        // sum of the 4 column quarters of each row into xs
        if (!trans) {
    #pragma unroll
            for (int c = 0; c < RW; c++) {
                acc[c] += __shfl_xor_sync(0xffffffffu, acc[c], 1);
                acc[c] += __shfl_xor_sync(0xffffffffu, acc[c], 2);
            }
            if (q == 0)
    #pragma unroll
                for (int c = 0; c < RW; c++) xs[r * kSweepRhs + c] = acc[c];
            __syncthreads();
        } else {
            for (int qq = 0; qq < 4; qq++) {
                if (q == qq)
    #pragma unroll
                    for (int c = 0; c < RW; c++) xs[r * kSweepRhs + c] = (qq ? xs[r * kSweepRhs + c] : T(0)) + acc[c];
                __syncthreads();
            }
        }
        if (Dinv) {
            // x_b = Dinv_b v, v = y_b - folded sums (in xs); thread (row rr, quarter qq)
    #pragma unroll
            for (int h = 0; h < 2; h++) {
                const int idx = tid + h * 256, i = idx / nrhs, c = idx - i * nrhs;
                if (idx < bs * nrhs) xs[i * kSweepRhs + c] = ypre[h] - xs[i * kSweepRhs + c];
            }
            __syncthreads();
            T xo[RW];
    #pragma unroll
            for (int c = 0; c < RW; c++) xo[c] = T(0);
    #pragma unroll
            for (int jj = 0; jj < 16; jj++) {
                const int j = qq * 16 + jj;
    #pragma unroll
                for (int c = 0; c < RW; c++)
                    if (c < nrhs) xo[c] = fma(dpre[jj], xs[j * kSweepRhs + c], xo[c]);
            }
    #pragma unroll
            for (int c = 0; c < RW; c++) {
                xo[c] += __shfl_xor_sync(0xffffffffu, xo[c], 1);
                xo[c] += __shfl_xor_sync(0xffffffffu, xo[c], 2);
            }
            if (qq == 0 && rr < bs && !s_fail)
    #pragma unroll
                for (int c = 0; c < RW; c++)
                    if (c < nrhs) __stcg(Y + (long long)(r0 + rr) * ldy + c, xo[c]);
        }
        // substitution: warp c solves right-hand side c; lane l holds rows l and l + 32
        if (!Dinv && warp < nrhs && !s_fail) {
            const int c = warp;
            T y[2];
    #pragma unroll
            for (int h = 0; h < 2; h++) {
                const int i = lane + 32 * h;
                T v = T(0);
                if (i < bs) v = ypre[h] - xs[i * kSweepRhs + c];
                y[h] = v;
            }
            if (fwd) {
                for (int k = 0; k < bs; k++) {
                    const int h = k >> 5;
                    T xk = __shfl_sync(0xffffffffu, h ? y[1] : y[0], k & 31) * inv[k];
                    if (lane == (k & 31)) {
                        if (h)
                            y[1] = xk;
                        else
                            y[0] = xk;
                    }
    #pragma unroll
                    for (int hh = 0; hh < 2; hh++) {
                        const int i = lane + 32 * hh;
                        if (i > k && i < bs) y[hh] = fma(-Ds[i * LDD + k], xk, y[hh]);
                    }
                }
            } else {
                for (int k = bs - 1; k >= 0; k--) {
                    const int h = k >> 5;
                    T xk = __shfl_sync(0xffffffffu, h ? y[1] : y[0], k & 31) * inv[k];
                    if (lane == (k & 31)) {
                        if (h)
                            y[1] = xk;
                        else
                            y[0] = xk;
                    }
    #pragma unroll
                    for (int hh = 0; hh < 2; hh++) {
                        const int i = lane + 32 * hh;
                        if (i < k) y[hh] = fma(-(trans ? Ds[k * LDD + i] : Ds[i * LDD + k]), xk, y[hh]);
                    }
                }
            }
    #pragma unroll
            for (int h = 0; h < 2; h++) {
                const int i = lane + 32 * h;
                if (i < bs) __stcg(Y + (long long)(r0 + i) * ldy + c, y[h]);
            }
        }
        __syncthreads();
        if (tid == 0) {
            if (s_fail) atomicCAS(status, 0, RL_ERR_TIMEOUT);
            __threadfence();
            // published even after a timeout, so no later block waits forever
            if (b != withhold) st_release(ctl + 1 + b, 1);
        }
    }
}

// Dinv_b = op(D_b)^-1 for every 64 x 64 diagonal block D_b of A (n x n, stored as TA),
// formed in T, one CTA per block: 64 threads, thread j solving op(D_b) x = e_j by
// substitution (op and the unit diagonal as in trsv_sweep_kernel's modes). Written
// row-major 64 x 64 per block, zero beyond a partial last block. |d_ii| < tiny records
// RL_ERR_DIV_BY_ZERO.
template <class T, class TA>
static __global__ void __launch_bounds__(64) diag_inverse_kernel(const TA *__restrict__ A, long long lda, int n, int mode,
                                                             T *__restrict__ Dinv, int *status, T tiny) {
    constexpr int BR = kSweepRows;
    __shared__ T M[BR][BR + 1];  // op(D_b)
    __shared__ T X[BR][BR + 1];  // column j: thread j's solution
    const int b = blockIdx.x, r0 = b * BR, bs = min(BR, n - r0), j = threadIdx.x;
    for (int idx = j; idx < BR * BR; idx += blockDim.x) {
        const int r = idx / BR, c = idx - r * BR;
        T v = T(0);
        if (r < bs && c < bs)
            v = T(mode == 3 ? A[(long long)(r0 + c) * lda + r0 + r] : A[(long long)(r0 + r) * lda + r0 + c]);
        M[r][c] = v;
        X[r][c] = T(0);
    }
    __syncthreads();
    const bool unit = mode == 0, lower = mode <= 1;
    if (j < bs) {
        if (!unit && absT(M[j][j]) < tiny) atomicCAS(status, 0, RL_ERR_DIV_BY_ZERO);
        if (lower) {
            for (int i = j; i < bs; i++) {
                T v = i == j ? T(1) : T(0);
                for (int k = j; k < i; k++) v = fma(-M[i][k], X[k][j], v);
                X[i][j] = unit ? v : v / M[i][i];
            }
        } else {
            for (int i = j; i >= 0; i--) {
                T v = i == j ? T(1) : T(0);
                for (int k = i + 1; k <= j; k++) v = fma(-M[i][k], X[k][j], v);
                X[i][j] = v / M[i][i];
            }
        }
    }
    __syncthreads();
    T *out = Dinv + (long long)b * BR * BR;
    for (int idx = j; idx < BR * BR; idx += blockDim.x) out[idx] = X[idx / BR][idx % BR];
}

// Row-wise solve X D^T = Y for the rows of Y (m x bs, stride ldy), D lower bs x bs:
// the Cholesky panel L21 = A21 L11^-T. Thread per row.
template <class T>
static __global__ void __launch_bounds__(128) trsm_right_lt_kernel(const T *D, long long ldd, int bs, T *Y, long long ldy,
                                                            int m) {
    __shared__ T Ds[64][65];
    for (int idx = threadIdx.x; idx < bs * bs; idx += blockDim.x) {
        const int i = idx / bs, j = idx - i * bs;
        Ds[i][j] = D[(long long)i * ldd + j];
    }
    __syncthreads();
    const int r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= m) return;
    T *y = Y + (long long)r * ldy;
    T x[64];
#pragma unroll
    for (int j = 0; j < 64; j++)
        if (j < bs) x[j] = y[j];
#pragma unroll
    for (int j = 0; j < 64; j++) {
        if (j < bs) {
            T s = x[j];
#pragma unroll
            for (int i = 0; i < 64; i++)
                if (i < j) s = fma(-x[i], Ds[j][i], s);
            x[j] = s / Ds[j][j];
        }
    }
#pragma unroll
    for (int j = 0; j < 64; j++)
        if (j < bs) y[j] = x[j];
}

// ------------------------------------------------------------- compact WY helpers --
// V (mrows x kb, row stride kb) = the panel's reflectors with the implicit unit diagonal
// and zeros above it.
template <class T>
static __global__ void extract_v_kernel(const T *P, long long lda, int mrows, int kb, T *V) {
    const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= (long long)mrows * kb) return;
    const int r = (int)(idx / kb), c = (int)(idx - (long long)r * kb);
    V[idx] = r > c ? P[(long long)r * lda + c] : (r == c ? T(1) : T(0));
}

// Partial Gram matrices of the reflector block V (mrows x kb, row stride kb, kb <= 64):
// CTA c sums V[r]^T V[r] over its chunk of rows into part[c] (64 x 64). A plain GEMM of
// this 64 x 64 product over thousands of rows is one tile, one CTA, one long K loop.
constexpr int kGramRows = 256;  // rows per chunk
template <class T>
static __global__ void __launch_bounds__(256) gram_partial_kernel(const T *__restrict__ V, int mrows, int kb,
                                                                  T *__restrict__ part) {
    __shared__ T Vs[32][64];
    const int tid = threadIdx.x, tx = tid & 15, ty = tid >> 4;
    const int rbeg = blockIdx.x * kGramRows, rend = min(mrows, rbeg + kGramRows);
    T acc[4][4];
#pragma unroll
    for (int a = 0; a < 4; a++)
#pragma unroll
        for (int b = 0; b < 4; b++) acc[a][b] = T(0);
    for (int r0 = rbeg; r0 < rend; r0 += 32) {
        for (int idx = tid; idx < 32 * 64; idx += 256) {
            const int r = idx >> 6, c = idx & 63;
            Vs[r][c] = (r0 + r < rend && c < kb) ? V[(long long)(r0 + r) * kb + c] : T(0);
        }
        __syncthreads();
#pragma unroll 4
        for (int r = 0; r < 32; r++) {
            T va[4], vb[4];
#pragma unroll
            for (int a = 0; a < 4; a++) va[a] = Vs[r][4 * ty + a];
#pragma unroll
            for (int b = 0; b < 4; b++) vb[b] = Vs[r][4 * tx + b];
#pragma unroll
            for (int a = 0; a < 4; a++)
#pragma unroll
                for (int b = 0; b < 4; b++) acc[a][b] = fma(va[a], vb[b], acc[a][b]);
        }
        __syncthreads();
    }
    T *out = part + (size_t)blockIdx.x * 64 * 64;
#pragma unroll
    for (int a = 0; a < 4; a++)
#pragma unroll
        for (int b = 0; b < 4; b++) out[(4 * ty + a) * 64 + 4 * tx + b] = acc[a][b];
}

// T factor of H_0 ... H_{kb-1} = I - V T V^T (upper triangular, kb x kb): the Gram
// matrix Gm = V^T V is the sum of the nparts partial Gram matrices (added in part order),
// then T[j][j] = tau_j, T[0:j, j] = -tau_j T[0:j, 0:j] Gm[0:j, j], all in shared memory.
template <class T>
static __global__ void __launch_bounds__(256) larft_kernel(const T *part, int nparts, const T *tau, int kb, T *Tm) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    T (*G)[65] = reinterpret_cast<T (*)[65]>(smem_raw);  // 64 x 65 each
    T (*Ts)[65] = G + 64;
    __shared__ T w[64];
    const int t = threadIdx.x;
    for (int idx = t; idx < 64 * 64; idx += blockDim.x) {
        T sum = T(0);
        for (int c = 0; c < nparts; c++) sum += part[(size_t)c * 64 * 64 + idx];
        G[idx >> 6][idx & 63] = sum;
        Ts[idx >> 6][idx & 63] = T(0);
    }
    __syncthreads();
    for (int j = 0; j < kb; j++) {
        const T tj = tau[j];
        if (t < j) {
            T s = T(0);
            for (int q = t; q < j; q++) s = fma(Ts[t][q], G[q][j], s);
            w[t] = -tj * s;
        }
        __syncthreads();
        if (t < j) Ts[t][j] = w[t];
        if (t == 0) Ts[j][j] = tj;
        __syncthreads();
    }
    for (int idx = t; idx < kb * kb; idx += blockDim.x) Tm[idx] = Ts[idx / kb][idx % kb];
}

// Identity-like start for first_k_columns: Q (m x k) = I[:, 0:k].
template <class T>
static __global__ void eye_kernel(T *Q, long long ldq, int m, int k) {
    const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= (long long)m * k) return;
    const int r = (int)(idx / k), c = (int)(idx - (long long)r * k);
    Q[(long long)r * ldq + c] = r == c ? T(1) : T(0);
}

// Gathers rows: Y[perm[i]][:] = B[i][:] (the reference's P * b, applied to nrhs columns).
template <class T>
static __global__ void permute_rows_kernel(const T *B, long long ldb, T *Y, long long ldy, int n, int nrhs,
                                    const uint64_t *perm) {
    const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= (long long)n * nrhs) return;
    const int i = (int)(idx / nrhs), c = (int)(idx - (long long)i * nrhs);
    Y[(long long)perm[i] * ldy + c] = B[(long long)i * ldb + c];
}

// det helpers: sequential fold of the diagonal in row order (the reference's fold), and
// the parity of a stored permutation by cycle resolution (permutation_matrix.rs:479-509).
template <class T>
static __global__ void det_kernel(const T *A, long long lda, int n, const uint64_t *perm, uint64_t *scratch, int square,
                           T *out) {
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    T d = T(1);
    for (int i = 0; i < n; i++) d = d * A[(long long)i * lda + i];
    if (square) {
        out[0] = d * d;
        return;
    }
    int odd = 0;
    if (perm) {
        for (int i = 0; i < n; i++) scratch[i] = perm[i];
        for (int i = 0; i < n; i++) {
            uint64_t target = scratch[i];
            while ((uint64_t)i != target) {
                const uint64_t nt = scratch[target];
                odd ^= 1;
                scratch[target] = target;
                target = nt;
            }
            scratch[i] = i;
        }
    }
    const T p_det = odd ? T(0) - T(1) : T(1);
    out[0] = p_det * d;
}

}  // namespace rl
