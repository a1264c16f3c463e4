// One-CTA dense factorisations and solves for systems with n <= CTA_NMAX (512).
//
// A CTA of CTA_THREADS threads owns one matrix that lives in global memory (L2-resident
// at these sizes) and runs a right-looking blocked algorithm over it:
//   * the current column panel (rows k0..n, NB columns) is staged in shared memory
//     column-major, factored there column by column (block-wide warp-shuffle argmax for
//     the LU pivot, first maximum on ties as in PartialPivLu::decompose,
//     src/matrix/decomposition/lu.rs:169-178), and written back;
//   * the panel's row swaps are applied to the other columns with each thread owning
//     whole columns, so rows move as contiguous (coalesced) runs;
//   * L11^-1 is formed once per panel (warp-shuffle forward substitution); per 64-column
//     slice, U12 = L11^-1 A12 is a small shared-memory GEMM, followed by the trailing
//     update A22 -= L21 U12 as 64x64 register-tiled blocks with L21 read from the
//     shared-memory panel.
// Cholesky uses the same panel machinery (the panel is the whole column block, so the
// diagonal block and L21 are factored together) followed by a lower-triangle SYRK.
// The factor type T is float (mixed precision) or double (plain FP64).
#pragma once

#include <climits>

#include "common.cuh"

namespace rl {

constexpr int CTA_THREADS = 256;
constexpr int CTA_WARPS = CTA_THREADS / 32;
constexpr int CTA_NMAX = 512;
constexpr int CTA_LDP = CTA_NMAX + 64;  // panel column stride (slack for 64-row tiles)

template <class T>
struct CtaNB;
template <>
struct CtaNB<float> {
    static constexpr int value = 32;
};
template <>
struct CtaNB<double> {
    static constexpr int value = 16;
};

// Shared-memory workspace of one CTA (dynamic shared memory).
template <class T>
struct CtaSmem {
    static constexpr int NB = CtaNB<T>::value;
    T P[NB * CTA_LDP];     // panel, column-major: P[c * CTA_LDP + r]
    T Bt[NB * 64];         // one 64-column slice of U12
    T Linv[NB * (NB + 1)]; // L11^-1 of the current LU panel
    T w[CTA_NMAX];         // factor-precision right-hand side / solution
    double x[CTA_NMAX];    // FP64 solution (refinement)
    double r[CTA_NMAX];    // FP64 residual
    int piv[CTA_NMAX];     // LAPACK-style pivots: step j swapped rows j and piv[j]
    double redd[CTA_WARPS * 2];
    T redv[CTA_WARPS];
    int redi[CTA_WARPS];
    int status;
    int item;
};

__device__ __forceinline__ float absT(float v) { return fabsf(v); }
__device__ __forceinline__ double absT(double v) { return fabs(v); }

template <class T>
__device__ __forceinline__ void ld4(const T *p, T (&o)[4]);
template <>
__device__ __forceinline__ void ld4<float>(const float *p, float (&o)[4]) {
    float4 v = *reinterpret_cast<const float4 *>(p);
    o[0] = v.x, o[1] = v.y, o[2] = v.z, o[3] = v.w;
}
template <>
__device__ __forceinline__ void ld4<double>(const double *p, double (&o)[4]) {
    double2 a = reinterpret_cast<const double2 *>(p)[0], b = reinterpret_cast<const double2 *>(p)[1];
    o[0] = a.x, o[1] = a.y, o[2] = b.x, o[3] = b.y;
}

// (|v|, index) maximum with the smallest index winning ties.
template <class T>
__device__ __forceinline__ void amax_combine(T &v, int &i, T v2, int i2) {
    if (v2 > v || (v2 == v && i2 < i)) {
        v = v2;
        i = i2;
    }
}

template <class T>
__device__ __forceinline__ void warp_amax(T &v, int &i) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        T v2 = __shfl_xor_sync(0xffffffffu, v, o);
        int i2 = __shfl_xor_sync(0xffffffffu, i, o);
        amax_combine(v, i, v2, i2);
    }
}

template <class T>
__device__ __forceinline__ T warp_sum(T v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}
template <class T>
__device__ __forceinline__ T warp_max(T v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v = fmax(v, __shfl_xor_sync(0xffffffffu, v, o));
    return v;
}

// Block-wide max of a double; every thread gets the result. Uses redd[0..WARPS).
template <class T>
__device__ double block_max(double v, CtaSmem<T> &S) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    v = warp_max(v);
    __syncthreads();
    if (lane == 0) S.redd[warp] = v;
    __syncthreads();
    double m = S.redd[0];
#pragma unroll
    for (int w = 1; w < CTA_WARPS; w++) m = fmax(m, S.redd[w]);
    return m;
}

// ---------------------------------------------------------------------------- LU --
// Factors the n x n matrix A (row stride lda) in place; S.piv receives the pivots.
// A pivot with |p| < tiny returns RL_ERR_DIV_BY_ZERO (tiny = epsilon reproduces the
// reference rule of lu.rs:179-183). Uniform across the CTA.
template <class T>
__device__ int cta_lu_factor(T *__restrict__ A, int lda, int n, CtaSmem<T> &S, T tiny) {
    constexpr int NB = CtaNB<T>::value;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    for (int k0 = 0; k0 < n; k0 += NB) {
        const int kb = min(NB, n - k0), mrows = n - k0;
        for (int idx = tid; idx < mrows * kb; idx += CTA_THREADS) {
            const int r = idx / kb, c = idx - r * kb;
            S.P[c * CTA_LDP + r] = A[(long long)(k0 + r) * lda + k0 + c];
        }
        __syncthreads();
        for (int j = 0; j < kb; j++) {
            T *col = S.P + j * CTA_LDP;
            T bv = T(-1);
            int bi = INT_MAX;
            for (int r = j + tid; r < mrows; r += CTA_THREADS) {
                const T v = absT(col[r]);
                if (v > bv) {
                    bv = v;
                    bi = r;
                }
            }
            warp_amax(bv, bi);
            if (lane == 0) {
                S.redv[warp] = bv;
                S.redi[warp] = bi;
            }
            __syncthreads();
            bv = S.redv[0];
            bi = S.redi[0];
#pragma unroll
            for (int w = 1; w < CTA_WARPS; w++) amax_combine(bv, bi, S.redv[w], S.redi[w]);
            if (bi == INT_MAX) {  // column of NaNs: keep the diagonal, as the reference does
                bi = j;
                bv = absT(col[j]);
            }
            if (bv < tiny) {
                __syncthreads();
                return RL_ERR_DIV_BY_ZERO;
            }
            if (bi != j && tid < kb) {
                T *cc = S.P + tid * CTA_LDP;
                const T t = cc[j];
                cc[j] = cc[bi];
                cc[bi] = t;
            }
            if (tid == 0) S.piv[k0 + j] = k0 + bi;
            __syncthreads();
            const T p = col[j];
            for (int r = j + 1 + tid; r < mrows; r += CTA_THREADS) {
                const T l = col[r] / p;
                col[r] = l;
                for (int c = j + 1; c < kb; c++) S.P[c * CTA_LDP + r] = fma(-l, S.P[c * CTA_LDP + j], S.P[c * CTA_LDP + r]);
            }
            __syncthreads();
        }
        for (int idx = tid; idx < mrows * kb; idx += CTA_THREADS) {
            const int r = idx / kb, c = idx - r * kb;
            A[(long long)(k0 + r) * lda + k0 + c] = S.P[c * CTA_LDP + r];
        }
        // Row swaps of this panel on all other columns: each thread owns whole columns
        // and replays the panel's swaps in order.
        for (int c = tid; c < n - kb; c += CTA_THREADS) {
            const int gc = c < k0 ? c : c + kb;
            for (int j = 0; j < kb; j++) {
                const int pr = S.piv[k0 + j];
                if (pr != k0 + j) {
                    T *a0 = A + (long long)(k0 + j) * lda + gc;
                    T *a1 = A + (long long)pr * lda + gc;
                    const T t = *a0;
                    *a0 = *a1;
                    *a1 = t;
                }
            }
        }
        __syncthreads();
        const int n2 = n - k0 - kb;
        if (n2 <= 0) continue;
        // L11^-1 (unit lower, NB x NB) by warp-shuffle forward substitution: warp w
        // solves L11 x = e_j for columns j = w, w + 8, ...; lane i holds x_i.
        for (int j = warp; j < NB; j += CTA_WARPS) {
            T x = (lane == j) ? T(1) : T(0);
            for (int k = j; k < NB - 1; k++) {
                const T xk = __shfl_sync(0xffffffffu, x, k);
                if (lane > k && lane < NB) x = fma(-S.P[k * CTA_LDP + lane], xk, x);
            }
            if (lane < NB) S.Linv[lane * (NB + 1) + j] = x;
        }
        __syncthreads();
        // Per 64-column slice: U12 = L11^-1 A12 as a small shared-memory GEMM (written
        // back to A), then A22 -= L21 * U12 over all row tiles, 4 x 4 outputs per thread.
        const int m2 = mrows - kb;
        const int tx = tid & 15, ty = tid >> 4;
        constexpr int RPT = NB / 4;  // U12 rows per thread in the slice solve
        for (int tj = 0; tj < n2; tj += 64) {
            for (int idx = tid; idx < NB * 64; idx += CTA_THREADS) {
                const int p = idx >> 6, cc = idx & 63;
                S.Bt[idx] = (tj + cc < n2) ? A[(long long)(k0 + p) * lda + k0 + kb + tj + cc] : T(0);
            }
            __syncthreads();
            {
                const int cc = tid & 63, rg = (tid >> 6) * RPT;
                T u[RPT];
#pragma unroll
                for (int i = 0; i < RPT; i++) u[i] = T(0);
#pragma unroll
                for (int k = 0; k < NB; k++) {
                    const T bk = S.Bt[k * 64 + cc];
#pragma unroll
                    for (int i = 0; i < RPT; i++) u[i] = fma(S.Linv[(rg + i) * (NB + 1) + k], bk, u[i]);
                }
                __syncthreads();
#pragma unroll
                for (int i = 0; i < RPT; i++) {
                    S.Bt[(rg + i) * 64 + cc] = u[i];
                    if (tj + cc < n2) A[(long long)(k0 + rg + i) * lda + k0 + kb + tj + cc] = u[i];
                }
            }
            __syncthreads();
            for (int ti = 0; ti < m2; ti += 64) {
                T acc[4][4];
#pragma unroll
                for (int i = 0; i < 4; i++)
#pragma unroll
                    for (int j = 0; j < 4; j++) acc[i][j] = T(0);
                const int rb = kb + ti + ty * 4;
#pragma unroll 8
                for (int p = 0; p < NB; p++) {
                    T a[4], b[4];
                    ld4<T>(&S.P[p * CTA_LDP + rb], a);
                    ld4<T>(&S.Bt[p * 64 + tx * 4], b);
#pragma unroll
                    for (int i = 0; i < 4; i++)
#pragma unroll
                        for (int j = 0; j < 4; j++) acc[i][j] = fma(a[i], b[j], acc[i][j]);
                }
#pragma unroll
                for (int i = 0; i < 4; i++) {
                    if (rb + i >= mrows) break;
                    T *row = A + (long long)(k0 + rb + i) * lda + k0 + kb + tj + tx * 4;
#pragma unroll
                    for (int j = 0; j < 4; j++)
                        if (tj + tx * 4 + j < n2) row[j] -= acc[i][j];
                }
            }
            __syncthreads();
        }
    }
    return RL_OK;
}

// ---------------------------------------------------------------------- Cholesky --
// Lower Cholesky in place; only the lower triangle is read or written. A diagonal with
// |d| < tiny or d < 0 returns RL_ERR_DECOMP_FAILURE (cholesky.rs:150-158 with
// tiny = epsilon). The diagonal is stored as d / sqrt(d), like cholesky.rs:160-163.
template <class T>
__device__ int cta_chol_factor(T *__restrict__ A, int lda, int n, CtaSmem<T> &S, T tiny) {
    constexpr int NB = CtaNB<T>::value;
    const int tid = threadIdx.x;
    for (int k0 = 0; k0 < n; k0 += NB) {
        const int kb = min(NB, n - k0), mrows = n - k0;
        for (int idx = tid; idx < mrows * kb; idx += CTA_THREADS) {
            const int r = idx / kb, c = idx - r * kb;
            if (r >= c) S.P[c * CTA_LDP + r] = A[(long long)(k0 + r) * lda + k0 + c];
        }
        __syncthreads();
        for (int j = 0; j < kb; j++) {
            T *col = S.P + j * CTA_LDP;
            const T d = col[j];
            if (absT(d) < tiny || d < T(0)) {
                __syncthreads();
                return RL_ERR_DECOMP_FAILURE;
            }
            const T s = sqrt(d);
            __syncthreads();
            for (int r = j + tid; r < mrows; r += CTA_THREADS) col[r] = col[r] / s;
            __syncthreads();
            for (int r = j + 1 + tid; r < mrows; r += CTA_THREADS) {
                const T l = col[r];
                const int cmax = min(kb - 1, r);
                for (int c = j + 1; c <= cmax; c++) S.P[c * CTA_LDP + r] = fma(-l, col[c], S.P[c * CTA_LDP + r]);
            }
            __syncthreads();
        }
        for (int idx = tid; idx < mrows * kb; idx += CTA_THREADS) {
            const int r = idx / kb, c = idx - r * kb;
            if (r >= c) A[(long long)(k0 + r) * lda + k0 + c] = S.P[c * CTA_LDP + r];
        }
        const int m2 = mrows - kb;
        if (m2 <= 0) {
            __syncthreads();
            continue;
        }
        // A22 -= L21 L21^T on the lower triangle; both operands come from the panel.
        const int tx = tid & 15, ty = tid >> 4;
        for (int ti = 0; ti < m2; ti += 64) {
            for (int tj = 0; tj <= ti; tj += 64) {
                T acc[4][4];
#pragma unroll
                for (int i = 0; i < 4; i++)
#pragma unroll
                    for (int j = 0; j < 4; j++) acc[i][j] = T(0);
                const int rb = kb + ti + ty * 4, cb = kb + tj + tx * 4;
#pragma unroll 8
                for (int p = 0; p < NB; p++) {
                    T a[4], b[4];
                    ld4<T>(&S.P[p * CTA_LDP + rb], a);
                    ld4<T>(&S.P[p * CTA_LDP + cb], b);
#pragma unroll
                    for (int i = 0; i < 4; i++)
#pragma unroll
                        for (int j = 0; j < 4; j++) acc[i][j] = fma(a[i], b[j], acc[i][j]);
                }
#pragma unroll
                for (int i = 0; i < 4; i++) {
                    const int r = rb + i;
                    if (r >= mrows) break;
                    T *row = A + (long long)(k0 + r) * lda + k0;
#pragma unroll
                    for (int j = 0; j < 4; j++) {
                        const int c = cb + j;
                        if (c <= r && c < mrows) row[c] -= acc[i][j];
                    }
                }
            }
        }
        __syncthreads();
    }
    return RL_OK;
}

// ------------------------------------------------------------------------- solves --
// In-place solves on the shared vector S.w (already permuted for LU). Triangles are read
// from global memory, 32 x 32 diagonal blocks by warp 0 with shuffles, the rest as
// warp-per-row (or thread-per-column) GEMV updates.

// Unit lower triangular solve L y = w (L strictly below the diagonal of A).
template <class T>
__device__ void cta_unit_lower_solve(const T *__restrict__ A, int lda, int n, CtaSmem<T> &S) {
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    for (int b0 = 0; b0 < n; b0 += 32) {
        const int bs = min(32, n - b0);
        if (warp == 0) {
            T wv = lane < bs ? S.w[b0 + lane] : T(0);
            const T *lrow = A + (long long)(b0 + lane) * lda + b0;
            for (int jj = 0; jj < bs - 1; jj++) {
                const T wj = __shfl_sync(0xffffffffu, wv, jj);
                if (lane > jj && lane < bs) wv = fma(-lrow[jj], wj, wv);
            }
            if (lane < bs) S.w[b0 + lane] = wv;
        }
        __syncthreads();
        for (int i = b0 + bs + warp; i < n; i += CTA_WARPS) {
            T s = lane < bs ? A[(long long)i * lda + b0 + lane] * S.w[b0 + lane] : T(0);
            s = warp_sum(s);
            if (lane == 0) S.w[i] -= s;
        }
        __syncthreads();
    }
}

// Upper triangular solve U x = w (U on and above the diagonal of A). |u_ii| < tiny
// returns RL_ERR_DIV_BY_ZERO (src/matrix/mod.rs:333-336).
template <class T>
__device__ int cta_upper_solve(const T *__restrict__ A, int lda, int n, CtaSmem<T> &S, T tiny) {
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    for (int b1 = n; b1 > 0; b1 -= 32) {
        const int b0 = max(0, b1 - 32), bs = b1 - b0;
        if (warp == 0) {
            int bad = 0;
            T wv = lane < bs ? S.w[b0 + lane] : T(0);
            const T *urow = A + (long long)(b0 + lane) * lda + b0;
            for (int jj = bs - 1; jj >= 0; jj--) {
                const T d = A[(long long)(b0 + jj) * lda + b0 + jj];
                if (absT(d) < tiny) bad = 1;
                if (lane == jj) wv = wv / d;
                const T wj = __shfl_sync(0xffffffffu, wv, jj);
                if (lane < jj) wv = fma(-urow[jj], wj, wv);
            }
            if (lane < bs) S.w[b0 + lane] = wv;
            if (lane == 0) S.status = bad;
        }
        __syncthreads();
        if (S.status) {
            __syncthreads();
            return RL_ERR_DIV_BY_ZERO;
        }
        for (int i = warp; i < b0; i += CTA_WARPS) {
            T s = lane < bs ? A[(long long)i * lda + b0 + lane] * S.w[b0 + lane] : T(0);
            s = warp_sum(s);
            if (lane == 0) S.w[i] -= s;
        }
        __syncthreads();
    }
    return RL_OK;
}

// Lower (non-unit) solve L y = w; |l_ii| < tiny -> RL_ERR_DIV_BY_ZERO (mod.rs:375-378).
template <class T>
__device__ int cta_lower_solve(const T *__restrict__ A, int lda, int n, CtaSmem<T> &S, T tiny) {
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    for (int b0 = 0; b0 < n; b0 += 32) {
        const int bs = min(32, n - b0);
        if (warp == 0) {
            int bad = 0;
            T wv = lane < bs ? S.w[b0 + lane] : T(0);
            const T *lrow = A + (long long)(b0 + lane) * lda + b0;
            for (int jj = 0; jj < bs; jj++) {
                const T d = A[(long long)(b0 + jj) * lda + b0 + jj];
                if (absT(d) < tiny) bad = 1;
                if (lane == jj) wv = wv / d;
                const T wj = __shfl_sync(0xffffffffu, wv, jj);
                if (lane > jj && lane < bs) wv = fma(-lrow[jj], wj, wv);
            }
            if (lane < bs) S.w[b0 + lane] = wv;
            if (lane == 0) S.status = bad;
        }
        __syncthreads();
        if (S.status) {
            __syncthreads();
            return RL_ERR_DIV_BY_ZERO;
        }
        for (int i = b0 + bs + warp; i < n; i += CTA_WARPS) {
            T s = lane < bs ? A[(long long)i * lda + b0 + lane] * S.w[b0 + lane] : T(0);
            s = warp_sum(s);
            if (lane == 0) S.w[i] -= s;
        }
        __syncthreads();
    }
    return RL_OK;
}

// Transposed solve L^T x = w with L lower (cholesky.rs:329-361).
template <class T>
__device__ int cta_lower_t_solve(const T *__restrict__ A, int lda, int n, CtaSmem<T> &S, T tiny) {
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    for (int b1 = n; b1 > 0; b1 -= 32) {
        const int b0 = max(0, b1 - 32), bs = b1 - b0;
        if (warp == 0) {
            int bad = 0;
            T wv = lane < bs ? S.w[b0 + lane] : T(0);
            for (int jj = bs - 1; jj >= 0; jj--) {
                const T *lrow = A + (long long)(b0 + jj) * lda + b0;  // row jj of L = column jj of L^T
                const T d = lrow[jj];
                if (absT(d) < tiny) bad = 1;
                if (lane == jj) wv = wv / d;
                const T wj = __shfl_sync(0xffffffffu, wv, jj);
                if (lane < jj) wv = fma(-lrow[lane], wj, wv);
            }
            if (lane < bs) S.w[b0 + lane] = wv;
            if (lane == 0) S.status = bad;
        }
        __syncthreads();
        if (S.status) {
            __syncthreads();
            return RL_ERR_DIV_BY_ZERO;
        }
        for (int i = tid; i < b0; i += CTA_THREADS) {
            T s = T(0);
            for (int jj = 0; jj < bs; jj++) s = fma(A[(long long)(b0 + jj) * lda + i], S.w[b0 + jj], s);
            S.w[i] -= s;
        }
        __syncthreads();
    }
    return RL_OK;
}

// Applies LAPACK-style pivots (S.piv) to S.w in order.
template <class T>
__device__ void cta_apply_pivots(int n, CtaSmem<T> &S) {
    if (threadIdx.x == 0) {
        for (int j = 0; j < n; j++) {
            const int p = S.piv[j];
            if (p != j) {
                const T t = S.w[j];
                S.w[j] = S.w[p];
                S.w[p] = t;
            }
        }
    }
    __syncthreads();
}

// Full solve with a factor: kind 0 = LU (pivots in S.piv), 1 = Cholesky.
template <class T>
__device__ int cta_factor_solve(const T *A, int lda, int n, int kind, CtaSmem<T> &S, T tiny) {
    if (kind == 1) {
        int st = cta_lower_solve(A, lda, n, S, tiny);
        if (st != RL_OK) return st;
        return cta_lower_t_solve(A, lda, n, S, tiny);
    }
    cta_apply_pivots(n, S);
    cta_unit_lower_solve(A, lda, n, S);
    return cta_upper_solve(A, lda, n, S, tiny);
}

// FP64 residual S.r = b - A S.x for the original matrix (type TI, row stride lda);
// returns max |r_i| (uniform).
template <class TI, class T>
__device__ double cta_residual(const TI *__restrict__ A, int lda, const TI *__restrict__ b, int n,
                               CtaSmem<T> &S) {
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    double mx = 0.0;
    for (int i = warp; i < n; i += CTA_WARPS) {
        const TI *row = A + (long long)i * lda;
        double s = 0.0;
        for (int j = lane; j < n; j += 32) s = fma((double)row[j], S.x[j], s);
        s = warp_sum(s);
        const double ri = (double)b[i] - s;
        if (lane == 0) S.r[i] = ri;
        mx = fmax(mx, fabs(ri));
    }
    (void)tid;
    return block_max(mx, S);
}

}  // namespace rl
