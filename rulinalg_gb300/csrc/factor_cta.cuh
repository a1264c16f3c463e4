// One-CTA dense factorisations and solves for systems with n <= CTA_NMAX (512).
//
// A CTA of CTA_THREADS threads owns one matrix that lives in global memory (its slot of
// the batch workspace, or the caller's buffer) and runs a right-looking blocked
// algorithm over it:
//   * the current column panel (rows k0..n, NB columns) is held in registers, two rows
//     per thread, and factored column by column in a rolled loop over a rotated panel
//     (row[k][0] is always the current column), with one barrier per column: warp
//     argmax on the hardware redux instructions for the LU pivot, first maximum on
//     ties as in PartialPivLu::decompose (src/matrix/decomposition/lu.rs:169-178);
//     rows keep their registers and only their positions move, so each row is written
//     once, at its final position (shared-memory panel for the update, global memory);
//   * the rows whose position changed are moved in the other columns through a
//     shared-memory stage, all loads in flight;
//   * L11^-1 is formed once per panel (warp-shuffle forward substitution); per
//     128-column slice, U12 = L11^-1 A12 is a small shared-memory GEMM, followed by the
//     trailing update A22 -= L21 U12 as 64x64 register-tiled blocks with L21 read from
//     the shared-memory panel.
// Cholesky uses the same register panel (the panel is the whole column block, so the
// diagonal block and L21 are factored together) followed by a lower-triangle SYRK.
// The factor type T is float (mixed precision) or double (plain FP64).
#pragma once

#include <climits>

#include "common.cuh"

namespace rl {

constexpr int CTA_THREADS = 256;
constexpr int CTA_WARPS = CTA_THREADS / 32;
constexpr int CTA_NMAX = 512;
constexpr int CTA_LDP = CTA_NMAX + 72;  // panel column stride: slack for 64-row tiles; 72 = 8 mod 32
                                        // so that a warp's 4 rows x 8 columns hit distinct banks
                                        // pairwise, and columns stay 16-byte aligned

template <class T>
struct CtaNB;
template <>
struct CtaNB<float> {
    static constexpr int value = 16;
};
template <>
struct CtaNB<double> {
    static constexpr int value = 16;
};

// CTAs per SM the one-CTA-per-system kernels are compiled for (register cap 65536 /
// (256 x value)); the FP32 workspace fits three in shared memory (four measured
// slower under the 64-register cap), the FP64 one two.
template <class T>
struct CtaOcc;
template <>
struct CtaOcc<float> {
    static constexpr int value = 3;
};
template <>
struct CtaOcc<double> {
    static constexpr int value = 2;
};

// Shared-memory workspace of one CTA (dynamic shared memory).
template <class T>
struct CtaSmem {
    // Every array starts on a 16-byte boundary (128-bit shared-memory accesses).
    static constexpr int NB = CtaNB<T>::value;
    alignas(16) T P[NB * CTA_LDP];     // panel, column-major: P[c * CTA_LDP + r]
    union alignas(16) {
        T Bt[NB * 128];            // factorisation: one 128-column slice of U12, row-swap staging
        double xr[2 * CTA_NMAX];   // refinement (after the factorisation): FP64 x, then FP64 r
    } u;
    alignas(16) T Linv[NB * (NB + 1)]; // L11^-1 of the current LU panel
    alignas(16) T w[CTA_NMAX];         // factor-precision right-hand side / solution
    alignas(16) int piv[CTA_NMAX];     // LAPACK-style pivots: step j swapped rows j and piv[j]
    alignas(16) int rowperm[CTA_NMAX]; // the same as a position -> original row map (solves)
    alignas(16) T cand[2][CTA_WARPS + 1][NB];  // per-warp pivot candidate rows (+ the position-j row),
                                               // double-buffered by column parity
    alignas(16) T colj[2][NB];                 // Cholesky: column j on the diagonal block's rows
    int moved_dst[2 * NB];         // panel rows whose position changed: destination ...
    int moved_src[2 * NB];         // ... and source (panel-relative)
    int nmoved;
    double redd[CTA_WARPS * 2];
    T redv[2][CTA_WARPS];
    int redi[2][CTA_WARPS];  // position of the warp's candidate
    int redq[2][CTA_WARPS];  // panel row of the warp's candidate
    int status;
    int item;
    __device__ double *x() { return u.xr; }             // FP64 solution (refinement)
    __device__ double *r() { return u.xr + CTA_NMAX; }  // FP64 residual
};

// double -> float, round to nearest even, by integer operations: the FP64 unit (which
// also runs the hardware conversion) is the scarce one on this part. Results in the
// normal float range are composed from the bit fields (the rounding carry may run into
// the exponent, up to infinity, as it should); zeros, subnormal results, infinities and
// NaNs take the hardware conversion.
__device__ __forceinline__ float f64_to_f32_rn(double x) {
    const unsigned long long b = (unsigned long long)__double_as_longlong(x);
    const unsigned hi = (unsigned)(b >> 32), lo = (unsigned)b;
    const unsigned e = (hi >> 20) & 0x7FFu;
    if (e - 897u > 253u) return __double2float_rn(x);  // float exponent outside [1, 254]
    unsigned f = (hi & 0x80000000u) | (((hi & 0x7FFFFFFFu) - 0x38000000u) << 3) | (lo >> 29);
    const unsigned rem = lo & 0x1FFFFFFFu;
    f += (rem > 0x10000000u || (rem == 0x10000000u && (f & 1u))) ? 1u : 0u;
    return __uint_as_float(f);
}

template <class TF, class TI>
__device__ __forceinline__ TF convert_to(TI v) {
    if constexpr (sizeof(TF) == 4 && sizeof(TI) == 8)
        return f64_to_f32_rn(v);
    else
        return (TF)v;
}

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

// row[0..4) -= acc[0..4) for the columns that exist (< lim); 128-bit when `vec` (row
// 16-byte aligned) and all four exist.
__device__ __forceinline__ void rmw4(float *row, const float (&acc)[4], int lim, bool vec) {
    if (vec && lim >= 4) {
        float4 v = *reinterpret_cast<float4 *>(row);
        v.x -= acc[0], v.y -= acc[1], v.z -= acc[2], v.w -= acc[3];
        *reinterpret_cast<float4 *>(row) = v;
    } else {
#pragma unroll
        for (int j = 0; j < 4; j++)
            if (j < lim) row[j] -= acc[j];
    }
}
__device__ __forceinline__ void rmw4(double *row, const double (&acc)[4], int lim, bool vec) {
    if (vec && lim >= 4) {
        double2 a = reinterpret_cast<double2 *>(row)[0], b = reinterpret_cast<double2 *>(row)[1];
        a.x -= acc[0], a.y -= acc[1], b.x -= acc[2], b.y -= acc[3];
        reinterpret_cast<double2 *>(row)[0] = a;
        reinterpret_cast<double2 *>(row)[1] = b;
    } else {
#pragma unroll
        for (int j = 0; j < 4; j++)
            if (j < lim) row[j] -= acc[j];
    }
}

// Global 4-element row segment load / store (128-bit when `vec` and all 4 exist).
template <class T>
__device__ __forceinline__ void gld4(const T *row, T (&v)[4], int lim, bool vec) {
    if (vec && lim >= 4) {
        ld4<T>(row, v);
    } else {
#pragma unroll
        for (int j = 0; j < 4; j++) v[j] = j < lim ? row[j] : T(0);
    }
}
__device__ __forceinline__ void gst4(float *row, const float (&v)[4], int lim, bool vec) {
    if (vec && lim >= 4) {
        *reinterpret_cast<float4 *>(row) = make_float4(v[0], v[1], v[2], v[3]);
    } else {
#pragma unroll
        for (int j = 0; j < 4; j++)
            if (j < lim) row[j] = v[j];
    }
}
__device__ __forceinline__ void gst4(double *row, const double (&v)[4], int lim, bool vec) {
    if (vec && lim >= 4) {
        reinterpret_cast<double2 *>(row)[0] = make_double2(v[0], v[1]);
        reinterpret_cast<double2 *>(row)[1] = make_double2(v[2], v[3]);
    } else {
#pragma unroll
        for (int j = 0; j < 4; j++)
            if (j < lim) row[j] = v[j];
    }
}

// Element idx of a rows x kb panel copy -> (r, c). When kb is a multiple of 8 every
// warp instruction covers 4 rows x 8 columns: 32-byte global segments per row and
// (with CTA_LDP = 8 mod 32) at most 2-way shared-memory bank conflicts on the
// column-major panel. Rows are padded to a multiple of 4 (callers check r < rows).
__device__ __forceinline__ void panel_rc(int idx, int kb, int &r, int &c) {
    if ((kb & 7) == 0) {
        const int lane = idx & 31, t = idx >> 5, groups = kb >> 3;
        c = ((t % groups) << 3) + (lane & 7);
        r = ((t / groups) << 2) + (lane >> 3);
    } else {
        r = idx / kb;
        c = idx - r * kb;
    }
}
__device__ __forceinline__ int panel_elems(int rows, int kb) { return ((kb & 7) == 0 ? (rows + 3) & ~3 : rows) * kb; }

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
__device__ __forceinline__ void warp_amax3(T &v, int &i, int &q) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        T v2 = __shfl_xor_sync(0xffffffffu, v, o);
        int i2 = __shfl_xor_sync(0xffffffffu, i, o);
        int q2 = __shfl_xor_sync(0xffffffffu, q, o);
        if (v2 > v || (v2 == v && i2 < i)) {
            v = v2;
            i = i2;
            q = q2;
        }
    }
}

// FP32 version on the hardware warp reductions: the largest |v| (non-negative floats
// order like their bits; NaN and the -1 "none" sentinel map to key 0), then the smallest
// position among the lanes holding it, then that lane's payload.
__device__ __forceinline__ void warp_amax3(float &v, int &i, int &q) {
    const unsigned key = (v >= 0.f) ? __float_as_uint(v) + 1u : 0u;
    const unsigned kmax = __reduce_max_sync(0xffffffffu, key);
    const unsigned ip = (key == kmax && key != 0u) ? (unsigned)i : 0xffffffffu;
    const unsigned imin = __reduce_min_sync(0xffffffffu, ip);
    if (kmax == 0u) {
        v = -1.f;
        i = INT_MAX;
        q = -1;
        return;
    }
    const int src = __ffs(__ballot_sync(0xffffffffu, ip == imin)) - 1;
    v = __shfl_sync(0xffffffffu, v, src);
    q = __shfl_sync(0xffffffffu, q, src);
    i = (int)imin;
}

template <class T>
__device__ __forceinline__ T warp_sum(T v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}
// Warp reduce-scatter of R partial sums per lane (R a power of two <= 32): returns, on
// every lane, the full sum over the warp of s[row] for row = lane >> (5 - log2 R). The
// first log2 R butterfly levels halve the values each lane holds (a lane keeps the half
// of the rows its partner gives away), the rest are a plain butterfly: R - 1 + 5 - log2 R
// additions per R rows instead of 5 R for a warp_sum per row. A fixed tree: the same
// inputs always give the same bits.
template <int R, class T>
__device__ __forceinline__ T warp_reduce_scatter(T (&s)[R], int lane, int &row) {
    constexpr int LOG = R >= 32 ? 5 : R >= 16 ? 4 : R >= 8 ? 3 : R >= 4 ? 2 : R >= 2 ? 1 : 0;
    static_assert((1 << LOG) == R, "R must be a power of two <= 32");
#pragma unroll
    for (int lv = 0; lv < LOG; lv++) {
        const int off = 16 >> lv, half = R >> (lv + 1);
        const bool up = (lane & off) != 0;
#pragma unroll
        for (int k = 0; k < half; k++) {
            const T keep = up ? s[k + half] : s[k];
            const T give = up ? s[k] : s[k + half];
            s[k] = keep + __shfl_xor_sync(0xffffffffu, give, off);
        }
    }
    T v = s[0];
#pragma unroll
    for (int off = 16 >> LOG; off > 0; off >>= 1) v += __shfl_xor_sync(0xffffffffu, v, off);
    row = lane >> (5 - LOG);
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

// Panel copies between global memory (row-major, row stride lda, from A[k0][k0]) and
// the column-major shared panel, K elements per thread per round so that K independent
// loads are in flight. LOWER_ONLY copies the elements on or below the diagonal only.
template <class T, bool LOWER_ONLY>
__device__ __forceinline__ void panel_load(const T *__restrict__ A, int lda, int k0, int mrows, int kb, CtaSmem<T> &S) {
    constexpr int K = 8;
    const int pe = panel_elems(mrows, kb);
    for (int base = threadIdx.x; base < pe; base += CTA_THREADS * K) {
        T v[K];
        int off[K];
#pragma unroll
        for (int k = 0; k < K; k++) {
            const int idx = base + k * CTA_THREADS;
            int r, c;
            panel_rc(idx, kb, r, c);
            const bool ok = idx < pe && r < mrows && (!LOWER_ONLY || r >= c);
            off[k] = ok ? c * CTA_LDP + r : -1;
            v[k] = ok ? A[(long long)(k0 + r) * lda + k0 + c] : T(0);
        }
#pragma unroll
        for (int k = 0; k < K; k++)
            if (off[k] >= 0) S.P[off[k]] = v[k];
    }
}

template <class T, bool LOWER_ONLY>
__device__ __forceinline__ void panel_store(T *__restrict__ A, int lda, int k0, int mrows, int kb, const CtaSmem<T> &S) {
    const int pe = panel_elems(mrows, kb);
    for (int idx = threadIdx.x; idx < pe; idx += CTA_THREADS) {
        int r, c;
        panel_rc(idx, kb, r, c);
        if (r < mrows && (!LOWER_ONLY || r >= c)) A[(long long)(k0 + r) * lda + k0 + c] = S.P[c * CTA_LDP + r];
    }
}


// One trailing-update tile: C -= L * U over NB, with L read from the shared panel at
// panel rows rb + h*64 + {0..3} (h < H) and U read from shared memory at bs[p * ldb +
// cb + h*64 + {0..3}]; C is global at A[(k0 + row) * lda + k0 + ccol], with at most
// `lim(row, col)` existing columns from col on. Every thread holds (4H) x (4H) outputs
// (H = 1: 64 x 64 tiles; 8 x 8 per thread spilled under the two-CTAs-per-SM register
// cap and padded the small trailing blocks, and measured slower).
template <class T>
struct TileCfg {
    static constexpr int H = 1;  // 4 x 4 per thread measured faster than 8 x 8 here
    static constexpr int TS = 64 * H;
};

template <class T, int NB, class Lim>
__device__ __forceinline__ void update_tile(T *__restrict__ A, int lda, int k0, int mrows, int row0, int col0,
                                           const T *__restrict__ P, const T *__restrict__ bs, int ldb, int bcol0,
                                           bool vec, Lim lim) {
    constexpr int H = TileCfg<T>::H, R = 4 * H;
    const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
    T cv[R][R];
#pragma unroll
    for (int i = 0; i < R; i++) {
        const int r = row0 + (i >> 2) * 64 + ty * 4 + (i & 3);
#pragma unroll
        for (int h = 0; h < H; h++) {
            const int c = col0 + h * 64 + tx * 4;
            T t4[4];
            if (r < mrows)
                gld4<T>(A + (long long)(k0 + r) * lda + k0 + c, t4, lim(r, c), vec);
            else
#pragma unroll
                for (int j = 0; j < 4; j++) t4[j] = T(0);
#pragma unroll
            for (int j = 0; j < 4; j++) cv[i][h * 4 + j] = t4[j];
        }
    }
#pragma unroll 4
    for (int p = 0; p < NB; p++) {
        T a[R], b[R];
#pragma unroll
        for (int h = 0; h < H; h++) {
            ld4<T>(&P[p * CTA_LDP + row0 + h * 64 + ty * 4], *reinterpret_cast<T(*)[4]>(&a[h * 4]));
            ld4<T>(&bs[p * ldb + bcol0 + h * 64 + tx * 4], *reinterpret_cast<T(*)[4]>(&b[h * 4]));
        }
#pragma unroll
        for (int i = 0; i < R; i++)
#pragma unroll
            for (int j = 0; j < R; j++) cv[i][j] = fma(-a[i], b[j], cv[i][j]);
    }
#pragma unroll
    for (int i = 0; i < R; i++) {
        const int r = row0 + (i >> 2) * 64 + ty * 4 + (i & 3);
        if (r >= mrows) continue;
#pragma unroll
        for (int h = 0; h < H; h++) {
            const int c = col0 + h * 64 + tx * 4;
            T t4[4];
#pragma unroll
            for (int j = 0; j < 4; j++) t4[j] = cv[i][h * 4 + j];
            gst4(A + (long long)(k0 + r) * lda + k0 + c, t4, lim(r, c), vec);
        }
    }
}

// ---------------------------------------------------------------------------- LU --
// Factors the n x n matrix A (row stride lda) in place; S.piv receives the pivots.
// A pivot with |p| < tiny returns RL_ERR_DIV_BY_ZERO (tiny = epsilon reproduces the
// reference rule of lu.rs:179-183). Uniform across the CTA.
template <class T>
__device__ int cta_lu_factor(T *__restrict__ A, int lda, int n, CtaSmem<T> &S, T tiny) {
    constexpr int NB = CtaNB<T>::value;
    constexpr int RPT = CTA_NMAX / CTA_THREADS;  // panel rows per thread
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    // 128-bit trailing-update accesses when every row start is 16-byte aligned
    const bool vec = (lda % 4) == 0 && (reinterpret_cast<uintptr_t>(A) % 16) == 0;
    for (int k0 = 0; k0 < n; k0 += NB) {
        const int kb = min(NB, n - k0), mrows = n - k0;
        // The panel lives in registers: thread t holds panel rows t and t + 256 (row q
        // of the panel is A[k0 + q][k0 .. k0 + kb)). Rows never move; pos[k] is the
        // row's current position (swaps exchange positions) and used[k] marks a row that
        // has become a pivot row.
        T row[RPT][NB];
        int pos[RPT];
        bool used[RPT];
#pragma unroll
        for (int k = 0; k < RPT; k++) {
            const int q = tid + k * CTA_THREADS;
            pos[k] = q;
            used[k] = q >= mrows;
            const T *src = A + (long long)(k0 + q) * lda + k0;
#pragma unroll
            for (int c = 0; c < NB; c++) row[k][c] = (q < mrows && c < kb) ? src[c] : T(0);
        }
        if (tid == 0) S.nmoved = 0;
        // One barrier per column, the column loop rolled: every row is kept rotated so
        // that row[k][0] holds the current column j. Step j combines the warps' argmax
        // candidates for column j (published at the end of the previous step, rotated
        // the same way), turns the active rows' row[k][0] into multipliers, updates
        // their columns j + 1 .. NB - 1 (indices 1 .. NB - 1 - j) with the pivot row,
        // and rotates every row left by one, the finished column-j entry going to the
        // end. After NB steps the rows are back in column order.
        auto publish = [&](int j, int par) {
            T bv = T(-1);
            int bi = INT_MAX, bq = -1, bk = -1;
#pragma unroll
            for (int k = 0; k < RPT; k++) {
                const T av = absT(row[k][0]);
                if (!used[k] && (av > bv || (av == bv && pos[k] < bi))) {
                    bv = av;
                    bi = pos[k];
                    bq = tid + k * CTA_THREADS;
                    bk = k;
                }
                if (pos[k] == j && tid + k * CTA_THREADS < mrows) {  // the row at position j (NaN fallback)
#pragma unroll
                    for (int c = 0; c < NB; c++) S.cand[par][CTA_WARPS][c] = row[k][c];
                }
            }
            T wv = bv;
            int wi = bi, wq = bq;
            warp_amax3(wv, wi, wq);
            if (wq >= 0 && wq == bq && bk >= 0) {  // this lane holds the warp's winner
#pragma unroll
                for (int k = 0; k < RPT; k++)
                    if (k == bk)
#pragma unroll
                        for (int c = 0; c < NB; c++) S.cand[par][warp][c] = row[k][c];
            }
            if (lane == 0) {
                S.redv[par][warp] = wv;
                S.redi[par][warp] = wi;
                S.redq[par][warp] = wq;
            }
        };
        auto rotate = [&]() {
#pragma unroll
            for (int k = 0; k < RPT; k++) {
                const T first = row[k][0];
#pragma unroll
                for (int c = 0; c < NB - 1; c++) row[k][c] = row[k][c + 1];
                row[k][NB - 1] = first;
            }
        };
        publish(0, 0);
        for (int j = 0; j < kb; j++) {
            const int par = j & 1;
            __syncthreads();
            T bv = S.redv[par][0];
            int bi = S.redi[par][0], bq = S.redq[par][0], bw = 0;
#pragma unroll
            for (int w = 1; w < CTA_WARPS; w++) {
                const T v2 = S.redv[par][w];
                const int i2 = S.redi[par][w];
                if (v2 > bv || (v2 == bv && i2 < bi)) {
                    bv = v2;
                    bi = i2;
                    bq = S.redq[par][w];
                    bw = w;
                }
            }
            if (bi == INT_MAX) {  // no comparable candidate (NaNs): keep the diagonal, as the reference does
                bi = j;
                bq = -1;
                bw = CTA_WARPS;
                bv = absT(S.cand[par][CTA_WARPS][0]);
            }
            if (bv < tiny) {
                __syncthreads();
                return RL_ERR_DIV_BY_ZERO;
            }
            if (tid == 0) S.piv[k0 + j] = k0 + bi;
            T prow[NB];
#pragma unroll
            for (int c = 0; c < NB; c++) prow[c] = S.cand[par][bw][c];
            const T p = prow[0];
            const T inv_p = T(1) / p;  // one division per column; multipliers l = a_rj * (1/p)
            const int act = NB - 1 - j;  // indices 1 .. act are the columns right of j
#pragma unroll
            for (int k = 0; k < RPT; k++) {
                const int q = tid + k * CTA_THREADS;
                const bool is_piv = (bq >= 0) ? (q == bq) : (pos[k] == j && q < mrows);
                if (is_piv) {
                    used[k] = true;
                    pos[k] = j;
                } else if (pos[k] == j) {
                    pos[k] = bi;  // the row that held position j takes the pivot's old position
                }
                if (!used[k]) {
                    // FP64 keeps gaussian_elimination's division (lu.rs:609); FP32 multiplies by 1/p
                    const T l = sizeof(T) == 8 ? row[k][0] / p : row[k][0] * inv_p;
                    row[k][0] = l;
#pragma unroll
                    for (int c = 1; c < NB; c++)
                        if (c <= act) row[k][c] = fma(-l, prow[c], row[k][c]);
                }
            }
            rotate();
            if (j + 1 < kb) publish(j + 1, par ^ 1);
        }
        for (int j = kb; j < NB; j++) rotate();  // a narrow last panel: back to column order
        __syncthreads();
        // Rows to their final positions: shared panel (column-major, position order, for
        // the trailing update), global A, and the list of rows whose position changed.
#pragma unroll
        for (int k = 0; k < RPT; k++) {
            const int q = tid + k * CTA_THREADS;
            if (q >= mrows) continue;
            T *dst = A + (long long)(k0 + pos[k]) * lda + k0;
#pragma unroll
            for (int c = 0; c < NB; c++) {
                if (c < kb) {
                    S.P[c * CTA_LDP + pos[k]] = row[k][c];
                    dst[c] = row[k][c];
                }
            }
            if (pos[k] != q) {
                const int m = atomicAdd(&S.nmoved, 1);
                S.moved_dst[m] = pos[k];
                S.moved_src[m] = q;
            }
        }
        __syncthreads();
        // The panel's row permutation on every other column, 64 columns at a time: the
        // (at most 2 NB) moved rows' sources are staged in shared memory (all loads in
        // flight), then written to their destinations.
        {
            const int nmv = S.nmoved;
            T *stage = S.u.Bt;  // NB * 64 >= 2 NB rows x 32 columns
            constexpr int CW = 32;
            for (int c0 = 0; c0 < n - kb && nmv > 0; c0 += CW) {
                constexpr int K = (2 * NB * CW) / CTA_THREADS;
                T v[K];
#pragma unroll
                for (int k = 0; k < K; k++) {
                    const int e = tid + k * CTA_THREADS, m = e / CW, cc = e % CW, c = c0 + cc;
                    const int gc = c < k0 ? c : c + kb;
                    v[k] = (m < nmv && c < n - kb) ? A[(long long)(k0 + S.moved_src[m]) * lda + gc] : T(0);
                }
#pragma unroll
                for (int k = 0; k < K; k++) stage[tid + k * CTA_THREADS] = v[k];
                __syncthreads();
#pragma unroll
                for (int k = 0; k < K; k++) {
                    const int e = tid + k * CTA_THREADS, m = e / CW, cc = e % CW, c = c0 + cc;
                    const int gc = c < k0 ? c : c + kb;
                    if (m < nmv && c < n - kb) A[(long long)(k0 + S.moved_dst[m]) * lda + gc] = stage[e];
                }
                __syncthreads();
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
        // Per 128-column slice: U12 = L11^-1 A12 as a small shared-memory GEMM (written
        // back to A), then A22 -= L21 * U12 tile by tile (update_tile).
        const int m2 = mrows - kb;
        constexpr int RPS = NB / 2;  // U12 rows per thread in the slice solve
        for (int tj = 0; tj < n2; tj += 128) {
            auto lim = [&](int, int c) { return kb + n2 - c; };
            {
                constexpr int K = NB * 128 / CTA_THREADS;
                T v[K];
#pragma unroll
                for (int k = 0; k < K; k++) {
                    const int idx = tid + k * CTA_THREADS, pp = idx >> 7, cc = idx & 127;
                    v[k] = (tj + cc < n2) ? A[(long long)(k0 + pp) * lda + k0 + kb + tj + cc] : T(0);
                }
#pragma unroll
                for (int k = 0; k < K; k++) S.u.Bt[tid + k * CTA_THREADS] = v[k];
            }
            __syncthreads();
            {
                const int cc = tid & 127, rg = (tid >> 7) * RPS;
                T u[RPS];
#pragma unroll
                for (int i = 0; i < RPS; i++) u[i] = T(0);
#pragma unroll
                for (int k = 0; k < NB; k++) {
                    const T bk = S.u.Bt[k * 128 + cc];
#pragma unroll
                    for (int i = 0; i < RPS; i++) u[i] = fma(S.Linv[(rg + i) * (NB + 1) + k], bk, u[i]);
                }
                __syncthreads();
#pragma unroll
                for (int i = 0; i < RPS; i++) {
                    S.u.Bt[(rg + i) * 128 + cc] = u[i];
                    if (tj + cc < n2) A[(long long)(k0 + rg + i) * lda + k0 + kb + tj + cc] = u[i];
                }
            }
            __syncthreads();
            constexpr int TS = TileCfg<T>::TS;
            for (int ti = 0; ti < m2; ti += TS)
                for (int tc = 0; tc < 128 && tj + tc < n2; tc += TS)
                    update_tile<T, NB>(A, lda, k0, mrows, kb + ti, kb + tj + tc, S.P, S.u.Bt, 128, tc, vec, lim);
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
    constexpr int RPT = CTA_NMAX / CTA_THREADS;  // panel rows per thread
    const int tid = threadIdx.x;
    const bool vec = (lda % 4) == 0 && (reinterpret_cast<uintptr_t>(A) % 16) == 0;
    for (int k0 = 0; k0 < n; k0 += NB) {
        const int kb = min(NB, n - k0), mrows = n - k0;
        // The panel lives in registers (thread t holds rows t and t + 256, lower part
        // only). One barrier per column: the diagonal block's column j is published to
        // shared memory by its rows' owners at the end of step j - 1.
        T row[RPT][NB];
#pragma unroll
        for (int k = 0; k < RPT; k++) {
            const int q = tid + k * CTA_THREADS;
            const T *src = A + (long long)(k0 + q) * lda + k0;
#pragma unroll
            for (int c = 0; c < NB; c++) row[k][c] = (q < mrows && c < kb && c <= q) ? src[c] : T(0);
        }
        if (tid < kb) S.colj[0][tid] = row[0][0];
        // The column loop is rolled, every row kept rotated so that row[k][0] holds the
        // current column j (see cta_lu_factor); after NB steps the rows are back in
        // column order.
        auto rotate = [&]() {
#pragma unroll
            for (int k = 0; k < RPT; k++) {
                const T first = row[k][0];
#pragma unroll
                for (int c = 0; c < NB - 1; c++) row[k][c] = row[k][c + 1];
                row[k][NB - 1] = first;
            }
        };
        for (int j = 0; j < kb; j++) {
            const int par = j & 1;
            __syncthreads();
            const T d = S.colj[par][j];
            if (absT(d) < tiny || d < T(0)) {
                __syncthreads();
                return RL_ERR_DECOMP_FAILURE;
            }
            const T s = sqrt(d);
            const T inv = T(1) / s;  // update factors; the stored entries keep the division
            const int act = kb - 1 - j;  // indices 1 .. act are the panel columns right of j
            T lc[NB];
            lc[0] = T(0);
#pragma unroll
            for (int c = 1; c < NB; c++) lc[c] = c <= act ? S.colj[par][j + c] * inv : T(0);
#pragma unroll
            for (int k = 0; k < RPT; k++) {
                const int q = tid + k * CTA_THREADS;
                if (q >= j && q < mrows) {
                    const T cr = row[k][0];
                    const T l = cr / s, li = cr * inv;
                    row[k][0] = l;
#pragma unroll
                    for (int c = 1; c < NB; c++)
                        if (c <= act && j + c <= q) row[k][c] = fma(-li, lc[c], row[k][c]);
                }
            }
            rotate();
            if (j + 1 < kb && tid < kb) S.colj[par ^ 1][tid] = row[0][0];  // rows tid < kb: row[0] of threads 0..kb-1
        }
        for (int j = kb; j < NB; j++) rotate();  // a narrow last panel: back to column order
        // Write the factored panel: shared (column-major, for the SYRK) and global (the
        // lower part only; the strict upper triangle is never written).
#pragma unroll
        for (int k = 0; k < RPT; k++) {
            const int q = tid + k * CTA_THREADS;
            if (q >= mrows) continue;
            T *dst = A + (long long)(k0 + q) * lda + k0;
#pragma unroll
            for (int c = 0; c < NB; c++) {
                if (c < kb && c <= q) {
                    S.P[c * CTA_LDP + q] = row[k][c];
                    dst[c] = row[k][c];
                }
            }
        }
        __syncthreads();
        const int m2 = mrows - kb;
        if (m2 <= 0) {
            __syncthreads();
            continue;
        }
        // A22 -= L21 L21^T on the lower triangle; both operands come from the panel.
        auto lim = [&](int r, int c) { return min(mrows, r + 1) - c; };
        constexpr int TS = TileCfg<T>::TS;
        for (int ti = 0; ti < m2; ti += TS)
            for (int tj = 0; tj <= ti; tj += TS)
                update_tile<T, NB>(A, lda, k0, mrows, kb + ti, kb + tj, S.P, S.P, CTA_LDP, kb + tj, vec, lim);
        __syncthreads();
    }
    return RL_OK;
}

// ------------------------------------------------------------------------- solves --
// In-place solves on the shared vector S.w, 32 x 32 blocks at a time. Triangles are read
// from global memory (the factor lives in L2) with coalesced row segments only: warp 0
// stages each diagonal block in a padded shared tile and solves it with the solution
// moving by shuffles; the off-block updates take 32 rows per warp (16 for FP64), lane c
// reading column c, and a butterfly reduce-scatter leaves row r's sum in lane r.

// w[i] -= sum_{c < bs} M[i][c] * w[b0 + c] for the rows i in [lo, hi) of M (M points at
// column b0 of row 0; row stride lda).
template <class T>
__device__ __noinline__ void cta_block_update(const T *__restrict__ M, int lda, int lo, int hi, int b0, int bs,
                                              CtaSmem<T> &S) {
    constexpr int RB = sizeof(T) == 4 ? 32 : 16;  // rows per warp pass
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const T y = lane < bs ? S.w[b0 + lane] : T(0);
    for (int r0 = lo + warp * RB; r0 < hi; r0 += CTA_WARPS * RB) {
        T p[RB];
#pragma unroll
        for (int r = 0; r < RB; r++) {
            const int i = r0 + r;
            p[r] = (i < hi && lane < bs) ? M[(long long)i * lda + lane] : T(0);
        }
#pragma unroll
        for (int r = 0; r < RB; r++) p[r] *= y;
#pragma unroll
        for (int s = 16; s >= RB; s >>= 1)
#pragma unroll
            for (int r = 0; r < RB; r++) p[r] += __shfl_xor_sync(0xffffffffu, p[r], s);
#pragma unroll
        for (int s = RB / 2; s >= 1; s >>= 1) {
            const bool up = lane & s;
#pragma unroll
            for (int k = 0; k < s; k++) {
                const T send = up ? p[k] : p[k + s];
                const T keep = up ? p[k + s] : p[k];
                p[k] = keep + __shfl_xor_sync(0xffffffffu, send, s);
            }
        }
        const int i = r0 + (lane & (RB - 1));
        if (lane < RB && i < hi) S.w[i] -= p[0];
    }
}

// 1 / d for the factor type's solves: FP32 multiplies by the reciprocal, FP64 divides.
template <class T>
__device__ __forceinline__ T solve_div(T v, T d, T inv) {
    return sizeof(T) == 8 ? v / d : v * inv;
}

// Warp 0: solves the bs x bs diagonal block at (b0, b0) in place on S.w[b0 ..]. The
// block's rows are staged in S.P (row r at r * 33); FORWARD runs top-down, TRANS takes
// the block's transpose (L^T), UNIT skips the diagonal. Returns 1 when a diagonal entry
// is below tiny (uniform over the warp).
template <class T, bool FORWARD, bool UNIT, bool TRANS>
__device__ __noinline__ int diag_block_solve(const T *__restrict__ A, int lda, int b0, int bs, CtaSmem<T> &S, T tiny) {
    const int lane = threadIdx.x & 31;
    T *D = S.P;
    {
        T v[32];
#pragma unroll
        for (int r = 0; r < 32; r++) v[r] = (r < bs && lane < bs) ? A[(long long)(b0 + r) * lda + b0 + lane] : T(0);
#pragma unroll
        for (int r = 0; r < 32; r++) D[r * 33 + lane] = v[r];
    }
    __syncwarp();
    // lane's equation row: element (lane, c) of the block (or of its transpose)
    auto elem = [&](int c) { return TRANS ? D[c * 33 + lane] : D[lane * 33 + c]; };
    const T d = UNIT ? T(1) : elem(lane);
    const int bad = UNIT ? 0 : __any_sync(0xffffffffu, lane < bs && absT(d) < tiny);
    const T inv = T(1) / d;
    T wv = lane < bs ? S.w[b0 + lane] : T(0);
    if (FORWARD) {
#pragma unroll 4
        for (int jj = 0; jj < bs; jj++) {
            if (!UNIT && lane == jj) wv = solve_div(wv, d, inv);
            const T wj = __shfl_sync(0xffffffffu, wv, jj);
            if (lane > jj) wv = fma(-elem(jj), wj, wv);
        }
    } else {
#pragma unroll 4
        for (int jj = bs - 1; jj >= 0; jj--) {
            if (!UNIT && lane == jj) wv = solve_div(wv, d, inv);
            const T wj = __shfl_sync(0xffffffffu, wv, jj);
            if (lane < jj) wv = fma(-elem(jj), wj, wv);
        }
    }
    if (lane < bs) S.w[b0 + lane] = wv;
    __syncwarp();
    return bad;
}

// Unit lower triangular solve L y = w (L strictly below the diagonal of A).
template <class T>
__device__ void cta_unit_lower_solve(const T *__restrict__ A, int lda, int n, CtaSmem<T> &S) {
    const int warp = threadIdx.x >> 5;
    for (int b0 = 0; b0 < n; b0 += 32) {
        const int bs = min(32, n - b0);
        if (warp == 0) diag_block_solve<T, true, true, false>(A, lda, b0, bs, S, T(0));
        __syncthreads();
        cta_block_update(A + b0, lda, b0 + bs, n, b0, bs, S);
        __syncthreads();
    }
}

// Upper triangular solve U x = w (U on and above the diagonal of A). |u_ii| < tiny
// returns RL_ERR_DIV_BY_ZERO (src/matrix/mod.rs:333-336).
template <class T>
__device__ int cta_upper_solve(const T *__restrict__ A, int lda, int n, CtaSmem<T> &S, T tiny) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    for (int b1 = n; b1 > 0; b1 -= 32) {
        const int b0 = max(0, b1 - 32), bs = b1 - b0;
        if (warp == 0) {
            const int bad = diag_block_solve<T, false, false, false>(A, lda, b0, bs, S, tiny);
            if (lane == 0) S.status = bad;
        }
        __syncthreads();
        if (S.status) {
            __syncthreads();
            return RL_ERR_DIV_BY_ZERO;
        }
        cta_block_update(A + b0, lda, 0, b0, b0, bs, S);
        __syncthreads();
    }
    return RL_OK;
}

// Lower (non-unit) solve L y = w; |l_ii| < tiny -> RL_ERR_DIV_BY_ZERO (mod.rs:375-378).
template <class T>
__device__ int cta_lower_solve(const T *__restrict__ A, int lda, int n, CtaSmem<T> &S, T tiny) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    for (int b0 = 0; b0 < n; b0 += 32) {
        const int bs = min(32, n - b0);
        if (warp == 0) {
            const int bad = diag_block_solve<T, true, false, false>(A, lda, b0, bs, S, tiny);
            if (lane == 0) S.status = bad;
        }
        __syncthreads();
        if (S.status) {
            __syncthreads();
            return RL_ERR_DIV_BY_ZERO;
        }
        cta_block_update(A + b0, lda, b0 + bs, n, b0, bs, S);
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
            const int bad = diag_block_solve<T, false, false, true>(A, lda, b0, bs, S, tiny);
            if (lane == 0) S.status = bad;
        }
        __syncthreads();
        if (S.status) {
            __syncthreads();
            return RL_ERR_DIV_BY_ZERO;
        }
        // w[i] -= sum_jj L[b0 + jj][i] w[b0 + jj] for i < b0: a thread per i, coalesced rows
        for (int i = tid; i < b0; i += CTA_THREADS) {
            T v[32];
#pragma unroll
            for (int jj = 0; jj < 32; jj++) v[jj] = jj < bs ? A[(long long)(b0 + jj) * lda + i] : T(0);
            T s = T(0);
#pragma unroll
            for (int jj = 0; jj < 32; jj++)
                if (jj < bs) s = fma(v[jj], S.w[b0 + jj], s);
            S.w[i] -= s;
        }
        __syncthreads();
    }
    return RL_OK;
}

// Row permutation of an LU factorisation as a position -> original row map (from the
// LAPACK-style pivots in S.piv), computed once per factorisation into S.rowperm.
template <class T>
__device__ void cta_build_rowperm(int n, CtaSmem<T> &S) {
    for (int i = threadIdx.x; i < n; i += CTA_THREADS) S.rowperm[i] = i;
    __syncthreads();
    if (threadIdx.x == 0) {
        for (int j = 0; j < n; j++) {
            const int p = S.piv[j];
            if (p != j) {
                const int t = S.rowperm[j];
                S.rowperm[j] = S.rowperm[p];
                S.rowperm[p] = t;
            }
        }
    }
    __syncthreads();
}

// Applies the row permutation to S.w as a gather through registers.
template <class T>
__device__ void cta_apply_pivots(int n, CtaSmem<T> &S) {
    T v[CTA_NMAX / CTA_THREADS];
#pragma unroll
    for (int k = 0; k < CTA_NMAX / CTA_THREADS; k++) {
        const int i = threadIdx.x + k * CTA_THREADS;
        v[k] = i < n ? S.w[S.rowperm[i]] : T(0);
    }
    __syncthreads();
#pragma unroll
    for (int k = 0; k < CTA_NMAX / CTA_THREADS; k++) {
        const int i = threadIdx.x + k * CTA_THREADS;
        if (i < n) S.w[i] = v[k];
    }
    __syncthreads();
}

// Full solve with a factor: kind 0 = LU (row permutation in S.rowperm), 1 = Cholesky.
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

// Row-block passes over an n x n row-major matrix: a warp covers R consecutive rows x
// 32 C columns per pass (lane owns columns lane + 32 c), every lane issuing its R C
// loads before using any. (C, R) is picked from n (n <= 32 C) so that a lane keeps 8 to
// 32 loads in flight.
template <int C, int R, class TI, class TF>
__device__ double copy_rows(const TI *__restrict__ A, int lda, int n, TF *__restrict__ W, int ldw) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    double mx = 0.0;
    for (int i0 = warp * R; i0 < n; i0 += CTA_WARPS * R) {
        TI v[R][C];
#pragma unroll
        for (int r = 0; r < R; r++)
#pragma unroll
            for (int c = 0; c < C; c++) {
                const int i = i0 + r, j = lane + 32 * c;
                v[r][c] = (32 * c < n && i < n && j < n) ? A[(long long)i * lda + j] : TI(0);
            }
#pragma unroll
        for (int r = 0; r < R; r++) {
            const int i = i0 + r;
            TF s = TF(0);
#pragma unroll
            for (int c = 0; c < C; c++) {
                if (32 * c >= n) continue;  // warp-uniform: chunks past n do nothing
                const int j = lane + 32 * c;
                const TF f = convert_to<TF>(v[r][c]);
                if (i < n && j < n) W[(long long)i * ldw + j] = f;
                s += absT(f);
            }
            s = warp_sum(s);
            mx = fmax(mx, (double)s);
        }
    }
    return mx;
}

// Copies A (TI, row stride lda) into the factor workspace W (TF, row stride ldw) and
// returns ||A||_inf of the converted copy (uniform).
template <class TI, class TF>
__device__ double cta_copy_convert(const TI *__restrict__ A, int lda, int n, TF *__restrict__ W, int ldw,
                                   CtaSmem<TF> &S) {
    constexpr int H = CtaOcc<TF>::value >= 4 ? 2 : 1;  // fewer loads in flight under a 64-register cap
    double mx;
    if (n > 256)
        mx = copy_rows<16, 2 / H>(A, lda, n, W, ldw);
    else if (n > 128)
        mx = copy_rows<8, 4 / H>(A, lda, n, W, ldw);
    else if (n > 64)
        mx = copy_rows<4, 4 / H>(A, lda, n, W, ldw);
    else
        mx = copy_rows<2, 4 / H>(A, lda, n, W, ldw);
    return block_max(mx, S);
}

template <int C, int R, class TI, class T>
__device__ double residual_rows(const TI *__restrict__ A, int lda, const TI *__restrict__ b, int n, CtaSmem<T> &S) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    double mx = 0.0;
    for (int i0 = warp * R; i0 < n; i0 += CTA_WARPS * R) {
        // column chunks at or past n are skipped by a warp-uniform test, not zero-filled:
        // C is fixed per size class (16 chunks for any n in (256, 512])
        TI v[R][C];
#pragma unroll
        for (int r = 0; r < R; r++)
#pragma unroll
            for (int c = 0; c < C; c++) {
                const int i = i0 + r, j = lane + 32 * c;
                v[r][c] = (32 * c < n && i < n && j < n) ? A[(long long)i * lda + j] : TI(0);
            }
        constexpr int LOG = R >= 4 ? 2 : R >= 2 ? 1 : 0;
        const int mine = i0 + (lane >> (5 - LOG));  // the row whose sum this lane ends with
        const double bl = mine < n ? (double)b[mine] : 0.0;
        double s[R];
#pragma unroll
        for (int r = 0; r < R; r++) s[r] = 0.0;
        // chunk by chunk, each row's terms in the same order; the chunks at or past n are
        // left by a warp-uniform branch (a predicated-off DFMA still takes the FP64 pipe)
#pragma unroll
        for (int c = 0; c < C; c++) {
            if (32 * c >= n) break;
            const int j = lane + 32 * c;
            const double xj = j < n ? S.x()[j] : 0.0;
#pragma unroll
            for (int r = 0; r < R; r++) s[r] = fma((double)v[r][c], xj, s[r]);
        }
        // the rows' warp sums with R - 1 + 5 - log2 R FP64 additions (a warp-wide FP64
        // instruction is tens of cycles of the SM's FP64 pipe on this part)
        int row;
        const double tot = warp_reduce_scatter<R>(s, lane, row);
        const double ri = bl - tot;
        if (i0 + row < n) {
            if ((lane & ((32 >> LOG) - 1)) == 0) S.r()[i0 + row] = ri;
            mx = fmax(mx, fabs(ri));
        }
    }
    return mx;
}

// FP64 residual S.r = b - A S.x for the original matrix (type TI, row stride lda);
// returns max |r_i| (uniform). Each lane sums its columns j = lane, lane + 32, ... in
// order, then the warp tree adds the lanes.
template <class TI, class T>
__device__ double cta_residual(const TI *__restrict__ A, int lda, const TI *__restrict__ b, int n, CtaSmem<T> &S) {
    constexpr int H = CtaOcc<T>::value >= 4 ? 2 : 1;
    double mx;
    if (n > 256)
        mx = residual_rows<16, 2 / H>(A, lda, b, n, S);
    else if (n > 128)
        mx = residual_rows<8, 4 / H>(A, lda, b, n, S);
    else if (n > 64)
        mx = residual_rows<4, 4 / H>(A, lda, b, n, S);
    else
        mx = residual_rows<2, 4 / H>(A, lda, b, n, S);
    return block_max(mx, S);
}

}  // namespace rl
