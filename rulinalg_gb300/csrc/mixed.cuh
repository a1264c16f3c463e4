// Kernels of the large-n mixed-precision solver and of the few-right-hand-side
// triangular solves: FP64 residual GEMV, column inf-norms, FP32 <-> FP64 scaling,
// warp-level diagonal-block triangular solves, GEMV updates, and the FP64 vector
// kernels of GMRES (deterministic two-stage reductions, single-thread Givens).
#pragma once

#include "factor_cta.cuh"

namespace rl {

// non-negative floating-point values order like their bit patterns
__device__ __forceinline__ void atomic_max_nonneg(unsigned long long *addr, double v) {
    atomicMax(addr, (unsigned long long)__double_as_longlong(v));
}

// A32 = (float)A (row stride ld32) and ||A||_inf (max row sum of |a|, FP32 accumulation)
// into *anorm_bits (bits of a non-negative double). Warp per row.
static __global__ void to_f32_rownorm_kernel(const double *__restrict__ A, long long lda, int n, float *__restrict__ A32,
                                      long long ld32, unsigned long long *anorm_bits) {
    const int lane = threadIdx.x & 31;
    const int wpb = blockDim.x >> 5;
    for (int i = blockIdx.x * wpb + (threadIdx.x >> 5); i < n; i += gridDim.x * wpb) {
        const double *row = A + (long long)i * lda;
        float *out = A32 + (long long)i * ld32;
        float s = 0.f;
        for (int j = lane; j < n; j += 32) {
            const float v = (float)row[j];
            out[j] = v;
            s += fabsf(v);
        }
        s = warp_sum(s);
        if (lane == 0) atomic_max_nonneg(anorm_bits, (double)s);
    }
}

// ||A||_inf in FP64 (max row sum of |a|) into *bits; warp per row.
static __global__ void rownorm_kernel(const double *__restrict__ A, long long lda, int n, unsigned long long *bits) {
    const int lane = threadIdx.x & 31;
    const int wpb = blockDim.x >> 5;
    for (int i = blockIdx.x * wpb + (threadIdx.x >> 5); i < n; i += gridDim.x * wpb) {
        const double *row = A + (long long)i * lda;
        double s = 0.0;
        for (int j = lane; j < n; j += 32) s += fabs(row[j]);
        s = warp_sum(s);
        if (lane == 0) atomic_max_nonneg(bits, s);
    }
}

// R = B - A X for nrhs <= 4 right-hand sides, FP64; warp per row (lanes stride the row).
// B == nullptr gives R = A X.
template <int NR>
static __global__ void residual_gemv_kernel(const double *__restrict__ A, long long lda, int n, const double *__restrict__ X,
                                     long long ldx, const double *__restrict__ B, long long ldb, double *__restrict__ R,
                                     long long ldr, int nrhs) {
    const int lane = threadIdx.x & 31;
    const int wpb = blockDim.x >> 5;
    for (int i = blockIdx.x * wpb + (threadIdx.x >> 5); i < n; i += gridDim.x * wpb) {
        const double *row = A + (long long)i * lda;
        double s[NR];
#pragma unroll
        for (int c = 0; c < NR; c++) s[c] = 0.0;
        // 8 columns' loads issued before their DFMAs (the same DFMAs, in the same order)
        for (int j0 = lane; j0 < n; j0 += 32 * 8) {
            double a[8], xv[8][NR];
#pragma unroll
            for (int u = 0; u < 8; u++) {
                const int j = j0 + 32 * u;
                a[u] = j < n ? row[j] : 0.0;
#pragma unroll
                for (int c = 0; c < NR; c++) xv[u][c] = (j < n && c < nrhs) ? X[(long long)j * ldx + c] : 0.0;
            }
#pragma unroll
            for (int u = 0; u < 8; u++)
                if (j0 + 32 * u < n)
#pragma unroll
                    for (int c = 0; c < NR; c++)
                        if (c < nrhs) s[c] = fma(a[u], xv[u][c], s[c]);
        }
#pragma unroll
        for (int c = 0; c < NR; c++) s[c] = warp_sum(s[c]);
        if (lane == 0)
#pragma unroll
            for (int c = 0; c < NR; c++)
                if (c < nrhs) R[(long long)i * ldr + c] = B ? B[(long long)i * ldb + c] - s[c] : s[c];
    }
}

// Per-column max |V[:, c]| into out[c] (bits), nrhs columns.
static __global__ void colnorm_kernel(const double *__restrict__ V, long long ldv, int n, int nrhs, unsigned long long *out) {
    const long long total = (long long)n * nrhs;
    for (long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x; e < total; e += (long long)gridDim.x * blockDim.x) {
        const int i = (int)(e / nrhs), c = (int)(e - (long long)i * nrhs);
        atomic_max_nonneg(out + c, fabs(V[(long long)i * ldv + c]));
    }
}

// W = (float)(R / scale[c]) for the active columns (scale given as bits of a double).
static __global__ void scale_to_f32_kernel(const double *__restrict__ R, long long ldr, int n, int nrhs,
                                    const unsigned long long *scale_bits, float *__restrict__ W, long long ldw) {
    const long long total = (long long)n * nrhs;
    for (long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x; e < total; e += (long long)gridDim.x * blockDim.x) {
        const int i = (int)(e / nrhs), c = (int)(e - (long long)i * nrhs);
        const double sc = __longlong_as_double((long long)scale_bits[c]);
        W[(long long)i * ldw + c] = (float)(sc > 0 ? R[(long long)i * ldr + c] / sc : 0.0);
    }
}

// X += scale[c] * W for the columns with active[c] != 0.
static __global__ void update_x_kernel(double *__restrict__ X, long long ldx, const float *__restrict__ W, long long ldw, int n,
                                int nrhs, const unsigned long long *scale_bits, const int *active) {
    const long long total = (long long)n * nrhs;
    for (long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x; e < total; e += (long long)gridDim.x * blockDim.x) {
        const int i = (int)(e / nrhs), c = (int)(e - (long long)i * nrhs);
        if (!active[c]) continue;
        const double sc = __longlong_as_double((long long)scale_bits[c]);
        X[(long long)i * ldx + c] = fma(sc, (double)W[(long long)i * ldw + c], X[(long long)i * ldx + c]);
    }
}

// X (double) = (double) W (float)
static __global__ void f32_to_f64_kernel(const float *__restrict__ W, long long ldw, int n, int nrhs, double *__restrict__ X,
                                  long long ldx) {
    const long long total = (long long)n * nrhs;
    for (long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x; e < total; e += (long long)gridDim.x * blockDim.x) {
        const int i = (int)(e / nrhs), c = (int)(e - (long long)i * nrhs);
        X[(long long)i * ldx + c] = (double)W[(long long)i * ldw + c];
    }
}

// ------------------------------------------------ few-right-hand-side triangular --
// Diagonal block solve for nrhs <= 8 right-hand sides: one warp per column, the
// bs x bs block (bs <= 64) staged in shared memory. mode 0: unit lower, 1: lower,
// 2: upper, 3: D^T with D lower. |d_ii| < tiny records RL_ERR_DIV_BY_ZERO. The block may
// be stored in a narrower type TA than the arithmetic type T (an FP32 factor applied in
// FP64 by GMRES-IR's preconditioner).
template <class T, class TA = T>
static __global__ void __launch_bounds__(256) trsv_diag_kernel(const TA *__restrict__ D, long long ldd, int bs,
                                                         T *__restrict__ Y, long long ldy, int nrhs, int mode,
                                                         int *status, T tiny) {
    __shared__ T Ds[64][65];
    __shared__ T ys[8][64];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    for (int idx = threadIdx.x; idx < bs * bs; idx += blockDim.x) {
        const int i = idx / bs, j = idx - i * bs;
        Ds[i][j] = T(D[(long long)i * ldd + j]);
    }
    const int c = w;
    if (c < nrhs)
        for (int i = lane; i < bs; i += 32) ys[c][i] = Y[(long long)i * ldy + c];
    __syncthreads();
    if (c >= nrhs) return;
    int bad = 0;
    if (mode <= 1) {
        for (int k = 0; k < bs; k++) {
            if (mode == 1 && lane == 0) {
                if (absT(Ds[k][k]) < tiny) bad = 1;
                ys[c][k] = ys[c][k] / Ds[k][k];
            }
            __syncwarp();
            const T yk = ys[c][k];
            for (int i = k + 1 + lane; i < bs; i += 32) ys[c][i] = fma(-Ds[i][k], yk, ys[c][i]);
            __syncwarp();
        }
    } else {
        for (int k = bs - 1; k >= 0; k--) {
            if (lane == 0) {
                if (absT(Ds[k][k]) < tiny) bad = 1;
                ys[c][k] = ys[c][k] / Ds[k][k];
            }
            __syncwarp();
            const T yk = ys[c][k];
            for (int i = lane; i < k; i += 32) ys[c][i] = fma(-(mode == 2 ? Ds[i][k] : Ds[k][i]), yk, ys[c][i]);
            __syncwarp();
        }
    }
    if (lane == 0 && bad) atomicCAS(status, 0, RL_ERR_DIV_BY_ZERO);
    for (int i = lane; i < bs; i += 32) Y[(long long)i * ldy + c] = ys[c][i];
}

// Yr[i][c] -= sum_j M[i][j] Yb[j][c] for i < rows, j < bs (<= 64), c < nrhs (<= 8);
// warp per row. transposed = true uses M[j][i] (M given with row stride ldm from the
// block's top-left, i.e. the block is bs x rows) and a thread per output row. M may be
// stored in a narrower type TA than the arithmetic type T.
template <class T, class TA = T>
static __global__ void gemv_update_kernel(const TA *__restrict__ M, long long ldm, int rows, int bs, const T *__restrict__ Yb,
                                   long long ldy, T *__restrict__ Yr, int nrhs, bool transposed) {
    if (!transposed) {
        const int lane = threadIdx.x & 31, wpb = blockDim.x >> 5;
        for (int i = blockIdx.x * wpb + (threadIdx.x >> 5); i < rows; i += gridDim.x * wpb) {
            const TA *row = M + (long long)i * ldm;
            const T m0 = lane < bs ? T(row[lane]) : T(0);
            const T m1 = lane + 32 < bs ? T(row[lane + 32]) : T(0);
            for (int c = 0; c < nrhs; c++) {
                T s = T(0);
                if (lane < bs) s = m0 * Yb[(long long)lane * ldy + c];
                if (lane + 32 < bs) s = fma(m1, Yb[(long long)(lane + 32) * ldy + c], s);
                s = warp_sum(s);
                if (lane == 0) Yr[(long long)i * ldy + c] -= s;
            }
        }
    } else {
        for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < rows; i += gridDim.x * blockDim.x) {
            for (int c = 0; c < nrhs; c++) {
                T s = T(0);
                for (int j = 0; j < bs; j++) s = fma(T(M[(long long)j * ldm + i]), Yb[(long long)j * ldy + c], s);
                Yr[(long long)i * ldy + c] -= s;
            }
        }
    }
}

// ------------------------------------------------------------ GMRES (FP64) --
// partial[j * P + blk] = sum over this block's chunk of V[j][i] * w[i], j < k1.
static __global__ void multi_dot_kernel(const double *__restrict__ V, long long ldv, int k1, const double *__restrict__ w, int n,
                                 double *partial) {
    __shared__ double red[8];
    const int j = blockIdx.y, P = gridDim.x;
    const int chunk = (n + P - 1) / P, lo = blockIdx.x * chunk, hi = min(n, lo + chunk);
    double s = 0.0;
    const double *v = V + (long long)j * ldv;
    for (int i = lo + threadIdx.x; i < hi; i += blockDim.x) s = fma(v[i], w[i], s);
    s = warp_sum(s);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = s;
    __syncthreads();
    if (threadIdx.x == 0) {
        double t = 0.0;
        for (int q = 0; q < (int)(blockDim.x >> 5); q++) t += red[q];
        partial[(long long)j * P + blockIdx.x] = t;
    }
}

// out[j] (+)= sum_p partial[j * P + p] in order (deterministic); accumulate != 0 adds.
static __global__ void reduce_partials_kernel(const double *partial, int P, int k1, double *out, int accumulate) {
    const int j = threadIdx.x;
    if (j >= k1) return;
    double t = 0.0;
    for (int p = 0; p < P; p++) t += partial[(long long)j * P + p];
    out[j] = accumulate ? out[j] + t : t;
}

// w[i] -= sum_j h[j] V[j][i]
static __global__ void multi_axpy_kernel(double *__restrict__ w, const double *__restrict__ V, long long ldv, int k1,
                                  const double *__restrict__ h, int n) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        double s = w[i];
        for (int j = 0; j < k1; j++) s = fma(-h[j], V[(long long)j * ldv + i], s);
        w[i] = s;
    }
}

// dst = src * (1 / sqrt(*nrm2)) and, when col != nullptr, col[0] = sqrt(*nrm2).
static __global__ void normalize_kernel(double *__restrict__ dst, const double *__restrict__ src, int n, const double *nrm2,
                                 double *col) {
    const double nr = sqrt(*nrm2);
    const double inv = nr > 0 ? 1.0 / nr : 0.0;
    if (col && blockIdx.x == 0 && threadIdx.x == 0) col[0] = nr;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) dst[i] = src[i] * inv;
}

// Arnoldi step k of GMRES: H column k holds h[0..k+1] (h[k+1] = ||w||); apply the
// previous Givens rotations, form rotation k, update g; out[0] = |g[k+1]|.
static __global__ void givens_kernel(double *H, int ldh, int k, double *cs, double *sn, double *g, double *out) {
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    double *h = H + (long long)k * ldh;  // column k stored contiguously
    for (int i = 0; i < k; i++) {
        const double t = cs[i] * h[i] + sn[i] * h[i + 1];
        h[i + 1] = -sn[i] * h[i] + cs[i] * h[i + 1];
        h[i] = t;
    }
    const double a = h[k], b = h[k + 1];
    const double r = hypot(a, b);
    const double c = r > 0 ? a / r : 1.0, s = r > 0 ? b / r : 0.0;
    cs[k] = c;
    sn[k] = s;
    h[k] = r;
    h[k + 1] = 0.0;
    g[k + 1] = -s * g[k];
    g[k] = c * g[k];
    out[0] = fabs(g[k + 1]);
}

// y = R^-1 g for the k1 x k1 upper triangle of the rotated H (columns contiguous).
static __global__ void hsolve_kernel(const double *H, int ldh, int k1, const double *g, double *y) {
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    for (int i = k1 - 1; i >= 0; i--) {
        double s = g[i];
        for (int j = i + 1; j < k1; j++) s -= H[(long long)j * ldh + i] * y[j];
        const double d = H[(long long)i * ldh + i];
        y[i] = d != 0 ? s / d : 0.0;
    }
}

// x[i] += sum_j y[j] V[j][i]
static __global__ void combine_kernel(double *__restrict__ x, const double *__restrict__ V, long long ldv, int k1,
                               const double *__restrict__ y, int n) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        double s = x[i];
        for (int j = 0; j < k1; j++) s = fma(y[j], V[(long long)j * ldv + i], s);
        x[i] = s;
    }
}

// ------------------------------------------------------- mixed-precision least squares --
// A32 = (float)A for an m x n matrix (row strides lda / ld32) and ||A||_inf in FP64 into
// *anorm_bits. Warp per row.
static __global__ void to_f32_rect_kernel(const double *__restrict__ A, long long lda, int m, int n,
                                          float *__restrict__ A32, long long ld32, unsigned long long *anorm_bits) {
    const int lane = threadIdx.x & 31;
    const int wpb = blockDim.x >> 5;
    for (int i = blockIdx.x * wpb + (threadIdx.x >> 5); i < m; i += gridDim.x * wpb) {
        const double *row = A + (long long)i * lda;
        float *out = A32 + (long long)i * ld32;
        double s = 0.0;
        for (int j = lane; j < n; j += 32) {
            const double v = row[j];
            out[j] = (float)v;
            s += fabs(v);
        }
        s = warp_sum(s);
        if (lane == 0) atomic_max_nonneg(anorm_bits, s);
    }
}

// r = b - A x for an m x n matrix and one right-hand side, FP64; warp per row.
static __global__ void resid_rect_kernel(const double *__restrict__ A, long long lda, int m, int n,
                                         const double *__restrict__ x, const double *__restrict__ b,
                                         double *__restrict__ r) {
    const int lane = threadIdx.x & 31;
    const int wpb = blockDim.x >> 5;
    for (int i = blockIdx.x * wpb + (threadIdx.x >> 5); i < m; i += gridDim.x * wpb) {
        const double *row = A + (long long)i * lda;
        double s0 = 0.0, s1 = 0.0;
        int j = lane;
        for (; j + 32 < n; j += 64) {
            s0 = fma(row[j], x[j], s0);
            s1 = fma(row[j + 32], x[j + 32], s1);
        }
        if (j < n) s0 = fma(row[j], x[j], s0);
        const double sum = warp_sum(s0 + s1);
        if (lane == 0) r[i] = b[i] - sum;
    }
}

// partial[c * n + j] = sum over the rows i of chunk c (rows_per rows) of A[i][j] r[i]:
// thread per column (coalesced rows), four independent accumulators.
static __global__ void gemv_t_partial_kernel(const double *__restrict__ A, long long lda, int m, int n,
                                             const double *__restrict__ r, int rows_per, double *__restrict__ partial) {
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= n) return;
    const int i0 = blockIdx.y * rows_per, i1 = min(m, i0 + rows_per);
    double a0 = 0.0, a1 = 0.0, a2 = 0.0, a3 = 0.0;
    int i = i0;
    for (; i + 3 < i1; i += 4) {
        a0 = fma(A[(long long)i * lda + j], r[i], a0);
        a1 = fma(A[(long long)(i + 1) * lda + j], r[i + 1], a1);
        a2 = fma(A[(long long)(i + 2) * lda + j], r[i + 2], a2);
        a3 = fma(A[(long long)(i + 3) * lda + j], r[i + 3], a3);
    }
    for (; i < i1; i++) a0 = fma(A[(long long)i * lda + j], r[i], a0);
    partial[(long long)blockIdx.y * n + j] = (a0 + a1) + (a2 + a3);
}

// g[j] = sum over chunks c (in order) of partial[c * n + j].
static __global__ void reduce_chunks_kernel(const double *__restrict__ partial, int chunks, int n, double *__restrict__ g) {
    for (int j = blockIdx.x * blockDim.x + threadIdx.x; j < n; j += gridDim.x * blockDim.x) {
        double s = 0.0;
        for (int c = 0; c < chunks; c++) s += partial[(long long)c * n + j];
        g[j] = s;
    }
}

// L = R^T (lower, row stride n) from the n x n upper triangle R at the top of a compact
// QR (row stride ldq); the strict upper part of L is zero.
static __global__ void upper_to_lower_t_kernel(const float *__restrict__ QR, long long ldq, int n, float *__restrict__ L) {
    const long long total = (long long)n * n;
    for (long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x; e < total; e += (long long)gridDim.x * blockDim.x) {
        const int i = (int)(e / n), j = (int)(e - (long long)i * n);
        L[e] = j <= i ? QR[(long long)j * ldq + i] : 0.f;
    }
}

// x += d
static __global__ void add_kernel(double *__restrict__ x, const double *__restrict__ d, int n) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) x[i] += d[i];
}

}  // namespace rl
