// Systems with n <= 32 solved by one warp each (used by batch_solve_kernel once its
// largest-first queue reaches them): lane i owns row i of the matrix in a padded
// per-warp shared tile (row stride 33, conflict-free both by rows and by columns), the
// factorisation and the triangular solves move values by shuffles, and no CTA barrier
// is involved, so the CTA's eight warps work on eight systems at once. The arithmetic
// follows the one-CTA path: partial pivoting with the first maximum on ties, FP32
// multipliers by the reciprocal (FP64 by division), the Cholesky diagonal stored as
// d / sqrt(d), FP64 residuals and the same refinement stopping rules.
#pragma once

#include "factor_cta.cuh"

// (included by batch.cuh after BatchDesc and kU64)

namespace rl {

constexpr int WARP_NMAX = 32;
constexpr int WARP_LDT = 33;  // tile row stride

// Factor the n x n tile (lane i = row i) in place. LU: rows are swapped in the tile and
// `perm` (per lane) follows them (position i holds original row perm). Uniform status.
template <class T>
__device__ int warp_factor(T *tile, int n, int kind, int &perm, T tiny) {
    const int lane = threadIdx.x & 31;
    perm = lane;
    if (kind == 0) {
        for (int j = 0; j < n; j++) {
            T v = (lane >= j && lane < n) ? absT(tile[lane * WARP_LDT + j]) : T(-1);
            int idx = lane;
            if (!(v >= T(0))) {  // not a candidate (outside the column, or NaN, which never wins)
                v = T(-1);
                idx = INT_MAX;
            }
            warp_amax(v, idx);  // largest |a|, smallest position on ties; the same in every lane
            if (idx == INT_MAX) {  // no comparable candidate (NaNs): keep the diagonal
                idx = j;
                v = absT(tile[j * WARP_LDT + j]);
            }
            if (v < tiny) return RL_ERR_DIV_BY_ZERO;
            if (idx != j) {
                const T a = tile[j * WARP_LDT + lane], b = tile[idx * WARP_LDT + lane];
                __syncwarp();
                tile[j * WARP_LDT + lane] = b;
                tile[idx * WARP_LDT + lane] = a;
                const int pj = __shfl_sync(0xffffffffu, perm, j), pi = __shfl_sync(0xffffffffu, perm, idx);
                if (lane == j) perm = pi;
                if (lane == idx) perm = pj;
            }
            __syncwarp();
            const T p = tile[j * WARP_LDT + j];
            const T inv_p = T(1) / p;
            if (lane > j && lane < n) {
                T *row = tile + lane * WARP_LDT;
                const T l = sizeof(T) == 8 ? row[j] / p : row[j] * inv_p;
                row[j] = l;
                for (int c = j + 1; c < n; c++) row[c] = fma(-l, tile[j * WARP_LDT + c], row[c]);
            }
            __syncwarp();
        }
        return RL_OK;
    }
    for (int j = 0; j < n; j++) {
        const T d = tile[j * WARP_LDT + j];
        if (absT(d) < tiny || d < T(0)) return RL_ERR_DECOMP_FAILURE;
        const T s = sqrt(d);
        const T inv = T(1) / s;
        T li = T(0);
        if (lane >= j && lane < n) {
            const T cr = tile[lane * WARP_LDT + j];
            li = cr * inv;  // update factor; the stored entry keeps the division
            tile[lane * WARP_LDT + j] = cr / s;
        }
        __syncwarp();
        for (int c = j + 1; c < n; c++) {
            const T lc = __shfl_sync(0xffffffffu, li, c);
            if (lane >= c && lane < n) tile[lane * WARP_LDT + c] = fma(-li, lc, tile[lane * WARP_LDT + c]);
        }
        __syncwarp();
    }
    return RL_OK;
}

// w (lane i holds w_i, already permuted for LU) <- A_f^-1 w with the factored tile.
// A pivot of U or a diagonal of L below tiny returns RL_ERR_DIV_BY_ZERO.
template <class T>
__device__ int warp_factor_solve(const T *tile, int n, int kind, T &w, T tiny) {
    const int lane = threadIdx.x & 31;
    const T d = lane < n ? tile[lane * WARP_LDT + lane] : T(1);
    if (__any_sync(0xffffffffu, lane < n && kind != 0 && absT(d) < tiny)) return RL_ERR_DIV_BY_ZERO;
    const T inv = T(1) / d;
    // forward: unit L (LU) or L (Cholesky)
    for (int j = 0; j < n; j++) {
        if (kind != 0 && lane == j) w = sizeof(T) == 8 ? w / d : w * inv;
        const T yj = __shfl_sync(0xffffffffu, w, j);
        if (lane > j && lane < n) w = fma(-tile[lane * WARP_LDT + j], yj, w);
    }
    if (kind == 0 && __any_sync(0xffffffffu, lane < n && absT(d) < tiny)) return RL_ERR_DIV_BY_ZERO;
    // backward: U (LU) or L^T (Cholesky: lane i reads column i of L)
    for (int j = n - 1; j >= 0; j--) {
        if (lane == j) w = sizeof(T) == 8 ? w / d : w * inv;
        const T xj = __shfl_sync(0xffffffffu, w, j);
        if (lane < j) w = fma(-(kind == 0 ? tile[lane * WARP_LDT + j] : tile[j * WARP_LDT + lane]), xj, w);
    }
    return RL_OK;
}

// FP64 residual r_i = b_i - sum_j A_ij x_j (lane i; A row-major, row stride n), and
// max |r_i| over the warp.
template <class TI>
__device__ double warp_residual(const TI *__restrict__ A, int n, double bl, double x, double &r) {
    const int lane = threadIdx.x & 31;
    double s = 0.0;
    for (int j = 0; j < n; j++) {
        const double xj = __shfl_sync(0xffffffffu, x, j);
        if (lane < n) s = fma((double)A[lane * n + j], xj, s);
    }
    r = lane < n ? bl - s : 0.0;
    return warp_max(fabs(r));
}

// One system by one warp; `tile` is the warp's WARP_NMAX x WARP_LDT slice of shared
// memory. Writes x, info, iters, berr like batch_solve_one; mixed-precision failures go
// to the FP64 fallback list.
template <class TI, class TF, bool MIXED>
__device__ void warp_solve_small(const BatchDesc &d, int sys, const TI *__restrict__ A, const TI *__restrict__ B,
                                 TI *__restrict__ X, TF *tile) {
    const int lane = threadIdx.x & 31;
    const int n = d.n[sys], kind = d.kind[sys];
    const TI *Ai = A + d.a_off[sys];
    const TI *bi = B + d.b_off[sys];
    TI *xi = X + d.b_off[sys];
    auto finish = [&](int st, int iters, double berr, double x) {
        if (st == RL_OK && lane < n) xi[lane] = (TI)x;
        if (lane == 0) {
            d.info[sys] = st;
            if (d.iters) d.iters[sys] = iters;
            if (d.berr) d.berr[sys] = berr;
        }
    };
    auto fallback = [&]() {
        if (lane == 0) d.fb_list[atomicAdd(d.fb_count, 1)] = sys;
    };
    if (n == 0) {
        finish(RL_OK, 0, 0.0, 0.0);
        return;
    }
    if (n > WARP_NMAX) {  // never scheduled here (see kWarpCost); refuse rather than overrun the tile
        if (MIXED)
            fallback();
        else
            finish(RL_ERR_INVALID_ARG, d.iters_tag, 0.0, 0.0);
        return;
    }
    // the matrix in the factor type, rows read coalesced; ||A||_inf of that copy
    for (int r = 0; r < n; r++) tile[r * WARP_LDT + lane] = lane < n ? convert_to<TF>(Ai[r * n + lane]) : TF(0);
    __syncwarp();
    TF rs = TF(0);
    if (lane < n)
        for (int j = 0; j < n; j++) rs += absT(tile[lane * WARP_LDT + j]);
    const double anorm = warp_max((double)rs);
    const double bl = lane < n ? (double)bi[lane] : 0.0;
    const double bnorm = warp_max(fabs(bl));
    const TF tiny = MIXED ? TF(FLT_MIN) : Eps<TF>::value;
    int perm = lane;
    int st = warp_factor<TF>(tile, n, kind, perm, tiny);
    TF w = TF(0);
    if (st == RL_OK) {
        const int src = kind == 0 ? perm : lane;
        w = lane < n ? (TF)bi[src < n ? src : 0] : TF(0);
        st = warp_factor_solve<TF>(tile, n, kind, w, tiny);
    }
    if (st != RL_OK) {
        if (MIXED)
            fallback();
        else
            finish(st, d.iters_tag, 0.0, 0.0);
        return;
    }
    double x = (double)w, r = 0.0;
    if (!MIXED) {
        const double rn = warp_residual(Ai, n, bl, x, r);
        const double xn = warp_max(fabs(x));
        const double den = anorm * xn + bnorm;
        finish(RL_OK, d.iters_tag, den > 0 ? rn / den : 0.0, x);
        return;
    }
    const double stop = sqrt((double)n) * kU64;
    double prev = INFINITY, rn = 0.0, xn = 0.0;
    bool ok = false;
    int it = 0;
    for (;; it++) {
        rn = warp_residual(Ai, n, bl, x, r);
        xn = warp_max(fabs(x));
        if (rn <= stop * anorm * xn) {
            ok = true;
            break;
        }
        if (it >= d.max_iters) break;
        if (it >= 2 && rn > 0.5 * prev) {
            ok = rn <= 10.0 * n * kU64 * (anorm * xn + bnorm);
            break;
        }
        prev = rn;
        const double scale = 1.0 / rn;
        const double rp = __shfl_sync(0xffffffffu, r, kind == 0 ? perm : lane);  // P r for LU
        TF c = lane < n ? (TF)(rp * scale) : TF(0);
        if (warp_factor_solve<TF>(tile, n, kind, c, tiny) != RL_OK) break;
        x = fma(rn, (double)c, x);
    }
    if (ok) {
        const double den = anorm * xn + bnorm;
        finish(RL_OK, it, den > 0 ? rn / den : 0.0, x);
    } else {
        fallback();
    }
}

}  // namespace rl
