// Mixed-precision single-system machinery shared by the solver entry points and the
// serving loop: FP64 residuals and norms, the FP32-factor preconditioner, GMRES-IR, the
// plain FP64 solve and the solver driver.
#pragma once

#include <cfloat>
#include <chrono>
#include <cmath>
#include <cstring>
#include <vector>

#include "dense_ops.cuh"

namespace rl {


constexpr double kU = 1.1102230246251565e-16;  // 2^-53

struct SolveOut {
    int iters = 0, gmres = 0, path = RL_PATH_REFINEMENT;
    double berr = 0.0;
};

inline int grid_rows(int rows, int per_block) {
    return std::max(1, std::min(8 * num_sms(), ceil_div(rows, per_block)));
}

inline double bits_to_double(unsigned long long b) {
    double d;
    memcpy(&d, &b, sizeof d);
    return d;
}

// R = B - A X (B == nullptr: R = A X), FP64.
inline rl_status residual_dev(const double *A, long long lda, int n, const double *X, long long ldx, const double *B,
                       long long ldb, double *R, long long ldr, int nrhs, cudaStream_t s) {
    if (nrhs <= 4) {
        // instantiated for the exact count: the FP64 pipe spends its ~64 cycles on a warp
        // DFMA whose predicate is off as well, so a 4-column instance on one column costs 4x
        const int g = grid_rows(n, 8);
        if (nrhs == 1)
            RL_LAUNCH(residual_gemv_kernel<1>, g, 256, 0, s, A, lda, n, X, ldx, B, ldb, R, ldr, nrhs);
        else if (nrhs == 2)
            RL_LAUNCH(residual_gemv_kernel<2>, g, 256, 0, s, A, lda, n, X, ldx, B, ldb, R, ldr, nrhs);
        else
            RL_LAUNCH(residual_gemv_kernel<4>, g, 256, 0, s, A, lda, n, X, ldx, B, ldb, R, ldr, nrhs);
        return RL_OK;
    }
    if (B)
        RL_TRY_CUDA(cudaMemcpy2DAsync(R, ldr * sizeof(double), B, ldb * sizeof(double), nrhs * sizeof(double), n,
                                      cudaMemcpyDeviceToDevice, s));
    return gemm<double, false, false>(n, nrhs, n, B ? -1.0 : 1.0, A, lda, X, ldx, B ? 1.0 : 0.0, R, ldr, s);
}

inline rl_status colnorm_dev(const double *V, long long ldv, int n, int nrhs, unsigned long long *out, cudaStream_t s) {
    RL_TRY_CUDA(cudaMemsetAsync(out, 0, nrhs * sizeof(unsigned long long), s));
    const long long tot = (long long)n * nrhs;
    RL_LAUNCH(colnorm_kernel, (int)std::min<long long>(4 * num_sms(), (tot + 255) / 256), 256, 0, s, V, ldv, n, nrhs, out);
    return RL_OK;
}

// Inverted 64 x 64 diagonal blocks of the two triangles of an FP32 factor (FP32, formed
// once) and the sweep flags that use them: the form of RL_TUNE_MIXED_SWEEP_INV.
struct SweepInv {
    const float *D1 = nullptr, *D2 = nullptr;
    int *ctl = nullptr;  // 2 x sweep_ctl_words(n, nrhs) words, zeroed before each pair of sweeps
};

// W <- M^-1 W with the FP32 factor (LU: ipiv swaps, unit L, U; Cholesky: L, L^T). No
// absolute-epsilon rule here: only a pivot below FLT_MIN counts as singular. With inv.D1
// set, the sweeps apply the diagonal blocks' inverses (up to kSweepGroups x kSweepRhs
// right-hand sides).
inline rl_status precond_solve(const float *F, int n, int kind, const int *ipiv, float *W, long long ldw, int nrhs,
                               int *dstatus, cudaStream_t s, const SweepInv &inv = SweepInv()) {
    const float tiny = FLT_MIN;
    const int m1 = kind == RL_KIND_LU ? 0 : 1, m2 = kind == RL_KIND_LU ? 2 : 3;
    if (kind == RL_KIND_LU) RL_TRY(laswp<float>(W, ldw, nrhs, 0, 0, ipiv, 0, n, s));
    if (inv.D1 && sweep_groups(nrhs) > 0) {
        const int words = sweep_ctl_words(n, nrhs);
        RL_TRY_CUDA(cudaMemsetAsync(inv.ctl, 0, 2 * words * sizeof(int), s));
        RL_TRY((tri_solve_inv_dev<float, float>(F, n, n, inv.D1, W, ldw, nrhs, m1, dstatus, s, tiny, inv.ctl)));
        return tri_solve_inv_dev<float, float>(F, n, n, inv.D2, W, ldw, nrhs, m2, dstatus, s, tiny, inv.ctl + words);
    }
    RL_TRY(tri_solve_dev<float>(F, n, n, W, ldw, nrhs, m1, dstatus, s, tiny));
    return tri_solve_dev<float>(F, n, n, W, ldw, nrhs, m2, dstatus, s, tiny);
}

// dst = M^-1 src for one FP64 vector with the solves in FP32 (the vector scaled by its
// inf-norm around them): the semi-normal-equations preconditioner of lstsq_mixed.
struct Minv32 {
    const float *F;
    int n, kind;
    const int *ipiv;
    float *w32;
    unsigned long long *bits;  // 1 scale
    int *one;                  // device int 1
    int *dstatus;
    rl_status apply(const double *src, double *dst, cudaStream_t s) const {
        RL_TRY(colnorm_dev(src, 1, n, 1, bits, s));
        const int g = std::min(4 * num_sms(), ceil_div(n, 256));
        RL_LAUNCH(scale_to_f32_kernel, g, 256, 0, s, src, 1LL, n, 1, bits, w32, 1LL);
        RL_TRY(precond_solve(F, n, kind, ipiv, w32, 1, 1, dstatus, s));
        RL_TRY_CUDA(cudaMemsetAsync(dst, 0, n * sizeof(double), s));
        RL_LAUNCH(update_x_kernel, g, 256, 0, s, dst, 1LL, w32, 1LL, n, 1, bits, one);
        return RL_OK;
    }
};

// dst = M^-1 src for one FP64 vector: the FP32 factor's row swaps and triangular solves
// in FP64 arithmetic, the factor's entries widened as they are read. Applied in the
// working precision the preconditioner lets GMRES-IR converge where the FP32-applied form
// stalls (Carson & Higham's analysis assumes it; on kappa = 1e8 systems with geometric
// singular values, n = 1024, a CPU model of both took 121 against 313 GMRES iterations).
// The block solves use the FP64 inverses of the two triangles' 64 x 64 diagonal blocks
// (D1 for L, D2 for U or L^T), formed once by init().
struct Minv {
    const float *F;
    int n, kind;
    const int *ipiv;
    int *dstatus;
    DevBuf<double> D1, D2;
    DevBuf<int> ctl;  // the two sweeps' ticket and block flags
    int mode1() const { return kind == RL_KIND_LU ? 0 : 1; }
    int mode2() const { return kind == RL_KIND_LU ? 2 : 3; }
    rl_status init(cudaStream_t s) {
        const size_t blocks = (size_t)ceil_div(n, kSweepRows) * kSweepRows * kSweepRows;
        RL_TRY(D1.alloc(blocks, s));
        RL_TRY(D2.alloc(blocks, s));
        RL_TRY(ctl.alloc(2 * (size_t)(1 + ceil_div(n, kSweepRows)), s));
        RL_TRY((diag_inverse<double, float>(F, n, n, mode1(), D1.p, dstatus, s, FLT_MIN)));
        return diag_inverse<double, float>(F, n, n, mode2(), D2.p, dstatus, s, FLT_MIN);
    }
    rl_status apply(const double *src, double *dst, cudaStream_t s) const {
        RL_TRY_CUDA(cudaMemcpyAsync(dst, src, n * sizeof(double), cudaMemcpyDeviceToDevice, s));
        const double tiny = FLT_MIN;
        if (kind == RL_KIND_LU) RL_TRY(laswp<double>(dst, 1, 1, 0, 0, ipiv, 0, n, s));
        const int words = 1 + ceil_div(n, kSweepRows);
        RL_TRY_CUDA(cudaMemsetAsync(ctl.p, 0, 2 * words * sizeof(int), s));
        RL_TRY((tri_solve_inv_dev<double, float>(F, n, n, D1.p, dst, 1, 1, mode1(), dstatus, s, tiny, ctl.p)));
        return tri_solve_inv_dev<double, float>(F, n, n, D2.p, dst, 1, 1, mode2(), dstatus, s, tiny, ctl.p + words);
    }
};

// Deterministic dot products h[j] = V[j] . w (j < k1) into out (accumulate adds).
struct Dots {
    double *partial;
    int P;
    rl_status run(const double *V, long long ldv, int k1, const double *w, int n, double *out, int accumulate,
                  cudaStream_t s) const {
        RL_LAUNCH(multi_dot_kernel, dim3(P, k1), 256, 0, s, V, ldv, k1, w, n, partial);
        RL_LAUNCH(reduce_partials_kernel, 1, 128, 0, s, partial, P, k1, out, accumulate);
        return RL_OK;
    }
};

// GMRES-IR on one column: x (contiguous, FP64) refined against b until the FP64
// backward-error test passes. Restarted GMRES(m) in FP64 on M^-1 A d = M^-1 r with
// CGS2 orthogonalisation; Givens rotations and the small triangular solve on the GPU.
// It gives up (ok = false) when a restart cycle does not cut the residual tenfold or when
// the host clock passes `deadline` (seconds, host_seconds()): past that an FP64
// refactorisation is the cheaper way to the answer.
inline double host_seconds() {
    return std::chrono::duration<double>(std::chrono::steady_clock::now().time_since_epoch()).count();
}

inline rl_status gmres_ir(const double *A, long long lda, int n, const Minv &M, const double *b, double *x, double anorm,
                   double bnorm, double deadline, SolveOut &out, bool &ok, cudaStream_t s) {
    NvtxRange nvtx_("rl.mixed.gmres_ir");
    constexpr int m = 64, outer_max = 5;
    const double inner_tol = 1e-8;
    DevBuf<double> V, H, cs, sn, g, y, w, r, t, nrm2, partial;
    DevBuf<unsigned long long> bits;
    const int P = std::min(2 * num_sms(), std::max(1, ceil_div(n, 2048)));
    RL_TRY(V.alloc((size_t)(m + 1) * n, s));
    RL_TRY(H.alloc((size_t)m * (m + 1), s));
    RL_TRY(cs.alloc(m, s));
    RL_TRY(sn.alloc(m, s));
    RL_TRY(g.alloc(m + 1, s));
    RL_TRY(y.alloc(m, s));
    RL_TRY(w.alloc(n, s));
    RL_TRY(r.alloc(n, s));
    RL_TRY(t.alloc(m + 1, s));
    RL_TRY(nrm2.alloc(1, s));
    RL_TRY(partial.alloc((size_t)P * (m + 1), s));
    RL_TRY(bits.alloc(2, s));
    Dots dots{partial.p, P};
    const int gv = std::min(4 * num_sms(), ceil_div(n, 256));
    ok = false;
    double prev_rn = INFINITY;
    for (int outer = 0; outer < outer_max; outer++) {
        RL_TRY(residual_dev(A, lda, n, x, 1, b, 1, r.p, 1, 1, s));
        RL_TRY(colnorm_dev(r.p, 1, n, 1, bits.p, s));
        RL_TRY(colnorm_dev(x, 1, n, 1, bits.p + 1, s));
        unsigned long long hb[2];
        RL_TRY_CUDA(cudaMemcpyAsync(hb, bits.p, sizeof hb, cudaMemcpyDeviceToHost, s));
        RL_TRY_CUDA(cudaStreamSynchronize(s));
        const double rn = bits_to_double(hb[0]), xn = bits_to_double(hb[1]);
        const double den = anorm * xn + bnorm;
        out.berr = den > 0 ? rn / den : 0.0;
        if (rn <= std::sqrt((double)n) * kU * anorm * xn) {
            ok = true;
            return RL_OK;
        }
        if (outer == outer_max - 1 || !(rn <= 0.1 * prev_rn)) {  // out of budget, or no progress:
            ok = out.berr <= 10.0 * n * kU;                        // accept within the 10 n u bound
            return RL_OK;
        }
        prev_rn = rn;
        // z = M^-1 r -> V[0] = z / ||z||, g = (||z||, 0, ...)
        RL_TRY(M.apply(r.p, w.p, s));
        RL_TRY(dots.run(w.p, 0, 1, w.p, n, nrm2.p, 0, s));
        RL_TRY_CUDA(cudaMemsetAsync(g.p, 0, (m + 1) * sizeof(double), s));
        RL_TRY_CUDA(cudaMemsetAsync(H.p, 0, (size_t)m * (m + 1) * sizeof(double), s));
        RL_LAUNCH(normalize_kernel, gv, 256, 0, s, V.p, w.p, n, nrm2.p, g.p);
        double beta = 0.0;
        RL_TRY_CUDA(cudaMemcpyAsync(&beta, g.p, sizeof beta, cudaMemcpyDeviceToHost, s));
        RL_TRY_CUDA(cudaStreamSynchronize(s));
        if (!(beta > 0)) return RL_OK;  // breakdown: let the caller refactor in FP64
        int k1 = 0;
        for (int k = 0; k < m; k++) {
            double *vk = V.p + (size_t)k * n;
            double *hk = H.p + (size_t)k * (m + 1);
            RL_TRY(residual_dev(A, lda, n, vk, 1, nullptr, 0, r.p, 1, 1, s));  // r = A v_k
            RL_TRY(M.apply(r.p, w.p, s));                                    // w = M^-1 A v_k
            // CGS2: h = V^T w, w -= V h, twice
            RL_TRY(dots.run(V.p, n, k + 1, w.p, n, hk, 0, s));
            RL_LAUNCH(multi_axpy_kernel, gv, 256, 0, s, w.p, V.p, (long long)n, k + 1, hk, n);
            RL_TRY(dots.run(V.p, n, k + 1, w.p, n, t.p, 0, s));
            RL_LAUNCH(multi_axpy_kernel, gv, 256, 0, s, w.p, V.p, (long long)n, k + 1, t.p, n);
            // h += t: reduce the second pass's partial sums (still in place) into h
            RL_LAUNCH(reduce_partials_kernel, 1, 128, 0, s, partial.p, P, k + 1, hk, 1);
            RL_TRY(dots.run(w.p, 0, 1, w.p, n, nrm2.p, 0, s));
            RL_LAUNCH(normalize_kernel, gv, 256, 0, s, V.p + (size_t)(k + 1) * n, w.p, n, nrm2.p, hk + k + 1);
            RL_LAUNCH(givens_kernel, 1, 32, 0, s, H.p, m + 1, k, cs.p, sn.p, g.p, nrm2.p);
            double res = 0.0;
            RL_TRY_CUDA(cudaMemcpyAsync(&res, nrm2.p, sizeof res, cudaMemcpyDeviceToHost, s));
            RL_TRY_CUDA(cudaStreamSynchronize(s));
            out.gmres++;
            k1 = k + 1;
            if (!(res > inner_tol * beta)) break;
            if (host_seconds() > deadline) return RL_OK;  // over budget: ok stays false
            // stagnating in the first cycle (a preconditioner too far off, kappa u_32 >> 1):
            // the refactor is cheaper than the iterations still ahead
            if (outer == 0 && k + 1 == 32 && res > 1e-3 * beta) return RL_OK;
        }
        RL_LAUNCH(hsolve_kernel, 1, 32, 0, s, H.p, m + 1, k1, g.p, y.p);
        RL_LAUNCH(combine_kernel, gv, 256, 0, s, x, V.p, (long long)n, k1, y.p, n);
        out.iters++;
    }
    return RL_OK;
}

// Plain FP64: copy A, factor, solve X = A^-1 B (LU: reference epsilon rules).
inline rl_status solve_fp64(const double *A, long long lda, int n, int kind, const double *B, long long ldb, double *X,
                     long long ldx, int nrhs, cudaStream_t s) {
    DevBuf<double> F;
    DevBuf<int> ipiv, st;
    RL_TRY(F.alloc((size_t)n * n, s));
    RL_TRY(ipiv.alloc(n, s));
    RL_TRY(st.alloc(1, s));
    RL_TRY_CUDA(cudaMemsetAsync(st.p, 0, sizeof(int), s));
    RL_TRY_CUDA(cudaMemcpy2DAsync(F.p, n * sizeof(double), A, lda * sizeof(double), n * sizeof(double), n,
                                  cudaMemcpyDeviceToDevice, s));
    RL_TRY_CUDA(cudaMemcpy2DAsync(X, ldx * sizeof(double), B, ldb * sizeof(double), nrhs * sizeof(double), n,
                                  cudaMemcpyDeviceToDevice, s));
    if (kind == RL_KIND_LU) {
        RL_TRY(lu_factor_dev<double>(F.p, n, n, ipiv.p, s));
        RL_TRY(laswp<double>(X, ldx, nrhs, 0, 0, ipiv.p, 0, n, s));
        RL_TRY(tri_solve_dev<double>(F.p, n, n, X, ldx, nrhs, 0, st.p, s));
        RL_TRY(tri_solve_dev<double>(F.p, n, n, X, ldx, nrhs, 2, st.p, s));
    } else {
        RL_TRY(chol_factor_dev<double>(F.p, n, n, s));
        RL_TRY(tri_solve_dev<double>(F.p, n, n, X, ldx, nrhs, 1, st.p, s));
        RL_TRY(tri_solve_dev<double>(F.p, n, n, X, ldx, nrhs, 3, st.p, s));
    }
    return read_status<double>(st.p, s);
}

// max over columns of the normwise backward error ||b - A x|| / (||A|| ||x|| + ||b||).
inline rl_status backward_error_dev(const double *A, long long lda, int n, const double *X, long long ldx, const double *B,
                             long long ldb, int nrhs, double &berr, cudaStream_t s) {
    DevBuf<double> R;
    DevBuf<unsigned long long> bits;
    RL_TRY(R.alloc((size_t)n * nrhs, s));
    RL_TRY(bits.alloc(3 * nrhs + 1, s));
    RL_TRY(residual_dev(A, lda, n, X, ldx, B, ldb, R.p, nrhs, nrhs, s));
    RL_TRY(colnorm_dev(R.p, nrhs, n, nrhs, bits.p, s));
    RL_TRY(colnorm_dev(X, ldx, n, nrhs, bits.p + nrhs, s));
    RL_TRY(colnorm_dev(B, ldb, n, nrhs, bits.p + 2 * nrhs, s));
    RL_TRY_CUDA(cudaMemsetAsync(bits.p + 3 * nrhs, 0, sizeof(unsigned long long), s));
    RL_LAUNCH(rownorm_kernel, grid_rows(n, 8), 256, 0, s, A, lda, n, bits.p + 3 * nrhs);
    std::vector<unsigned long long> hb(3 * nrhs + 1);
    RL_TRY_CUDA(cudaMemcpyAsync(hb.data(), bits.p, hb.size() * sizeof(unsigned long long), cudaMemcpyDeviceToHost, s));
    RL_TRY_CUDA(cudaStreamSynchronize(s));
    const double anorm = bits_to_double(hb[3 * nrhs]);
    berr = 0.0;
    for (int c = 0; c < nrhs; c++) {
        const double den = anorm * bits_to_double(hb[nrhs + c]) + bits_to_double(hb[2 * nrhs + c]);
        berr = std::max(berr, den > 0 ? bits_to_double(hb[c]) / den : 0.0);
    }
    return RL_OK;
}

// A matrix factored for mixed-precision solves: the FP32 factor (LU with pivots, or
// Cholesky) and ||A||_inf, with the FP64 matrix kept for residuals (borrowed from the
// caller, or an owned device copy for resident factors). solve() may be called any
// number of times with new right-hand sides; the FP64 factor is built only if a solve
// needs the fallback, and kept.
struct MixedFactor {
    int n = 0, kind = RL_KIND_LU;
    const double *A = nullptr;
    long long lda = 0;
    double *A_own = nullptr;
    float *F = nullptr;
    int *ipiv = nullptr;
    double anorm = 0.0;
    bool f32_ok = false;
    double *F64 = nullptr;
    int *ipiv64 = nullptr;
    float *Dinv = nullptr;  // RL_TUNE_MIXED_SWEEP_INV: both triangles' inverted diagonal blocks
    rl_status f64_status = RL_OK;
    bool f64_ready = false;
    cudaStream_t home = nullptr;  // stream the buffers were allocated on

    MixedFactor() = default;
    MixedFactor(const MixedFactor &) = delete;
    MixedFactor &operator=(const MixedFactor &) = delete;
    ~MixedFactor() { release(); }

    void release() {
        void *ps[] = {A_own, F, ipiv, F64, ipiv64, Dinv};
        for (void *p : ps)
            if (p) cudaFreeAsync(p, home);
        A_own = nullptr, F = nullptr, ipiv = nullptr, F64 = nullptr, ipiv64 = nullptr, Dinv = nullptr;
    }

    size_t dinv_elems() const { return (size_t)ceil_div(n, kSweepRows) * kSweepRows * kSweepRows; }

    size_t bytes() const {
        size_t b = (size_t)n * n * sizeof(float) + (size_t)n * sizeof(int);
        if (A_own) b += (size_t)n * n * sizeof(double);
        if (F64) b += (size_t)n * n * sizeof(double) + (size_t)n * sizeof(int);
        if (Dinv) b += 2 * dinv_elems() * sizeof(float);
        return b;
    }

    // The inverted diagonal blocks for the sweeps (formed on first use).
    rl_status ensure_dinv(int *dstatus, cudaStream_t s) {
        if (Dinv) return RL_OK;
        RL_TRY(alloc(Dinv, 2 * dinv_elems(), s));
        const int m1 = kind == RL_KIND_LU ? 0 : 1, m2 = kind == RL_KIND_LU ? 2 : 3;
        RL_TRY((diag_inverse<float, float>(F, n, n, m1, Dinv, dstatus, s, FLT_MIN)));
        return diag_inverse<float, float>(F, n, n, m2, Dinv + dinv_elems(), dstatus, s, FLT_MIN);
    }

    template <class T>
    rl_status alloc(T *&p, size_t count, cudaStream_t s) {
        RL_TRY_CUDA(cudaMallocAsync(reinterpret_cast<void **>(&p), std::max<size_t>(1, count) * sizeof(T), s));
        return RL_OK;
    }

    // own = true copies A into the factor (resident factors outlive the caller's buffer);
    // adopt = true takes ownership of `a` itself (a device buffer from cudaMallocAsync).
    rl_status factor(const double *a, long long lda_, int n_, int kind_, bool own, cudaStream_t s, bool adopt = false) {
        NvtxRange nvtx_("rl.mixed.factor_fp32");
        n = n_;
        kind = kind_;
        home = s;
        if (adopt) {
            A_own = const_cast<double *>(a);
            A = a;
            lda = lda_;
        } else if (own) {
            RL_TRY(alloc(A_own, (size_t)n * n, s));
            RL_TRY_CUDA(cudaMemcpy2DAsync(A_own, n * sizeof(double), a, lda_ * sizeof(double), n * sizeof(double), n,
                                          cudaMemcpyDeviceToDevice, s));
            A = A_own;
            lda = n;
        } else {
            A = a;
            lda = lda_;
        }
        RL_TRY(alloc(F, (size_t)n * n, s));
        RL_TRY(alloc(ipiv, (size_t)n, s));
        DevBuf<unsigned long long> nb;
        RL_TRY(nb.alloc(1, s));
        RL_TRY_CUDA(cudaMemsetAsync(nb.p, 0, sizeof(unsigned long long), s));
        RL_LAUNCH(to_f32_rownorm_kernel, grid_rows(n, 8), 256, 0, s, A, lda, n, F, (long long)n, nb.p);
        const rl_status fst = kind == RL_KIND_LU ? lu_factor_dev<float>(F, n, n, ipiv, s, FLT_MIN)
                                                 : chol_factor_dev<float>(F, n, n, s, FLT_MIN);
        if (fst != RL_OK && fst != RL_ERR_DIV_BY_ZERO && fst != RL_ERR_DECOMP_FAILURE) return fst;
        f32_ok = fst == RL_OK;
        unsigned long long hb = 0;
        RL_TRY_CUDA(cudaMemcpyAsync(&hb, nb.p, sizeof hb, cudaMemcpyDeviceToHost, s));
        RL_TRY_CUDA(cudaStreamSynchronize(s));
        anorm = bits_to_double(hb);
        return RL_OK;
    }

    // FP64 factor of A (reference epsilon rules), built once.
    rl_status ensure_fp64(cudaStream_t s) {
        if (f64_ready) return f64_status;
        RL_TRY(alloc(F64, (size_t)n * n, s));
        RL_TRY(alloc(ipiv64, (size_t)n, s));
        RL_TRY_CUDA(cudaMemcpy2DAsync(F64, n * sizeof(double), A, lda * sizeof(double), n * sizeof(double), n,
                                      cudaMemcpyDeviceToDevice, s));
        f64_status = kind == RL_KIND_LU ? lu_factor_dev<double>(F64, n, n, ipiv64, s)
                                        : chol_factor_dev<double>(F64, n, n, s);
        f64_ready = true;
        return f64_status;
    }

    rl_status solve_with_fp64(const double *B, long long ldb, double *X, long long ldx, int nrhs, SolveOut &out,
                              cudaStream_t s) {
        NvtxRange nvtx_("rl.mixed.fp64_refactor_solve");
        out.path = RL_PATH_FP64;
        RL_TRY(ensure_fp64(s));
        DevBuf<int> st;
        RL_TRY(st.alloc(1, s));
        RL_TRY_CUDA(cudaMemsetAsync(st.p, 0, sizeof(int), s));
        RL_TRY_CUDA(cudaMemcpy2DAsync(X, ldx * sizeof(double), B, ldb * sizeof(double), nrhs * sizeof(double), n,
                                      cudaMemcpyDeviceToDevice, s));
        if (kind == RL_KIND_LU) {
            RL_TRY(laswp<double>(X, ldx, nrhs, 0, 0, ipiv64, 0, n, s));
            RL_TRY(tri_solve_dev<double>(F64, n, n, X, ldx, nrhs, 0, st.p, s));
            RL_TRY(tri_solve_dev<double>(F64, n, n, X, ldx, nrhs, 2, st.p, s));
        } else {
            RL_TRY(tri_solve_dev<double>(F64, n, n, X, ldx, nrhs, 1, st.p, s));
            RL_TRY(tri_solve_dev<double>(F64, n, n, X, ldx, nrhs, 3, st.p, s));
        }
        RL_TRY(read_status<double>(st.p, s));
        return backward_error_dev(A, lda, n, X, ldx, B, ldb, nrhs, out.berr, s);
    }

    rl_status solve(const double *B, long long ldb, double *X, long long ldx, int nrhs, SolveOut &out, cudaStream_t s) {
        NvtxRange nvtx_("rl.mixed.refine");
        out = SolveOut();
        if (!f32_ok) return solve_with_fp64(B, ldb, X, ldx, nrhs, out, s);
        DevBuf<float> W;
        DevBuf<double> R;
        DevBuf<int> dstatus, active;
        DevBuf<unsigned long long> nb;  // bnorm, rnorm, xnorm per column
        RL_TRY(W.alloc((size_t)n * nrhs, s));
        RL_TRY(R.alloc((size_t)n * nrhs, s));
        RL_TRY(dstatus.alloc(2, s));
        RL_TRY(active.alloc(nrhs + 1, s));
        RL_TRY(nb.alloc(3 * nrhs, s));
        unsigned long long *bn_b = nb.p, *rn_b = nb.p + nrhs, *xn_b = nb.p + 2 * nrhs;
        RL_TRY_CUDA(cudaMemsetAsync(dstatus.p, 0, 2 * sizeof(int), s));
        SweepInv inv;
        DevBuf<int> sweep_ctl;
        if (tune(RL_TUNE_MIXED_SWEEP_INV) && sweep_groups(nrhs) > 0 && n > CTA_NMAX && !g_shared_gpu) {
            RL_TRY(ensure_dinv(dstatus.p, s));
            RL_TRY(sweep_ctl.alloc(2 * (size_t)sweep_ctl_words(n, nrhs), s));
            inv = SweepInv{Dinv, Dinv + dinv_elems(), sweep_ctl.p};
        }
        std::vector<int> act(nrhs + 1, 1);
        RL_TRY_CUDA(cudaMemcpyAsync(active.p, act.data(), act.size() * sizeof(int), cudaMemcpyHostToDevice, s));
        RL_TRY(colnorm_dev(B, ldb, n, nrhs, bn_b, s));
        const long long tot = (long long)n * nrhs;
        const int ge = (int)std::min<long long>(4 * num_sms(), (tot + 255) / 256);
        std::vector<int> conv(nrhs, 0), near(nrhs, 0);
        std::vector<double> prev(nrhs, INFINITY), bnorm(nrhs, 0.0);
        // x0 = M^-1 b
        RL_LAUNCH(scale_to_f32_kernel, ge, 256, 0, s, B, ldb, n, nrhs, bn_b, W.p, (long long)nrhs);
        RL_TRY(precond_solve(F, n, kind, ipiv, W.p, nrhs, nrhs, dstatus.p, s, inv));
        RL_TRY_CUDA(cudaMemset2DAsync(X, ldx * sizeof(double), 0, nrhs * sizeof(double), n, s));
        RL_LAUNCH(update_x_kernel, ge, 256, 0, s, X, ldx, W.p, (long long)nrhs, n, nrhs, bn_b, active.p);
        std::vector<unsigned long long> hb(3 * nrhs);
        bool stalled = false, need_fp64 = false, diverged = false;
        const int max_steps = (int)tune(RL_TUNE_MIXED_REFINE_STEPS);
        for (int it = 0;; it++) {
            RL_TRY(residual_dev(A, lda, n, X, ldx, B, ldb, R.p, nrhs, nrhs, s));
            RL_TRY(colnorm_dev(R.p, nrhs, n, nrhs, rn_b, s));
            RL_TRY(colnorm_dev(X, ldx, n, nrhs, xn_b, s));
            int dst = 0;
            RL_TRY_CUDA(cudaMemcpyAsync(hb.data(), nb.p, hb.size() * sizeof(unsigned long long), cudaMemcpyDeviceToHost, s));
            RL_TRY_CUDA(cudaMemcpyAsync(&dst, dstatus.p, sizeof(int), cudaMemcpyDeviceToHost, s));
            RL_TRY_CUDA(cudaStreamSynchronize(s));
            if (dst != 0) {  // the FP32 factor met a pivot below FLT_MIN in a solve
                need_fp64 = true;
                break;
            }
            int all = 1;
            double berr = 0;
            for (int c = 0; c < nrhs; c++) {
                bnorm[c] = bits_to_double(hb[c]);
                const double rn = bits_to_double(hb[nrhs + c]), xn = bits_to_double(hb[2 * nrhs + c]);
                conv[c] = rn <= std::sqrt((double)n) * kU * anorm * xn;
                const double den = anorm * xn + bnorm[c];
                berr = std::max(berr, den > 0 ? rn / den : 0.0);
                near[c] = rn <= 10.0 * n * kU * den;
                // Stalling: less than 10% progress in a step. Slow but steady refinement
                // (kappa u_32 ~ 0.5, a step costs a GEMV and two triangular solves) is
                // cheaper to finish than an FP64 refactor; LAPACK dsgesv allows 30 steps.
                if (!conv[c] && it >= 1 && rn > 0.9 * prev[c]) stalled = true;
                // Diverging: the first correction made the residual grow (kappa u_32 > 1):
                // the FP32 factor is too far off for GMRES-IR to pay off against the refactor.
                if (!conv[c] && it == 1 && rn > prev[c]) diverged = true;
                if (!std::isfinite(rn)) stalled = diverged = true;
                prev[c] = rn;
                all &= conv[c];
                act[c] = !conv[c];
            }
            out.berr = berr;
            out.iters = it;
            // LAPACK dsgesv's test and step limit (30); a column that stalls or runs out
            // of steps is accepted within the 10 n u backward-error bound (the batched
            // solver's rule), where a large n's residual floor can sit above the test
            if (all || stalled || it >= max_steps) {
                for (int c = 0; c < nrhs; c++) conv[c] |= near[c];
                break;
            }
            RL_TRY_CUDA(cudaMemcpyAsync(active.p, act.data(), nrhs * sizeof(int), cudaMemcpyHostToDevice, s));
            RL_LAUNCH(scale_to_f32_kernel, ge, 256, 0, s, R.p, (long long)nrhs, n, nrhs, rn_b, W.p, (long long)nrhs);
            RL_TRY(precond_solve(F, n, kind, ipiv, W.p, nrhs, nrhs, dstatus.p, s, inv));
            RL_LAUNCH(update_x_kernel, ge, 256, 0, s, X, ldx, W.p, (long long)nrhs, n, nrhs, rn_b, active.p);
        }
        if (!need_fp64) {
            bool all_ok = true;
            for (int c = 0; c < nrhs; c++) all_ok &= conv[c] != 0;
            if (all_ok) return RL_OK;
            need_fp64 = diverged;
        }
        if (!need_fp64) {
            // GMRES-IR on each remaining column, within a budget of the estimated time of
            // the FP64 refactor it would otherwise save: the panel chain (~3.3 us per column
            // measured) plus 2/3 n^3 flops for LU, 1/3 n^3 for Cholesky, at the ~1 TFLOP/s
            // of the FP64 blocked factorisations. A first correction that grew
            // (kappa u_32 > 1) does not tell a system GMRES-IR converges on (kappa ~ 1e8)
            // from one it never will (kappa ~ 1e10); the GMRES residual does (gmres_ir).
            out.path = RL_PATH_GMRES;
            const double fp64_s =
                3.3e-6 * n + (kind == RL_KIND_LU ? 2.0 / 3.0 : 1.0 / 3.0) * (double)n * n * n / 1.0e12;
            const double deadline = host_seconds() + fp64_s;
            DevBuf<double> xb, bb;
            RL_TRY(xb.alloc(n, s));
            RL_TRY(bb.alloc(n, s));
            Minv M{F, n, kind, ipiv, dstatus.p + 1, {}, {}, {}};
            RL_TRY(M.init(s));
            for (int c = 0; c < nrhs && !need_fp64; c++) {
                if (conv[c]) continue;
                RL_TRY_CUDA(cudaMemcpy2DAsync(xb.p, sizeof(double), X + c, ldx * sizeof(double), sizeof(double), n,
                                              cudaMemcpyDeviceToDevice, s));
                RL_TRY_CUDA(cudaMemcpy2DAsync(bb.p, sizeof(double), B + c, ldb * sizeof(double), sizeof(double), n,
                                              cudaMemcpyDeviceToDevice, s));
                SolveOut o;
                bool ok = false;
                RL_TRY(gmres_ir(A, lda, n, M, bb.p, xb.p, anorm, bnorm[c], deadline, o, ok, s));
                int dst = 0;
                RL_TRY_CUDA(cudaMemcpyAsync(&dst, dstatus.p + 1, sizeof(int), cudaMemcpyDeviceToHost, s));
                RL_TRY_CUDA(cudaStreamSynchronize(s));
                if (!ok || dst) {
                    need_fp64 = true;
                    break;
                }
                RL_TRY_CUDA(cudaMemcpy2DAsync(X + c, ldx * sizeof(double), xb.p, sizeof(double), sizeof(double), n,
                                              cudaMemcpyDeviceToDevice, s));
                out.gmres += o.gmres;
                out.iters += o.iters;
            }
            if (!need_fp64) return backward_error_dev(A, lda, n, X, ldx, B, ldb, nrhs, out.berr, s);
        }
        const int it = out.iters, gm = out.gmres;
        RL_TRY(solve_with_fp64(B, ldb, X, ldx, nrhs, out, s));
        out.iters = it;
        out.gmres = gm;
        return RL_OK;
    }
};

// The mixed-precision solver for one call: factor, solve, release.
inline rl_status solve_mixed(const double *A, long long lda, int n, int kind, const double *B, long long ldb, double *X,
                             long long ldx, int nrhs, SolveOut &out, cudaStream_t s) {
    MixedFactor mf;
    RL_TRY(mf.factor(A, lda, n, kind, false, s));
    return mf.solve(B, ldb, X, ldx, nrhs, out, s);
}

// ----------------------------------------------------------------- least squares --
// min ||A x - b||_2 (m >= n, one right-hand side, device pointers) in FP64: Householder
// QR of [A | b], then R x = (Q^T b)[0:n] (HouseholderQr composition, qr.rs:250-275).
inline rl_status lstsq_fp64(const double *A, long long lda, int m, int n, const double *b, double *x, cudaStream_t s) {
    if (m < n) return RL_ERR_SHAPE;
    const long long ld = n + 1;
    DevBuf<double> Ab, tau;
    DevBuf<int> st;
    RL_TRY(Ab.alloc((size_t)m * ld, s));
    RL_TRY(tau.alloc(std::max(1, n), s));
    RL_TRY(st.alloc(1, s));
    RL_TRY_CUDA(cudaMemsetAsync(st.p, 0, sizeof(int), s));
    RL_TRY_CUDA(cudaMemcpy2DAsync(Ab.p, ld * sizeof(double), A, lda * sizeof(double), n * sizeof(double), m,
                                  cudaMemcpyDeviceToDevice, s));
    RL_TRY_CUDA(cudaMemcpy2DAsync(Ab.p + n, ld * sizeof(double), b, sizeof(double), sizeof(double), m,
                                  cudaMemcpyDeviceToDevice, s));
    RL_TRY(qr_factor_dev<double>(Ab.p, ld, m, (int)ld, n, tau.p, s));
    RL_TRY(tri_solve_dev<double>(Ab.p, ld, n, Ab.p + n, ld, 1, 2, st.p, s));
    RL_TRY(read_status<double>(st.p, s));
    RL_TRY_CUDA(cudaMemcpy2DAsync(x, sizeof(double), Ab.p + n, ld * sizeof(double), sizeof(double), n,
                                  cudaMemcpyDeviceToDevice, s));
    return RL_OK;
}

// g = A^T r for an m x n FP64 matrix (deterministic: fixed chunks, summed in order).
struct GemvT {
    double *partial;
    int chunks, rows_per;
    rl_status run(const double *A, long long lda, int m, int n, const double *r, double *g, cudaStream_t s) const {
        RL_LAUNCH(gemv_t_partial_kernel, dim3(ceil_div(n, 256), chunks), 256, 0, s, A, lda, m, n, r, rows_per, partial);
        RL_LAUNCH(reduce_chunks_kernel, std::min(4 * num_sms(), ceil_div(n, 256)), 256, 0, s, partial, chunks, n, g);
        return RL_OK;
    }
};

// Least squares in mixed precision: Householder QR of the FP32 copy of A gives R with
// R^T R ~ A^T A; the corrected semi-normal equations refine in FP64,
//   r = b - A x,  g = A^T r,  x += (R^T R)^-1 g   (R solves in FP32, g scaled),
// until the correction is below 4u ||x|| (converged to working precision), or stalls
// below 1e3 u ||x|| (the floor the FP64 residual leaves when b is far from range(A)).
// A correction that stalls higher, a pivot of R below FLT_MIN, or ten steps without
// convergence send the problem to FP64 QR instead. berr reports ||A^T r|| / (||A|| (||A|| ||x|| + ||b||)),
// inf-norms, for the returned x.
inline rl_status lstsq_mixed(const double *A, long long lda, int m, int n, const double *b, double *x, SolveOut &out,
                             cudaStream_t s) {
    NvtxRange nvtx_("rl.mixed.lstsq");
    out = SolveOut();
    if (m < n) return RL_ERR_SHAPE;
    if (n == 0) return RL_OK;
    DevBuf<float> Q32, L, tau32, w32;
    DevBuf<double> r, g, dx, partial;
    DevBuf<unsigned long long> bits;  // 0 anorm, 1 bnorm, 2 scale, 3 xn, 4 dxn, 5 gn
    DevBuf<int> dstatus, one;
    const int rows_per = 256, chunks = ceil_div(m, rows_per);
    RL_TRY(Q32.alloc((size_t)m * n, s));
    RL_TRY(L.alloc((size_t)n * n, s));
    RL_TRY(tau32.alloc(n, s));
    RL_TRY(w32.alloc(n, s));
    RL_TRY(r.alloc(m, s));
    RL_TRY(g.alloc(n, s));
    RL_TRY(dx.alloc(n, s));
    RL_TRY(partial.alloc((size_t)chunks * n, s));
    RL_TRY(bits.alloc(6, s));
    RL_TRY(dstatus.alloc(1, s));
    RL_TRY(one.alloc(1, s));
    RL_TRY_CUDA(cudaMemsetAsync(bits.p, 0, 6 * sizeof(unsigned long long), s));
    RL_TRY_CUDA(cudaMemsetAsync(dstatus.p, 0, sizeof(int), s));
    const int h_one = 1;
    RL_TRY_CUDA(cudaMemcpyAsync(one.p, &h_one, sizeof(int), cudaMemcpyHostToDevice, s));
    RL_LAUNCH(to_f32_rect_kernel, grid_rows(m, 8), 256, 0, s, A, lda, m, n, Q32.p, (long long)n, bits.p);
    RL_TRY(colnorm_dev(b, 1, m, 1, bits.p + 1, s));
    RL_TRY(qr_factor_dev<float>(Q32.p, n, m, n, n, tau32.p, s));
    RL_LAUNCH(upper_to_lower_t_kernel, (int)std::min<long long>(8 * num_sms(), ((long long)n * n + 255) / 256), 256, 0, s,
              Q32.p, (long long)n, n, L.p);
    Minv32 M{L.p, n, RL_KIND_CHOLESKY, nullptr, w32.p, bits.p + 2, one.p, dstatus.p};
    GemvT At{partial.p, chunks, rows_per};
    const int gv = std::min(4 * num_sms(), ceil_div(n, 256));
    // x0 = (R^T R)^-1 A^T b
    RL_TRY(At.run(A, lda, m, n, b, g.p, s));
    RL_TRY(M.apply(g.p, x, s));
    bool ok = false;
    double prev = INFINITY, anorm = 0.0, bnorm = 0.0, xn = 0.0;
    for (int it = 0; it < 10; it++) {
        RL_LAUNCH(resid_rect_kernel, grid_rows(m, 8), 256, 0, s, A, lda, m, n, x, b, r.p);
        RL_TRY(At.run(A, lda, m, n, r.p, g.p, s));
        RL_TRY(M.apply(g.p, dx.p, s));
        RL_LAUNCH(add_kernel, gv, 256, 0, s, x, dx.p, n);
        RL_TRY(colnorm_dev(x, 1, n, 1, bits.p + 3, s));
        RL_TRY(colnorm_dev(dx.p, 1, n, 1, bits.p + 4, s));
        unsigned long long hb[5];
        int dst = 0;
        RL_TRY_CUDA(cudaMemcpyAsync(hb, bits.p, sizeof hb, cudaMemcpyDeviceToHost, s));
        RL_TRY_CUDA(cudaMemcpyAsync(&dst, dstatus.p, sizeof(int), cudaMemcpyDeviceToHost, s));
        RL_TRY_CUDA(cudaStreamSynchronize(s));
        anorm = bits_to_double(hb[0]);
        bnorm = bits_to_double(hb[1]);
        xn = bits_to_double(hb[3]);
        const double dn = bits_to_double(hb[4]);
        out.iters = it + 1;
        if (dst != 0 || !std::isfinite(dn)) break;
        if (dn <= 4.0 * kU * xn) {
            ok = true;
            break;
        }
        if (it >= 1 && dn > 0.5 * prev) {
            // Stalled. With a large residual b - Ax the FP64 evaluation of A^T r leaves a
            // correction floor of about kappa^2 u ||x||: a floor this low is converged,
            // anything above it is left to FP64 QR.
            ok = dn <= 1e3 * kU * xn;
            break;
        }
        prev = dn;
    }
    if (!ok) {
        out.path = RL_PATH_FP64;
        RL_TRY(lstsq_fp64(A, lda, m, n, b, x, s));
        RL_TRY(colnorm_dev(x, 1, n, 1, bits.p + 3, s));
    }
    // reported quality: the normal-equations residual of the returned x
    RL_LAUNCH(resid_rect_kernel, grid_rows(m, 8), 256, 0, s, A, lda, m, n, x, b, r.p);
    RL_TRY(At.run(A, lda, m, n, r.p, g.p, s));
    RL_TRY(colnorm_dev(g.p, 1, n, 1, bits.p + 5, s));
    unsigned long long hb[6];
    RL_TRY_CUDA(cudaMemcpyAsync(hb, bits.p, sizeof hb, cudaMemcpyDeviceToHost, s));
    RL_TRY_CUDA(cudaStreamSynchronize(s));
    anorm = bits_to_double(hb[0]);
    bnorm = bits_to_double(hb[1]);
    xn = bits_to_double(hb[3]);
    const double den = anorm * (anorm * xn + bnorm);
    out.berr = den > 0 ? bits_to_double(hb[5]) / den : 0.0;
    return RL_OK;
}

}  // namespace rl
