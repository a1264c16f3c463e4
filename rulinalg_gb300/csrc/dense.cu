// Single-matrix entry points: GEMM, PartialPivLu, Cholesky, HouseholderQr and the
// Matrix::solve/inverse/det conveniences. Host-pointer calls copy the operands to the
// GPU (row stride preserved by 2D copies), run the kernels on the calling thread's
// default stream and copy the results back. Matrices with n <= 512 are factored by one
// CTA (factor_cta.cuh); larger ones by the blocked multi-CTA path (dense.cuh + GEMM).
#include <algorithm>
#include <type_traits>
#include <vector>

#include "dense_ops.cuh"
#include "gemm_tc.cuh"

namespace rl {

namespace {

// ------------------------------------------------------------- host entry points --

// The public GEMM: FP32 with at least one 128 x 128 tile's worth of C and K >= 256 runs
// on the tensor cores (3xTF32, FP32 accuracy); everything else, and all FP64, on the
// SIMT kernel; both split a long K when the product has few output tiles (gemm()).
template <class T>
rl_status gemm_public(int m, int n, int k, const T *a, long long lda, const T *b, long long ldb, T *c, long long ldc,
                      cudaStream_t s, bool &used_tc) {
    NvtxRange nvtx_("rl.gemm");
    used_tc = false;
    if constexpr (std::is_same<T, float>::value) used_tc = sgemm_tc_eligible(m, n, k);
    return gemm<T, false, false>(m, n, k, T(1), a, lda, b, ldb, T(0), c, ldc, s);
}

template <class T>
rl_status gemm_host(size_t m, size_t k, size_t n, const T *a, size_t rsa, const T *b, size_t rsb, T *c, size_t rsc) {
    if (m == 0 || n == 0) return RL_OK;
    if (!c || (k && (!a || !b))) return RL_ERR_INVALID_ARG;
    if (!fits_int(m) || !fits_int(n) || !fits_int(k)) return RL_ERR_INVALID_ARG;
    if ((m > 1 && rsa < k) || (k > 1 && rsb < n) || (m > 1 && rsc < n)) return RL_ERR_INVALID_ARG;
    RL_TRY(ensure_device());
    cudaStream_t s = cudaStreamPerThread;
    DevBuf<T> dA, dB, dC;
    RL_TRY(dA.alloc(m * k, s));
    RL_TRY(dB.alloc(k * n, s));
    RL_TRY(dC.alloc(m * n, s));
    RL_TRY(copy_h2d(dA.p, k, a, rsa, m, k, s));
    RL_TRY(copy_h2d(dB.p, n, b, rsb, k, n, s));
    bool used_tc = false;
    RL_TRY(gemm_public<T>((int)m, (int)n, (int)k, dA.p, (long long)k, dB.p, (long long)n, dC.p, (long long)n, s,
                          used_tc));
    RL_TRY(copy_d2h(c, rsc, dC.p, n, m, n, s));
    RL_TRY_CUDA(cudaStreamSynchronize(s));
    if (used_tc) RL_TRY(sgemm_tc_status(s));
    return RL_OK;
}

template <class T>
rl_status gemm_dev(size_t m, size_t k, size_t n, const T *a, size_t rsa, const T *b, size_t rsb, T *c, size_t rsc,
                   void *stream) {
    if (m == 0 || n == 0) return RL_OK;
    if (!c || (k && (!a || !b))) return RL_ERR_INVALID_ARG;
    if (!fits_int(m) || !fits_int(n) || !fits_int(k)) return RL_ERR_INVALID_ARG;
    RL_TRY(ensure_device());
    bool used_tc = false;
    return gemm_public<T>((int)m, (int)n, (int)k, a, (long long)rsa, b, (long long)rsb, c, (long long)rsc,
                          resolve_stream(stream), used_tc);
}

template <class T>
rl_status lu_decompose_host(size_t n, T *a, size_t lda, uint64_t *perm) {
    if (n == 0) return RL_OK;
    if (!a || !perm || lda < n || !fits_int(n)) return RL_ERR_INVALID_ARG;
    RL_TRY(ensure_device());
    cudaStream_t s = cudaStreamPerThread;
    DevBuf<T> dA;
    DevBuf<int> dpiv;
    DevBuf<uint64_t> dperm, scratch;
    RL_TRY(dA.alloc(n * n, s));
    RL_TRY(dpiv.alloc(n, s));
    RL_TRY(dperm.alloc(n, s));
    RL_TRY(scratch.alloc(n, s));
    RL_TRY(copy_h2d(dA.p, n, a, lda, n, n, s));
    rl_status st = lu_factor_dev<T>(dA.p, (long long)n, (int)n, dpiv.p, s);
    if (st == RL_OK) {
        RL_LAUNCH(ipiv_to_perm_kernel, 1, 32, 0, s, dpiv.p, (int)n, dperm.p, scratch.p);
        RL_TRY_CUDA(cudaMemcpyAsync(perm, dperm.p, n * sizeof(uint64_t), cudaMemcpyDeviceToHost, s));
    }
    RL_TRY(copy_d2h(a, lda, dA.p, n, n, n, s));
    RL_TRY_CUDA(cudaStreamSynchronize(s));
    return st;
}

template <class T>
rl_status lu_solve_host(size_t n, size_t nrhs, const T *lu, size_t lda, const uint64_t *perm, T *b, size_t ldb) {
    if (n == 0 || nrhs == 0) return RL_OK;
    if (!lu || !perm || !b || lda < n || (n > 1 && ldb < nrhs) || !fits_int(n) || !fits_int(nrhs))
        return RL_ERR_INVALID_ARG;
    RL_TRY(check_perm(n, perm));
    RL_TRY(ensure_device());
    cudaStream_t s = cudaStreamPerThread;
    DevBuf<T> dA, dB;
    DevBuf<uint64_t> dperm;
    RL_TRY(dA.alloc(n * n, s));
    RL_TRY(dB.alloc(n * nrhs, s));
    RL_TRY(dperm.alloc(n, s));
    RL_TRY(copy_h2d(dA.p, n, lu, lda, n, n, s));
    RL_TRY(copy_h2d(dB.p, nrhs, b, ldb, n, nrhs, s));
    RL_TRY_CUDA(cudaMemcpyAsync(dperm.p, perm, n * sizeof(uint64_t), cudaMemcpyHostToDevice, s));
    rl_status st = factor_solve_dev<T>(dA.p, (long long)n, (int)n, 0, dperm.p, dB.p, (long long)nrhs, (int)nrhs, s);
    if (st == RL_OK) RL_TRY(copy_d2h(b, ldb, dB.p, nrhs, n, nrhs, s));
    RL_TRY_CUDA(cudaStreamSynchronize(s));
    return st;
}

// inverse from factors: solve with the identity (n right-hand sides)
template <class T>
rl_status inverse_from_factors(const T *dF, int n, int kind, const uint64_t *dperm, T *inv, size_t ldi,
                               cudaStream_t s) {
    DevBuf<T> dX;
    RL_TRY(dX.alloc((size_t)n * n, s));
    const long long nn = (long long)n * n;
    RL_LAUNCH(eye_kernel<T>, (int)((nn + 255) / 256), 256, 0, s, dX.p, (long long)n, n, n);
    rl_status st = factor_solve_dev<T>(dF, n, n, kind, dperm, dX.p, n, n, s);
    if (st == RL_OK) RL_TRY(copy_d2h(inv, ldi, dX.p, (size_t)n, (size_t)n, (size_t)n, s));
    RL_TRY_CUDA(cudaStreamSynchronize(s));
    return st;
}

template <class T>
rl_status lu_inverse_host(size_t n, const T *lu, size_t lda, const uint64_t *perm, T *inv, size_t ldi) {
    if (n == 0) return RL_OK;
    if (!lu || !perm || !inv || lda < n || ldi < n || !fits_int(n)) return RL_ERR_INVALID_ARG;
    RL_TRY(check_perm(n, perm));
    RL_TRY(ensure_device());
    cudaStream_t s = cudaStreamPerThread;
    DevBuf<T> dA;
    DevBuf<uint64_t> dperm;
    RL_TRY(dA.alloc(n * n, s));
    RL_TRY(dperm.alloc(n, s));
    RL_TRY(copy_h2d(dA.p, n, lu, lda, n, n, s));
    RL_TRY_CUDA(cudaMemcpyAsync(dperm.p, perm, n * sizeof(uint64_t), cudaMemcpyHostToDevice, s));
    return inverse_from_factors<T>(dA.p, (int)n, 0, dperm.p, inv, ldi, s);
}

// det from the diagonal of a factor (copied alone) and, for LU, the permutation.
template <class T>
rl_status det_host(size_t n, const T *f, size_t lda, const uint64_t *perm, int square, T *det) {
    if (!det) return RL_ERR_INVALID_ARG;
    if (n == 0) {  // the determinant of an empty matrix is 1 (lu.rs:288-290, cholesky.rs:172-174)
        *det = T(1);
        return RL_OK;
    }
    if (!f || lda < n || !fits_int(n) || (!square && !perm)) return RL_ERR_INVALID_ARG;
    if (perm) RL_TRY(check_perm(n, perm));
    RL_TRY(ensure_device());
    cudaStream_t s = cudaStreamPerThread;
    DevBuf<T> dd, dout;
    DevBuf<uint64_t> dperm, scratch;
    RL_TRY(dd.alloc(n, s));
    RL_TRY(dout.alloc(1, s));
    RL_TRY(scratch.alloc(n, s));
    RL_TRY_CUDA(cudaMemcpy2DAsync(dd.p, sizeof(T), f, (lda + 1) * sizeof(T), sizeof(T), n, cudaMemcpyHostToDevice, s));
    if (perm) {
        RL_TRY(dperm.alloc(n, s));
        RL_TRY_CUDA(cudaMemcpyAsync(dperm.p, perm, n * sizeof(uint64_t), cudaMemcpyHostToDevice, s));
    }
    RL_LAUNCH(det_kernel<T>, 1, 32, 0, s, dd.p, 0LL, (int)n, perm ? dperm.p : nullptr, scratch.p, square, dout.p);
    RL_TRY_CUDA(cudaMemcpyAsync(det, dout.p, sizeof(T), cudaMemcpyDeviceToHost, s));
    RL_TRY_CUDA(cudaStreamSynchronize(s));
    return RL_OK;
}

template <class T>
rl_status chol_decompose_host(size_t n, T *a, size_t lda) {
    if (n == 0) return RL_OK;
    if (!a || lda < n || !fits_int(n)) return RL_ERR_INVALID_ARG;
    RL_TRY(ensure_device());
    cudaStream_t s = cudaStreamPerThread;
    DevBuf<T> dA;
    RL_TRY(dA.alloc(n * n, s));
    RL_TRY(copy_h2d(dA.p, n, a, lda, n, n, s));
    rl_status st = chol_factor_dev<T>(dA.p, (long long)n, (int)n, s);
    RL_TRY(copy_d2h(a, lda, dA.p, n, n, n, s));
    RL_TRY_CUDA(cudaStreamSynchronize(s));
    return st;
}

template <class T>
rl_status chol_solve_host(size_t n, size_t nrhs, const T *l, size_t ldl, T *b, size_t ldb) {
    if (n == 0 || nrhs == 0) return RL_OK;
    if (!l || !b || ldl < n || (n > 1 && ldb < nrhs) || !fits_int(n) || !fits_int(nrhs)) return RL_ERR_INVALID_ARG;
    RL_TRY(ensure_device());
    cudaStream_t s = cudaStreamPerThread;
    DevBuf<T> dA, dB;
    RL_TRY(dA.alloc(n * n, s));
    RL_TRY(dB.alloc(n * nrhs, s));
    RL_TRY(copy_h2d(dA.p, n, l, ldl, n, n, s));
    RL_TRY(copy_h2d(dB.p, nrhs, b, ldb, n, nrhs, s));
    rl_status st = factor_solve_dev<T>(dA.p, (long long)n, (int)n, 1, nullptr, dB.p, (long long)nrhs, (int)nrhs, s);
    if (st == RL_OK) RL_TRY(copy_d2h(b, ldb, dB.p, nrhs, n, nrhs, s));
    RL_TRY_CUDA(cudaStreamSynchronize(s));
    return st;
}

template <class T>
rl_status chol_inverse_host(size_t n, const T *l, size_t ldl, T *inv, size_t ldi) {
    if (n == 0) return RL_OK;
    if (!l || !inv || ldl < n || ldi < n || !fits_int(n)) return RL_ERR_INVALID_ARG;
    RL_TRY(ensure_device());
    cudaStream_t s = cudaStreamPerThread;
    DevBuf<T> dA;
    RL_TRY(dA.alloc(n * n, s));
    RL_TRY(copy_h2d(dA.p, n, l, ldl, n, n, s));
    return inverse_from_factors<T>(dA.p, (int)n, 1, nullptr, inv, ldi, s);
}

template <class T>
rl_status qr_decompose_host(size_t m, size_t n, T *a, size_t lda, T *tau) {
    const size_t p = std::min(m, n);
    if (m == 0 || n == 0) return RL_OK;
    if (!a || !tau || lda < n || !fits_int(m) || !fits_int(n)) return RL_ERR_INVALID_ARG;
    RL_TRY(ensure_device());
    cudaStream_t s = cudaStreamPerThread;
    DevBuf<T> dA, dt;
    RL_TRY(dA.alloc(m * n, s));
    RL_TRY(dt.alloc(p, s));
    RL_TRY(copy_h2d(dA.p, n, a, lda, m, n, s));
    rl_status st = qr_factor_dev<T>(dA.p, (long long)n, (int)m, (int)n, (int)p, dt.p, s);
    if (st == RL_OK) {
        RL_TRY(copy_d2h(a, lda, dA.p, n, m, n, s));
        RL_TRY_CUDA(cudaMemcpyAsync(tau, dt.p, p * sizeof(T), cudaMemcpyDeviceToHost, s));
    }
    RL_TRY_CUDA(cudaStreamSynchronize(s));
    return st;
}

template <class T>
rl_status qr_first_k_host(size_t m, size_t n, const T *qr, size_t lda, const T *tau, size_t k, T *q, size_t ldq) {
    if (k > m) return RL_ERR_SHAPE;  // householder.rs:241-242
    if (m == 0 || k == 0) return RL_OK;
    const size_t p = std::min(m, n);
    if (!qr || !q || (p && !tau) || lda < n || ldq < k || !fits_int(m) || !fits_int(n)) return RL_ERR_INVALID_ARG;
    RL_TRY(ensure_device());
    cudaStream_t s = cudaStreamPerThread;
    DevBuf<T> dA, dt, dQ;
    RL_TRY(dA.alloc(std::max<size_t>(1, m * n), s));
    RL_TRY(dt.alloc(std::max<size_t>(1, p), s));
    RL_TRY(dQ.alloc(m * k, s));
    RL_TRY(copy_h2d(dA.p, n, qr, lda, m, n, s));
    if (p) RL_TRY_CUDA(cudaMemcpyAsync(dt.p, tau, p * sizeof(T), cudaMemcpyHostToDevice, s));
    RL_TRY(qr_first_k_dev<T>(dA.p, (long long)n, (int)m, (int)n, dt.p, (int)k, dQ.p, (long long)k, s));
    RL_TRY(copy_d2h(q, ldq, dQ.p, k, m, k, s));
    RL_TRY_CUDA(cudaStreamSynchronize(s));
    return RL_OK;
}

template <class T>
rl_status qr_apply_q_host(size_t m, size_t n, const T *qr, size_t lda, const T *tau, size_t q, T *x, size_t ldx,
                          bool trans) {
    if (m == 0 || q == 0) return RL_OK;
    const size_t p = std::min(m, n);
    if (!qr || !x || (p && !tau) || lda < n || ldx < q || !fits_int(m) || !fits_int(n) || !fits_int(q))
        return RL_ERR_INVALID_ARG;
    RL_TRY(ensure_device());
    cudaStream_t s = cudaStreamPerThread;
    DevBuf<T> dA, dt, dX;
    RL_TRY(dA.alloc(std::max<size_t>(1, m * n), s));
    RL_TRY(dt.alloc(std::max<size_t>(1, p), s));
    RL_TRY(dX.alloc(m * q, s));
    RL_TRY(copy_h2d(dA.p, n, qr, lda, m, n, s));
    if (p) RL_TRY_CUDA(cudaMemcpyAsync(dt.p, tau, p * sizeof(T), cudaMemcpyHostToDevice, s));
    RL_TRY(copy_h2d(dX.p, q, x, ldx, m, q, s));
    RL_TRY(qr_apply_q_dev<T>(dA.p, (long long)n, (int)m, (int)n, dt.p, (int)q, dX.p, (long long)q, trans, s));
    RL_TRY(copy_d2h(x, ldx, dX.p, q, m, q, s));
    RL_TRY_CUDA(cudaStreamSynchronize(s));
    return RL_OK;
}

// U X = B (upper = true, back_substitution) or L X = B (forward_substitution) for an
// n x n triangle (the other triangle's values are ignored) and n x nrhs B, overwritten
// by X.
template <class T>
rl_status trsv_host(size_t n, size_t nrhs, const T *t, size_t ldt, T *b, size_t ldb, bool upper) {
    if (n == 0 || nrhs == 0) return RL_OK;
    if (!t || !b || ldt < n || ldb < nrhs || !fits_int(n) || !fits_int(nrhs)) return RL_ERR_INVALID_ARG;
    RL_TRY(ensure_device());
    cudaStream_t s = cudaStreamPerThread;
    DevBuf<T> dT, dB;
    DevBuf<int> st;
    RL_TRY(dT.alloc(n * n, s));
    RL_TRY(dB.alloc(n * nrhs, s));
    RL_TRY(st.alloc(1, s));
    RL_TRY_CUDA(cudaMemsetAsync(st.p, 0, sizeof(int), s));
    RL_TRY(copy_h2d(dT.p, n, t, ldt, n, n, s));
    RL_TRY(copy_h2d(dB.p, nrhs, b, ldb, n, nrhs, s));
    RL_TRY(tri_solve_dev<T>(dT.p, (long long)n, (int)n, dB.p, (long long)nrhs, (int)nrhs, upper ? 2 : 1, st.p, s));
    const rl_status r = read_status<T>(st.p, s);
    if (r != RL_OK) return r;
    RL_TRY(copy_d2h(b, ldb, dB.p, nrhs, n, nrhs, s));
    RL_TRY_CUDA(cudaStreamSynchronize(s));
    return RL_OK;
}

template <class T>
rl_status qr_lstsq_host(size_t m, size_t n, T *a, size_t lda, const T *b, T *x) {
    if (m < n) return RL_ERR_SHAPE;
    if (n == 0) return RL_OK;
    if (!a || !b || !x || lda < n || !fits_int(m) || !fits_int(n + 1)) return RL_ERR_INVALID_ARG;
    RL_TRY(ensure_device());
    cudaStream_t s = cudaStreamPerThread;
    const size_t ld = n + 1;  // [A | b]
    DevBuf<T> dA, dt;
    DevBuf<int> st;
    RL_TRY(dA.alloc(m * ld, s));
    RL_TRY(dt.alloc(n, s));
    RL_TRY(st.alloc(1, s));
    RL_TRY_CUDA(cudaMemsetAsync(st.p, 0, sizeof(int), s));
    RL_TRY(copy_h2d(dA.p, ld, a, lda, m, n, s));
    RL_TRY_CUDA(cudaMemcpy2DAsync(dA.p + n, ld * sizeof(T), b, sizeof(T), sizeof(T), m, cudaMemcpyHostToDevice, s));
    RL_TRY(qr_factor_dev<T>(dA.p, (long long)ld, (int)m, (int)ld, (int)n, dt.p, s));
    // R1 x = (Q^T b)[0:n], the last column after the factorisation.
    RL_TRY(tri_solve_dev<T>(dA.p, (long long)ld, (int)n, dA.p + n, (long long)ld, 1, 2, st.p, s));
    rl_status r = read_status<T>(st.p, s);
    if (r == RL_OK)
        RL_TRY_CUDA(cudaMemcpy2DAsync(x, sizeof(T), dA.p + n, ld * sizeof(T), sizeof(T), n, cudaMemcpyDeviceToHost, s));
    RL_TRY(copy_d2h(a, lda, dA.p, ld, m, n, s));
    RL_TRY_CUDA(cudaStreamSynchronize(s));
    return r;
}

// Matrix::solve (impl_mat.rs:354-356): decompose + one solve, factors stay on the GPU.
template <class T>
rl_status matrix_solve_host(size_t n, T *a, size_t lda, T *b) {
    if (n == 0) return RL_OK;
    if (!a || !b || lda < n || !fits_int(n)) return RL_ERR_INVALID_ARG;
    RL_TRY(ensure_device());
    cudaStream_t s = cudaStreamPerThread;
    DevBuf<T> dA, dB;
    DevBuf<int> dpiv;
    DevBuf<uint64_t> dperm, scratch;
    RL_TRY(dA.alloc(n * n, s));
    RL_TRY(dB.alloc(n, s));
    RL_TRY(dpiv.alloc(n, s));
    RL_TRY(dperm.alloc(n, s));
    RL_TRY(scratch.alloc(n, s));
    RL_TRY(copy_h2d(dA.p, n, a, lda, n, n, s));
    RL_TRY_CUDA(cudaMemcpyAsync(dB.p, b, n * sizeof(T), cudaMemcpyHostToDevice, s));
    rl_status st = lu_factor_dev<T>(dA.p, (long long)n, (int)n, dpiv.p, s);
    if (st == RL_OK) {
        RL_LAUNCH(ipiv_to_perm_kernel, 1, 32, 0, s, dpiv.p, (int)n, dperm.p, scratch.p);
        st = factor_solve_dev<T>(dA.p, (long long)n, (int)n, 0, dperm.p, dB.p, 1, 1, s);
    }
    if (st == RL_OK) RL_TRY_CUDA(cudaMemcpyAsync(b, dB.p, n * sizeof(T), cudaMemcpyDeviceToHost, s));
    RL_TRY(copy_d2h(a, lda, dA.p, n, n, n, s));
    RL_TRY_CUDA(cudaStreamSynchronize(s));
    return st;
}

template <class T>
rl_status matrix_inverse_host(size_t n, T *a, size_t lda, T *inv, size_t ldi) {
    if (n == 0) return RL_OK;
    if (!a || !inv || lda < n || ldi < n || !fits_int(n)) return RL_ERR_INVALID_ARG;
    RL_TRY(ensure_device());
    cudaStream_t s = cudaStreamPerThread;
    DevBuf<T> dA;
    DevBuf<int> dpiv;
    DevBuf<uint64_t> dperm, scratch;
    RL_TRY(dA.alloc(n * n, s));
    RL_TRY(dpiv.alloc(n, s));
    RL_TRY(dperm.alloc(n, s));
    RL_TRY(scratch.alloc(n, s));
    RL_TRY(copy_h2d(dA.p, n, a, lda, n, n, s));
    rl_status st = lu_factor_dev<T>(dA.p, (long long)n, (int)n, dpiv.p, s);
    if (st != RL_OK) {
        RL_TRY_CUDA(cudaStreamSynchronize(s));
        return st;
    }
    RL_LAUNCH(ipiv_to_perm_kernel, 1, 32, 0, s, dpiv.p, (int)n, dperm.p, scratch.p);
    return inverse_from_factors<T>(dA.p, (int)n, 0, dperm.p, inv, ldi, s);
}

// Matrix::det closed forms (impl_mat.rs:412-423) evaluated on the device, in the
// reference's operation order; flag[0] receives 1 when the matrix is diagonal.
template <class T>
__global__ void det_small_kernel(const T *A, int n, const int *isdiag, T *out) {
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
#define A_(i, j) A[(i) * n + (j)]
    if (*isdiag) {
        T d = T(1);
        for (int i = 0; i < n; i++) d = d * A_(i, i);
        out[0] = d;
    } else if (n == 2) {
        out[0] = (A_(0, 0) * A_(1, 1)) - (A_(0, 1) * A_(1, 0));
    } else if (n == 3) {
        out[0] = (A_(0, 0) * A_(1, 1) * A_(2, 2)) + (A_(0, 1) * A_(1, 2) * A_(2, 0)) + (A_(0, 2) * A_(1, 0) * A_(2, 1)) -
                 (A_(0, 0) * A_(1, 2) * A_(2, 1)) - (A_(0, 1) * A_(1, 0) * A_(2, 2)) - (A_(0, 2) * A_(1, 1) * A_(2, 0));
    }
#undef A_
}

template <class T>
__global__ void offdiag_kernel(const T *A, int n, int *notdiag) {
    const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= (long long)n * n) return;
    const int i = (int)(idx / n), j = (int)(idx - (long long)i * n);
    if (i != j && A[idx] != T(0)) atomicExch(notdiag, 1);
}

template <class T>
rl_status matrix_det_host(size_t n, T *a, size_t lda, T *det) {
    if (!det) return RL_ERR_INVALID_ARG;
    if (n == 0) {
        *det = T(1);
        return RL_OK;
    }
    if (!a || lda < n || !fits_int(n)) return RL_ERR_INVALID_ARG;
    RL_TRY(ensure_device());
    cudaStream_t s = cudaStreamPerThread;
    DevBuf<T> dA, dout;
    DevBuf<int> flag;
    RL_TRY(dA.alloc(n * n, s));
    RL_TRY(dout.alloc(1, s));
    RL_TRY(flag.alloc(2, s));
    RL_TRY_CUDA(cudaMemsetAsync(flag.p, 0, 2 * sizeof(int), s));
    RL_TRY(copy_h2d(dA.p, n, a, lda, n, n, s));
    const long long nn = (long long)n * n;
    RL_LAUNCH(offdiag_kernel<T>, (int)((nn + 255) / 256), 256, 0, s, dA.p, (int)n, flag.p);
    int notdiag = 0;
    RL_TRY_CUDA(cudaMemcpyAsync(&notdiag, flag.p, sizeof(int), cudaMemcpyDeviceToHost, s));
    RL_TRY_CUDA(cudaStreamSynchronize(s));
    if (!notdiag || n == 2 || n == 3) {
        int one = notdiag ? 0 : 1;
        RL_TRY_CUDA(cudaMemcpyAsync(flag.p + 1, &one, sizeof(int), cudaMemcpyHostToDevice, s));
        RL_LAUNCH(det_small_kernel<T>, 1, 32, 0, s, dA.p, (int)n, flag.p + 1, dout.p);
        RL_TRY_CUDA(cudaMemcpyAsync(det, dout.p, sizeof(T), cudaMemcpyDeviceToHost, s));
        RL_TRY_CUDA(cudaStreamSynchronize(s));
        return RL_OK;
    }
    DevBuf<int> dpiv;
    DevBuf<uint64_t> dperm, scratch;
    RL_TRY(dpiv.alloc(n, s));
    RL_TRY(dperm.alloc(n, s));
    RL_TRY(scratch.alloc(n, s));
    rl_status st = lu_factor_dev<T>(dA.p, (long long)n, (int)n, dpiv.p, s);
    if (st == RL_ERR_DIV_BY_ZERO) {  // a decomposition failure maps to 0 (impl_mat.rs:424-426)
        *det = T(0);
        RL_TRY_CUDA(cudaStreamSynchronize(s));
        return RL_OK;
    }
    RL_TRY(st);
    RL_LAUNCH(ipiv_to_perm_kernel, 1, 32, 0, s, dpiv.p, (int)n, dperm.p, scratch.p);
    RL_LAUNCH(det_kernel<T>, 1, 32, 0, s, dA.p, (long long)n, (int)n, dperm.p, scratch.p, 0, dout.p);
    RL_TRY_CUDA(cudaMemcpyAsync(det, dout.p, sizeof(T), cudaMemcpyDeviceToHost, s));
    RL_TRY_CUDA(cudaStreamSynchronize(s));
    return RL_OK;
}

}  // namespace
}  // namespace rl

using namespace rl;

extern "C" {

rl_status rl_sgemm(size_t m, size_t k, size_t n, const float *a, size_t rsa, const float *b, size_t rsb, float *c,
                   size_t rsc) {
    return gemm_host<float>(m, k, n, a, rsa, b, rsb, c, rsc);
}
rl_status rl_dgemm(size_t m, size_t k, size_t n, const double *a, size_t rsa, const double *b, size_t rsb, double *c,
                   size_t rsc) {
    return gemm_host<double>(m, k, n, a, rsa, b, rsb, c, rsc);
}
rl_status rl_sgemm_dev(size_t m, size_t k, size_t n, const float *a, size_t rsa, const float *b, size_t rsb, float *c,
                       size_t rsc, void *stream) {
    return gemm_dev<float>(m, k, n, a, rsa, b, rsb, c, rsc, stream);
}
rl_status rl_dgemm_dev(size_t m, size_t k, size_t n, const double *a, size_t rsa, const double *b, size_t rsb,
                       double *c, size_t rsc, void *stream) {
    return gemm_dev<double>(m, k, n, a, rsa, b, rsb, c, rsc, stream);
}

rl_status rl_slu_decompose(size_t n, float *a, size_t lda, uint64_t *perm) { return lu_decompose_host<float>(n, a, lda, perm); }
rl_status rl_dlu_decompose(size_t n, double *a, size_t lda, uint64_t *perm) { return lu_decompose_host<double>(n, a, lda, perm); }
rl_status rl_slu_solve(size_t n, size_t nrhs, const float *lu, size_t lda, const uint64_t *perm, float *b, size_t ldb) {
    return lu_solve_host<float>(n, nrhs, lu, lda, perm, b, ldb);
}
rl_status rl_dlu_solve(size_t n, size_t nrhs, const double *lu, size_t lda, const uint64_t *perm, double *b, size_t ldb) {
    return lu_solve_host<double>(n, nrhs, lu, lda, perm, b, ldb);
}
rl_status rl_slu_inverse(size_t n, const float *lu, size_t lda, const uint64_t *perm, float *inv, size_t ldi) {
    return lu_inverse_host<float>(n, lu, lda, perm, inv, ldi);
}
rl_status rl_dlu_inverse(size_t n, const double *lu, size_t lda, const uint64_t *perm, double *inv, size_t ldi) {
    return lu_inverse_host<double>(n, lu, lda, perm, inv, ldi);
}
rl_status rl_slu_det(size_t n, const float *lu, size_t lda, const uint64_t *perm, float *det) {
    return det_host<float>(n, lu, lda, perm, 0, det);
}
rl_status rl_dlu_det(size_t n, const double *lu, size_t lda, const uint64_t *perm, double *det) {
    return det_host<double>(n, lu, lda, perm, 0, det);
}

rl_status rl_scholesky_decompose(size_t n, float *a, size_t lda) { return chol_decompose_host<float>(n, a, lda); }
rl_status rl_dcholesky_decompose(size_t n, double *a, size_t lda) { return chol_decompose_host<double>(n, a, lda); }
rl_status rl_scholesky_solve(size_t n, size_t nrhs, const float *l, size_t ldl, float *b, size_t ldb) {
    return chol_solve_host<float>(n, nrhs, l, ldl, b, ldb);
}
rl_status rl_dcholesky_solve(size_t n, size_t nrhs, const double *l, size_t ldl, double *b, size_t ldb) {
    return chol_solve_host<double>(n, nrhs, l, ldl, b, ldb);
}
rl_status rl_scholesky_inverse(size_t n, const float *l, size_t ldl, float *inv, size_t ldi) {
    return chol_inverse_host<float>(n, l, ldl, inv, ldi);
}
rl_status rl_dcholesky_inverse(size_t n, const double *l, size_t ldl, double *inv, size_t ldi) {
    return chol_inverse_host<double>(n, l, ldl, inv, ldi);
}
rl_status rl_scholesky_det(size_t n, const float *l, size_t ldl, float *det) {
    return det_host<float>(n, l, ldl, nullptr, 1, det);
}
rl_status rl_dcholesky_det(size_t n, const double *l, size_t ldl, double *det) {
    return det_host<double>(n, l, ldl, nullptr, 1, det);
}

rl_status rl_sqr_decompose(size_t m, size_t n, float *a, size_t lda, float *tau) {
    return qr_decompose_host<float>(m, n, a, lda, tau);
}
rl_status rl_dqr_decompose(size_t m, size_t n, double *a, size_t lda, double *tau) {
    return qr_decompose_host<double>(m, n, a, lda, tau);
}
rl_status rl_sqr_first_k_columns(size_t m, size_t n, const float *qr, size_t lda, const float *tau, size_t k, float *q,
                                 size_t ldq) {
    return qr_first_k_host<float>(m, n, qr, lda, tau, k, q, ldq);
}
rl_status rl_dqr_first_k_columns(size_t m, size_t n, const double *qr, size_t lda, const double *tau, size_t k,
                                 double *q, size_t ldq) {
    return qr_first_k_host<double>(m, n, qr, lda, tau, k, q, ldq);
}
rl_status rl_sqr_q_apply(size_t m, size_t n, const float *qr, size_t lda, const float *tau, size_t q, float *x,
                         size_t ldx) {
    return qr_apply_q_host<float>(m, n, qr, lda, tau, q, x, ldx, false);
}
rl_status rl_dqr_q_apply(size_t m, size_t n, const double *qr, size_t lda, const double *tau, size_t q, double *x,
                         size_t ldx) {
    return qr_apply_q_host<double>(m, n, qr, lda, tau, q, x, ldx, false);
}
rl_status rl_sqr_q_apply_t(size_t m, size_t n, const float *qr, size_t lda, const float *tau, size_t q, float *x,
                           size_t ldx) {
    return qr_apply_q_host<float>(m, n, qr, lda, tau, q, x, ldx, true);
}
rl_status rl_dqr_q_apply_t(size_t m, size_t n, const double *qr, size_t lda, const double *tau, size_t q, double *x,
                           size_t ldx) {
    return qr_apply_q_host<double>(m, n, qr, lda, tau, q, x, ldx, true);
}
rl_status rl_strsv_upper(size_t n, size_t nrhs, const float *u, size_t ldu, float *b, size_t ldb) {
    return trsv_host<float>(n, nrhs, u, ldu, b, ldb, true);
}
rl_status rl_dtrsv_upper(size_t n, size_t nrhs, const double *u, size_t ldu, double *b, size_t ldb) {
    return trsv_host<double>(n, nrhs, u, ldu, b, ldb, true);
}
rl_status rl_strsv_lower(size_t n, size_t nrhs, const float *l, size_t ldl, float *b, size_t ldb) {
    return trsv_host<float>(n, nrhs, l, ldl, b, ldb, false);
}
rl_status rl_dtrsv_lower(size_t n, size_t nrhs, const double *l, size_t ldl, double *b, size_t ldb) {
    return trsv_host<double>(n, nrhs, l, ldl, b, ldb, false);
}
rl_status rl_sqr_least_squares(size_t m, size_t n, float *a, size_t lda, const float *b, float *x) {
    return qr_lstsq_host<float>(m, n, a, lda, b, x);
}
rl_status rl_dqr_least_squares(size_t m, size_t n, double *a, size_t lda, const double *b, double *x) {
    return qr_lstsq_host<double>(m, n, a, lda, b, x);
}

rl_status rl_smatrix_solve(size_t n, float *a, size_t lda, float *b) { return matrix_solve_host<float>(n, a, lda, b); }
rl_status rl_dmatrix_solve(size_t n, double *a, size_t lda, double *b) { return matrix_solve_host<double>(n, a, lda, b); }
rl_status rl_smatrix_inverse(size_t n, float *a, size_t lda, float *inv, size_t ldi) {
    return matrix_inverse_host<float>(n, a, lda, inv, ldi);
}
rl_status rl_dmatrix_inverse(size_t n, double *a, size_t lda, double *inv, size_t ldi) {
    return matrix_inverse_host<double>(n, a, lda, inv, ldi);
}
rl_status rl_smatrix_det(size_t n, float *a, size_t lda, float *det) { return matrix_det_host<float>(n, a, lda, det); }
rl_status rl_dmatrix_det(size_t n, double *a, size_t lda, double *det) { return matrix_det_host<double>(n, a, lda, det); }

}  // extern "C"
