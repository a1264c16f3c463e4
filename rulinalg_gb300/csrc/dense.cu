// Single-matrix entry points: GEMM, PartialPivLu, Cholesky, HouseholderQr and the
// Matrix::solve/inverse/det conveniences. Host-pointer calls copy the operands to the
// GPU (row stride preserved by 2D copies), run the kernels on the calling thread's
// default stream and copy the results back. Matrices with n <= 512 are factored by one
// CTA (factor_cta.cuh); larger ones by the blocked multi-CTA path (dense.cuh + GEMM).
#include <algorithm>
#include <type_traits>
#include <vector>

#include "batch.cuh"
#include "dense.cuh"
#include "gemm.cuh"

namespace rl {

namespace {

template <class T>
rl_status read_status(const int *dstatus, cudaStream_t s) {
    int h = 0;
    RL_TRY_CUDA(cudaMemcpyAsync(&h, dstatus, sizeof(int), cudaMemcpyDeviceToHost, s));
    RL_TRY_CUDA(cudaStreamSynchronize(s));
    return h;
}

template <class K>
rl_status set_smem(K kern, size_t bytes) {
    static_assert(std::is_pointer<K>::value, "kernel pointer");
    if (bytes > 48 * 1024)
        RL_TRY_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes));
    return RL_OK;
}

// One CTA factors a matrix with n <= CTA_NMAX; kind 0 LU (ipiv out), 1 Cholesky.
template <class T>
rl_status factor_small(T *A, long long lda, int n, int kind, int *ipiv, cudaStream_t s) {
    DevBuf<int> st;
    RL_TRY(st.alloc(1, s));
    RL_TRY_CUDA(cudaMemsetAsync(st.p, 0, sizeof(int), s));
    const size_t smem = cta_smem_bytes<T>();
    RL_TRY(set_smem(factor_one_kernel<T>, smem));
    RL_LAUNCH(factor_one_kernel<T>, 1, CTA_THREADS, smem, s, A, (int)lda, n, kind, ipiv, st.p, Eps<T>::value);
    return read_status<T>(st.p, s);
}

// Cooperative panel geometry: G CTAs of rows_per rows each.
template <class T>
void panel_geometry(int mrows, int &G, int &rows_per) {
    const int target = std::is_same<T, double>::value ? 64 : 128;
    G = std::max(1, std::min(num_sms(), (mrows + target - 1) / target));
    rows_per = (mrows + G - 1) / G;
}

template <class T>
rl_status launch_coop(void *kern, int G, size_t smem, void **args, cudaStream_t s) {
    RL_TRY_CUDA(cudaLaunchCooperativeKernel(kern, dim3(G), dim3(256), args, smem, s));
    count_launch();
    return RL_OK;
}

// Blocked right-looking LU for any n: cooperative panel, row swaps, U12 solve, GEMM.
template <class T>
rl_status lu_factor_dev(T *A, long long lda, int n, int *ipiv, cudaStream_t s) {
    if (n <= 0) return RL_OK;
    if (n <= CTA_NMAX) return factor_small<T>(A, lda, n, 0, ipiv, s);
    constexpr int NB = PanelNB<T>::value;
    int Gmax, rp;
    panel_geometry<T>(n, Gmax, rp);
    if ((size_t)rp * (NB + 1) * sizeof(T) > 200 * 1024) return RL_ERR_INVALID_ARG;  // n beyond ~50k
    DevBuf<T> cand, rowj;
    DevBuf<PanelSync> sync;
    RL_TRY(cand.alloc((size_t)2 * Gmax * (2 + NB), s));
    RL_TRY(rowj.alloc(2 * NB, s));
    RL_TRY(sync.alloc(1, s));
    auto pk = lu_panel_kernel<T>;
    RL_TRY(set_smem(pk, 200 * 1024));
    const size_t tsm = sizeof(T) * (64 * 65 + 64 * 64);
    RL_TRY(set_smem(trsm_diag_kernel<T>, tsm));
    T tiny = Eps<T>::value;
    for (int k0 = 0; k0 < n; k0 += NB) {
        const int kb = std::min(NB, n - k0), mrows = n - k0;
        int G, rows_per;
        panel_geometry<T>(mrows, G, rows_per);
        const size_t smem = ((size_t)rows_per * (NB + 1) + NB) * sizeof(T);
        RL_TRY_CUDA(cudaMemsetAsync(sync.p, 0, sizeof(PanelSync), s));
        T *P = A + (long long)k0 * lda + k0;
        int *ip = ipiv + k0;
        void *args[] = {&P, &lda, (void *)&mrows, (void *)&kb, &k0, &rows_per, &ip, &cand.p, &rowj.p, &sync.p, &tiny};
        RL_TRY(launch_coop<T>((void *)pk, G, smem, args, s));
        int err = 0;
        RL_TRY_CUDA(cudaMemcpyAsync(&err, &sync.p->err, sizeof(int), cudaMemcpyDeviceToHost, s));
        RL_TRY_CUDA(cudaStreamSynchronize(s));
        if (err) return err;
        const int nother = n - kb;
        if (nother > 0)
            RL_LAUNCH(laswp_kernel<T>, ceil_div(nother, 256), 256, 0, s, A, lda, n, k0, k0 + kb, ipiv, k0, k0 + kb);
        const int n2 = n - k0 - kb;
        if (n2 > 0) {
            DevBuf<int> st;
            RL_TRY(st.alloc(1, s));
            RL_TRY_CUDA(cudaMemsetAsync(st.p, 0, sizeof(int), s));
            RL_LAUNCH(trsm_diag_kernel<T>, ceil_div(n2, 64), 64, tsm, s, P, lda, kb, P + kb, lda, n2, 0, st.p, tiny);
            RL_TRY((gemm<T, false, false>(n2, n2, kb, T(-1), P + (long long)kb * lda, lda, P + kb, lda, T(1),
                                         P + (long long)kb * lda + kb, lda, s)));
        }
    }
    return RL_OK;
}

// Blocked right-looking Cholesky: diagonal block by one CTA, L21 = A21 L11^-T, SYRK.
template <class T>
rl_status chol_factor_dev(T *A, long long lda, int n, cudaStream_t s) {
    if (n <= 0) return RL_OK;
    if (n <= CTA_NMAX) return factor_small<T>(A, lda, n, 1, nullptr, s);
    constexpr int NB = PanelNB<T>::value;
    for (int k0 = 0; k0 < n; k0 += NB) {
        const int kb = std::min(NB, n - k0), mrows = n - k0;
        T *P = A + (long long)k0 * lda + k0;
        RL_TRY(factor_small<T>(P, lda, kb, 1, nullptr, s));
        const int m2 = mrows - kb;
        if (m2 > 0) {
            RL_LAUNCH(trsm_right_lt_kernel<T>, ceil_div(m2, 128), 128, 0, s, P, lda, kb, P + (long long)kb * lda, lda,
                      m2);
            T *L21 = P + (long long)kb * lda;
            RL_TRY((gemm<T, false, true, true>(m2, m2, kb, T(-1), L21, lda, L21, lda, T(1), L21 + kb, lda, s)));
        }
    }
    return RL_OK;
}

// Blocked Householder QR with compact-WY trailing updates; nrefl reflectors
// (min(m, n) for a plain QR; n for the augmented least-squares matrix).
template <class T>
rl_status qr_factor_dev(T *A, long long lda, int m, int n, int nrefl, T *tau, cudaStream_t s) {
    if (nrefl <= 0) return RL_OK;
    constexpr int NB = PanelNB<T>::value;
    int Gmax, rp;
    panel_geometry<T>(m, Gmax, rp);
    if ((size_t)rp * (NB + 1) * sizeof(T) > 200 * 1024) return RL_ERR_INVALID_ARG;
    DevBuf<T> part, x0buf, V, Gm, Tm, W1, W2;
    DevBuf<PanelSync> sync;
    RL_TRY(part.alloc((size_t)2 * Gmax * (1 + NB), s));
    RL_TRY(x0buf.alloc(2, s));
    RL_TRY(sync.alloc(1, s));
    RL_TRY(V.alloc((size_t)m * NB, s));
    RL_TRY(Gm.alloc(NB * NB, s));
    RL_TRY(Tm.alloc(NB * NB, s));
    RL_TRY(W1.alloc((size_t)NB * std::max(1, n), s));
    RL_TRY(W2.alloc((size_t)NB * std::max(1, n), s));
    auto pk = qr_panel_kernel<T>;
    RL_TRY(set_smem(pk, 200 * 1024));
    for (int k0 = 0; k0 < nrefl; k0 += NB) {
        const int kb = std::min(NB, nrefl - k0), mrows = m - k0;
        int G, rows_per;
        panel_geometry<T>(mrows, G, rows_per);
        const size_t smem = ((size_t)rows_per * (NB + 1) + NB) * sizeof(T);
        RL_TRY_CUDA(cudaMemsetAsync(sync.p, 0, sizeof(PanelSync), s));
        T *P = A + (long long)k0 * lda + k0;
        T *tk = tau + k0;
        void *args[] = {&P, &lda, (void *)&mrows, (void *)&kb, &rows_per, &tk, &part.p, &x0buf.p, &sync.p};
        RL_TRY(launch_coop<T>((void *)pk, G, smem, args, s));
        int err = 0;
        RL_TRY_CUDA(cudaMemcpyAsync(&err, &sync.p->err, sizeof(int), cudaMemcpyDeviceToHost, s));
        RL_TRY_CUDA(cudaStreamSynchronize(s));
        if (err) return err;
        const int n2 = n - k0 - kb;
        if (n2 <= 0) continue;
        const long long mk = (long long)mrows * kb;
        RL_LAUNCH(extract_v_kernel<T>, (int)((mk + 255) / 256), 256, 0, s, P, lda, mrows, kb, V.p);
        RL_TRY((gemm<T, true, false>(kb, kb, mrows, T(1), V.p, kb, V.p, kb, T(0), Gm.p, kb, s)));
        RL_LAUNCH(larft_kernel<T>, 1, 64, 0, s, Gm.p, tk, kb, Tm.p);
        T *A2 = P + kb;
        RL_TRY((gemm<T, true, false>(kb, n2, mrows, T(1), V.p, kb, A2, lda, T(0), W1.p, n2, s)));
        RL_TRY((gemm<T, true, false>(kb, n2, kb, T(1), Tm.p, kb, W1.p, n2, T(0), W2.p, n2, s)));
        RL_TRY((gemm<T, false, false>(mrows, n2, kb, T(-1), V.p, kb, W2.p, n2, T(1), A2, lda, s)));
    }
    return RL_OK;
}

// Q[:, 0:k] of a compact QR (HouseholderComposition::first_k_columns): reflector panels
// applied in reverse order to I[:, 0:k], each as Q2 -= V (T (V^T Q2)).
template <class T>
rl_status qr_first_k_dev(const T *QR, long long lda, int m, int n, const T *tau, int k, T *Q, long long ldq,
                         cudaStream_t s) {
    if (m <= 0 || k <= 0) return RL_OK;
    constexpr int NB = PanelNB<T>::value;
    const long long mk = (long long)m * k;
    RL_LAUNCH(eye_kernel<T>, (int)((mk + 255) / 256), 256, 0, s, Q, ldq, m, k);
    const int jmax = std::min(std::min(m, n), k);
    if (jmax <= 0) return RL_OK;
    DevBuf<T> V, Gm, Tm, W1, W2;
    RL_TRY(V.alloc((size_t)m * NB, s));
    RL_TRY(Gm.alloc(NB * NB, s));
    RL_TRY(Tm.alloc(NB * NB, s));
    RL_TRY(W1.alloc((size_t)NB * k, s));
    RL_TRY(W2.alloc((size_t)NB * k, s));
    for (int k0 = ((jmax - 1) / NB) * NB; k0 >= 0; k0 -= NB) {
        const int kb = std::min(NB, jmax - k0), mrows = m - k0, nc = k - k0;
        const T *P = QR + (long long)k0 * lda + k0;
        const long long mkb = (long long)mrows * kb;
        RL_LAUNCH(extract_v_kernel<T>, (int)((mkb + 255) / 256), 256, 0, s, P, lda, mrows, kb, V.p);
        RL_TRY((gemm<T, true, false>(kb, kb, mrows, T(1), V.p, kb, V.p, kb, T(0), Gm.p, kb, s)));
        RL_LAUNCH(larft_kernel<T>, 1, 64, 0, s, Gm.p, tau + k0, kb, Tm.p);
        T *Q2 = Q + (long long)k0 * ldq + k0;
        RL_TRY((gemm<T, true, false>(kb, nc, mrows, T(1), V.p, kb, Q2, ldq, T(0), W1.p, nc, s)));
        RL_TRY((gemm<T, false, false>(kb, nc, kb, T(1), Tm.p, kb, W1.p, nc, T(0), W2.p, nc, s)));
        RL_TRY((gemm<T, false, false>(mrows, nc, kb, T(-1), V.p, kb, W2.p, nc, T(1), Q2, ldq, s)));
    }
    return RL_OK;
}

// Blocked triangular solve op(A) X = Y in place (A n x n, Y n x nrhs).
// mode 0: unit lower, 1: lower, 2: upper, 3: L^T with L lower. |d_ii| < eps is
// recorded as RL_ERR_DIV_BY_ZERO in *dstatus.
template <class T>
rl_status tri_solve_dev(const T *A, long long lda, int n, T *Y, long long ldy, int nrhs, int mode, int *dstatus,
                        cudaStream_t s) {
    if (n <= 0 || nrhs <= 0) return RL_OK;
    constexpr int NB = 64;
    const size_t tsm = sizeof(T) * (64 * 65 + 64 * 64);
    RL_TRY(set_smem(trsm_diag_kernel<T>, tsm));
    const T tiny = Eps<T>::value;
    const int gr = ceil_div(nrhs, 64);
    if (mode == 0 || mode == 1) {
        for (int b0 = 0; b0 < n; b0 += NB) {
            const int bs = std::min(NB, n - b0);
            const T *D = A + (long long)b0 * lda + b0;
            T *Yb = Y + (long long)b0 * ldy;
            RL_LAUNCH(trsm_diag_kernel<T>, gr, 64, tsm, s, D, lda, bs, Yb, ldy, nrhs, mode, dstatus, tiny);
            const int rest = n - b0 - bs;
            if (rest > 0)
                RL_TRY((gemm<T, false, false>(rest, nrhs, bs, T(-1), A + (long long)(b0 + bs) * lda + b0, lda, Yb, ldy,
                                              T(1), Yb + (long long)bs * ldy, ldy, s)));
        }
    } else {
        for (int b1 = n; b1 > 0; b1 -= NB) {
            const int b0 = std::max(0, b1 - NB), bs = b1 - b0;
            const T *D = A + (long long)b0 * lda + b0;
            T *Yb = Y + (long long)b0 * ldy;
            RL_LAUNCH(trsm_diag_kernel<T>, gr, 64, tsm, s, D, lda, bs, Yb, ldy, nrhs, mode, dstatus, tiny);
            if (b0 > 0) {
                if (mode == 2)
                    RL_TRY((gemm<T, false, false>(b0, nrhs, bs, T(-1), A + b0, lda, Yb, ldy, T(1), Y, ldy, s)));
                else
                    RL_TRY((gemm<T, true, false>(b0, nrhs, bs, T(-1), A + (long long)b0 * lda, lda, Yb, ldy, T(1), Y,
                                                 ldy, s)));
            }
        }
    }
    return RL_OK;
}

__global__ void ipiv_to_perm_kernel(const int *ipiv, int n, uint64_t *perm, uint64_t *scratch) {
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    for (int i = 0; i < n; i++) scratch[i] = i;
    for (int j = 0; j < n; j++) {
        const int p = ipiv[j];
        const uint64_t t = scratch[j];
        scratch[j] = scratch[p];
        scratch[p] = t;
    }
    for (int i = 0; i < n; i++) perm[scratch[i]] = i;  // the stored form is the inverse
}

// Solve with factors already on the device. kind 0 = LU (dperm: stored permutation),
// 1 = Cholesky. B (n x nrhs, stride ldb) is overwritten.
template <class T>
rl_status factor_solve_dev(const T *F, long long lda, int n, int kind, const uint64_t *dperm, T *B, long long ldb,
                           int nrhs, cudaStream_t s) {
    if (n <= 0 || nrhs <= 0) return RL_OK;
    DevBuf<int> st;
    RL_TRY(st.alloc(1, s));
    RL_TRY_CUDA(cudaMemsetAsync(st.p, 0, sizeof(int), s));
    if (n <= CTA_NMAX) {
        const size_t smem = cta_smem_bytes<T>();
        RL_TRY(set_smem(solve_one_kernel<T>, smem));
        RL_LAUNCH(solve_one_kernel<T>, nrhs, CTA_THREADS, smem, s, F, (int)lda, n, kind, kind ? nullptr : dperm, B, ldb,
                  st.p, Eps<T>::value);
        return read_status<T>(st.p, s);
    }
    if (kind == 1) {
        RL_TRY(tri_solve_dev<T>(F, lda, n, B, ldb, nrhs, 1, st.p, s));
        RL_TRY(tri_solve_dev<T>(F, lda, n, B, ldb, nrhs, 3, st.p, s));
        return read_status<T>(st.p, s);
    }
    DevBuf<T> Y;
    RL_TRY(Y.alloc((size_t)n * nrhs, s));
    const long long tot = (long long)n * nrhs;
    RL_LAUNCH(permute_rows_kernel<T>, (int)((tot + 255) / 256), 256, 0, s, B, ldb, Y.p, (long long)nrhs, n, nrhs,
              dperm);
    RL_TRY(tri_solve_dev<T>(F, lda, n, Y.p, nrhs, nrhs, 0, st.p, s));
    RL_TRY(tri_solve_dev<T>(F, lda, n, Y.p, nrhs, nrhs, 2, st.p, s));
    RL_TRY_CUDA(cudaMemcpy2DAsync(B, ldb * sizeof(T), Y.p, nrhs * sizeof(T), nrhs * sizeof(T), n,
                                  cudaMemcpyDeviceToDevice, s));
    return read_status<T>(st.p, s);
}

rl_status check_perm(size_t n, const uint64_t *perm) {
    std::vector<unsigned char> seen(n, 0);
    for (size_t i = 0; i < n; i++) {
        if (perm[i] >= n || seen[perm[i]]) return RL_ERR_INVALID_PERMUTATION;
        seen[perm[i]] = 1;
    }
    return RL_OK;
}

bool fits_int(size_t v) { return v <= (size_t)INT32_MAX; }

// ------------------------------------------------------------- host entry points --

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
    RL_TRY((gemm<T, false, false>((int)m, (int)n, (int)k, T(1), dA.p, (long long)k, dB.p, (long long)n, T(0), dC.p,
                                  (long long)n, s)));
    RL_TRY(copy_d2h(c, rsc, dC.p, n, m, n, s));
    RL_TRY_CUDA(cudaStreamSynchronize(s));
    return RL_OK;
}

template <class T>
rl_status gemm_dev(size_t m, size_t k, size_t n, const T *a, size_t rsa, const T *b, size_t rsb, T *c, size_t rsc,
                   void *stream) {
    if (m == 0 || n == 0) return RL_OK;
    if (!c || (k && (!a || !b))) return RL_ERR_INVALID_ARG;
    if (!fits_int(m) || !fits_int(n) || !fits_int(k)) return RL_ERR_INVALID_ARG;
    RL_TRY(ensure_device());
    return gemm<T, false, false>((int)m, (int)n, (int)k, T(1), a, (long long)rsa, b, (long long)rsb, T(0), c,
                                 (long long)rsc, resolve_stream(stream));
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
