// Device-side orchestration shared by the host entry points: blocked factorisations
// (LU, Cholesky, Householder QR), Q formation, triangular solves and factor solves on
// buffers already on the GPU. Every function launches on the given stream; the ones
// that return a numerical status synchronise to read it.
#pragma once

#include <algorithm>
#include <type_traits>
#include <vector>

#include "batch.cuh"
#include "dense.cuh"
#include "gemm.cuh"
#include "mixed.cuh"

namespace rl {


template <class T>
inline rl_status read_status(const int *dstatus, cudaStream_t s) {
    int h = 0;
    RL_TRY_CUDA(cudaMemcpyAsync(&h, dstatus, sizeof(int), cudaMemcpyDeviceToHost, s));
    RL_TRY_CUDA(cudaStreamSynchronize(s));
    return h;
}

template <class K>
inline rl_status set_smem(K kern, size_t bytes) {
    static_assert(std::is_pointer<K>::value, "kernel pointer");
    if (bytes > 48 * 1024)
        RL_TRY_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes));
    return RL_OK;
}

// One CTA factors a matrix with n <= CTA_NMAX; kind 0 LU (ipiv out), 1 Cholesky.
template <class T>
rl_status factor_small(T *A, long long lda, int n, int kind, int *ipiv, cudaStream_t s, T tiny = Eps<T>::value) {
    DevBuf<int> st;
    RL_TRY(st.alloc(1, s));
    RL_TRY_CUDA(cudaMemsetAsync(st.p, 0, sizeof(int), s));
    const size_t smem = cta_smem_bytes<T>();
    RL_TRY(set_smem(factor_one_kernel<T>, smem));
    RL_LAUNCH(factor_one_kernel<T>, 1, CTA_THREADS, smem, s, A, (int)lda, n, kind, ipiv, st.p, tiny);
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

// Largest thread-block cluster (16 or 8 CTAs, 0: none) on which `kern` can run with
// `smem` bytes of dynamic shared memory per CTA; sets the kernel's attributes.
template <class K>
int probe_cluster(K kern, size_t smem) {
    int found = 0;
    if (cudaFuncSetAttribute(kern, cudaFuncAttributeNonPortableClusterSizeAllowed, 1) == cudaSuccess &&
        cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) == cudaSuccess) {
        for (int c : {16, 8}) {
            cudaLaunchConfig_t cfg = {};
            cudaLaunchAttribute at[1];
            at[0].id = cudaLaunchAttributeClusterDimension;
            at[0].val.clusterDim.x = c;
            at[0].val.clusterDim.y = 1;
            at[0].val.clusterDim.z = 1;
            cfg.gridDim = dim3(c);
            cfg.blockDim = dim3(256);
            cfg.dynamicSmemBytes = smem;
            cfg.attrs = at;
            cfg.numAttrs = 1;
            int nclusters = 0;
            if (cudaOccupancyMaxActiveClusters(&nclusters, kern, &cfg) == cudaSuccess && nclusters >= 1) {
                found = c;
                break;
            }
        }
    }
    cudaGetLastError();  // a refused query is not an error of the factorisation
    return found;
}

// Cluster size and rows per CTA for a panel of mrows rows of row_bytes each plus `extra`
// bytes per CTA: about `target_rows` rows per CTA, clamped to [2, cmax] and to at least
// the CTAs that the shared memory needs; 0 when even cmax CTAs would need more than
// kClusterSmem bytes each. FP64 panels take 64 rows per CTA (their row updates run at
// the SM's FP64 rate, so every SM added shortens a column); FP32 panels take 256 (their
// updates are cheap: up to 16 CTAs measured the same), which leaves the SMs of a GPC to
// other streams' kernels where fewer will do.
template <class T>
constexpr int panel_target_rows() {
    return sizeof(T) == 8 ? 64 : 256;
}
constexpr size_t kClusterSmem = 224 * 1024;
inline int cluster_shape(int mrows, size_t row_bytes, size_t extra, int cmax, int target_rows, int &rows_per) {
    const int cmin = (int)(((size_t)mrows * row_bytes + (kClusterSmem - extra) - 1) / (kClusterSmem - extra));
    if (cmin > cmax || cmax == 0) return 0;
    int C = std::max(cmin, std::min(cmax, ceil_div(mrows, target_rows)));
    C = std::max(C, 2);
    rows_per = ceil_div(mrows, C);
    return C;
}

template <class K, class... Args>
rl_status launch_cluster(K kern, int C, size_t smem, cudaStream_t s, Args... args) {
    cudaLaunchConfig_t cfg = {};
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeClusterDimension;
    at[0].val.clusterDim.x = C;
    at[0].val.clusterDim.y = 1;
    at[0].val.clusterDim.z = 1;
    cfg.gridDim = dim3(C);
    cfg.blockDim = dim3(256);
    cfg.dynamicSmemBytes = smem;
    cfg.stream = s;
    cfg.attrs = at;
    cfg.numAttrs = 1;
    RL_TRY_CUDA(cudaLaunchKernelEx(&cfg, kern, args...));
    count_launch();
    return RL_OK;
}

// The LU panel on one cluster when it fits (launched = true), else nothing.
template <class T>
rl_status lu_panel_cluster(T *P, long long lda, int mrows, int kb, int k0, int *ipiv, int *err, T tiny, cudaStream_t s,
                           bool &launched) {
    constexpr int NB = PanelNB<T>::value;
    launched = false;
    // look-ahead form (RL_TUNE_PANEL_LOOKAHEAD): three table slots instead of two
    const bool la = tune(RL_TUNE_PANEL_LOOKAHEAD) != 0;
    auto kern = la ? lu_panel_cluster_la_kernel<T> : lu_panel_cluster_kernel<T>;
    static const int cmax_hw = probe_cluster(lu_panel_cluster_kernel<T>, kClusterSmem);
    static const int cmax_hw_la = probe_cluster(lu_panel_cluster_la_kernel<T>, kClusterSmem);
    const int cmax = std::min<int>(la ? cmax_hw_la : cmax_hw, (int)tune(RL_TUNE_PANEL_CLUSTER_MAX));
    const int slots = la ? 3 : 2;
    const size_t row_bytes = (NB + 1) * sizeof(T), extra = (slots * 16 * NB + slots * NB) * sizeof(T);
    int rows_per = 0;
    const int C = cluster_shape(mrows, row_bytes, extra, cmax, panel_target_rows<T>(), rows_per);
    if (C == 0) return RL_OK;
    int tpr = 1;  // threads per row: every thread busy when the CTA holds few rows
    while (tpr < 8 && rows_per * tpr * 2 <= 256) tpr *= 2;
    RL_TRY(launch_cluster(kern, C, (size_t)rows_per * row_bytes + extra, s, P, lda, mrows, kb, k0, rows_per, tpr, ipiv,
                          err, tiny));
    launched = true;
    return RL_OK;
}

// The Householder panel on one cluster when it fits (launched = true), else nothing.
template <class T>
rl_status qr_panel_cluster(T *P, long long lda, int mrows, int kb, T *tau, cudaStream_t s, bool &launched) {
    constexpr int NB = PanelNB<T>::value;
    launched = false;
    auto kern = qr_panel_cluster_kernel<T>;
    static const int cmax_hw = probe_cluster(kern, kClusterSmem);
    const int cmax = std::min<int>(cmax_hw, (int)tune(RL_TUNE_PANEL_CLUSTER_MAX));
    const size_t row_bytes = (NB + 2) * sizeof(T), extra = (NB + 16 * NB + 16 + 1) * sizeof(T);
    int rows_per = 0;
    const int C = cluster_shape(mrows, row_bytes, extra, cmax, panel_target_rows<T>(), rows_per);
    if (C == 0) return RL_OK;
    RL_TRY(launch_cluster(kern, C, (size_t)rows_per * row_bytes + extra, s, P, lda, mrows, kb, rows_per, tau));
    launched = true;
    return RL_OK;
}

// op(A) Y = Y' in place (triangular solve; modes and paths at the definition below).
template <class T, class TA = T>
rl_status tri_solve_dev(const TA *A, long long lda, int n, T *Y, long long ldy, int nrhs, int mode, int *dstatus,
                        cudaStream_t s, T tiny = Eps<T>::value);

// Outer block width of the blocked Cholesky. FP32 (the mixed-precision factor and
// Matrix<f32>): 256-column blocks, each factored with the 64-column panels confined to
// the block, then ONE trailing update of K = 256 on the tensor cores (tcgen05, 3xTF32;
// the K = 64 updates of the inner panels measured slower there and stay on the SIMT
// kernel). FP64: 0, one block spanning the matrix (every update is a K = 64 DFMA GEMM,
// already at the FP64 rate). The FP32 LU takes its width from RL_TUNE_LU_OUTER_NB.
template <class T>
constexpr int outer_nb() {
    return std::is_same<T, float>::value ? 256 : 0;
}

// Blocked right-looking LU for any n: panel (one cluster, or a cooperative grid for
// panels too tall for a cluster), row swaps, U12 solve, GEMM. Within an outer block the
// swaps, U12 solves and updates of each 64-column panel cover the block's columns only;
// the block's swaps reach the other columns afterwards (LAPACK's getrf order), then
// U12 = L11^-1 A12 and A22 -= L21 U12 with K = the block width. The pivots are those of
// partial pivoting over the whole column either way.
template <class T>
rl_status lu_factor_dev(T *A, long long lda, int n, int *ipiv, cudaStream_t s, T tiny = Eps<T>::value) {
    NvtxRange nvtx_("rl.lu.factor");
    if (n <= 0) return RL_OK;
    if (n <= CTA_NMAX) return factor_small<T>(A, lda, n, 0, ipiv, s, tiny);
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
    // The error word is sticky across panels (only the barrier counter is reset per
    // launch) and read once at the end: a failed panel leaves identity pivots, the work
    // after it runs on in-range indices, and every later panel stops at its first barrier.
    RL_TRY_CUDA(cudaMemsetAsync(sync.p, 0, sizeof(PanelSync), s));
    unsigned long long wns = wait_ns();
    int NBO = n;  // FP32: outer blocks of RL_TUNE_LU_OUTER_NB columns (a multiple of NB)
    if constexpr (std::is_same<T, float>::value) {
        // automatic: at n = 2048 / 4096 one level measured 9.4 / 20.5 ms against 10.5 / 24.2
        // with 256-column blocks; at 8192 / 16384 1024-column blocks 58.2 / 171 ms against
        // 59.1 / 179 with 512, 62.4 / 206 with 256 and 62.0 / 229 with one level (mixed
        // solves, nrhs 1)
        const long long v = tune(RL_TUNE_LU_OUTER_NB);
        const int w = v < 0 ? (n < 6144 ? 0 : 1024) : (int)(v / NB) * NB;
        if (w >= NB) NBO = w;
    }
    for (int K0 = 0; K0 < n; K0 += NBO) {
        const int K1 = std::min(n, K0 + NBO), KB = K1 - K0;
        for (int k0 = K0; k0 < K1; k0 += NB) {
            const int kb = std::min(NB, K1 - k0), mrows = n - k0;
            int G, rows_per;
            panel_geometry<T>(mrows, G, rows_per);
            const size_t smem = ((size_t)rows_per * (NB + 1) + NB) * sizeof(T);
            T *P = A + (long long)k0 * lda + k0;
            int *ip = ipiv + k0;
            bool clustered = false;
            RL_TRY(lu_panel_cluster<T>(P, lda, mrows, kb, k0, ip, &sync.p->err, tiny, s, clustered));
            if (!clustered) {
                if (k0 > 0) RL_TRY_CUDA(cudaMemsetAsync(&sync.p->ctr, 0, sizeof(unsigned), s));
                void *args[] = {&P,       &lda,   (void *)&mrows, (void *)&kb, &k0,  &rows_per,
                                &ip,      &cand.p, &rowj.p,       &sync.p,     &tiny, &wns};
                RL_TRY(launch_coop<T>((void *)pk, G, smem, args, s));
            }
            // the swaps in the block's other columns (every other column for one block)
            RL_TRY(laswp<T>(A + K0, lda, KB, k0 - K0, k0 - K0 + kb, ipiv, k0, k0 + kb, s));
            const int n2 = K1 - k0 - kb, m2 = mrows - kb;
            if (n2 > 0) {
                // mode 0 (unit lower triangle) has no pivot to check: no status word
                RL_LAUNCH(trsm_diag_kernel<T>, ceil_div(n2, kTrsmCols), 128, 0, s, P, lda, kb, P + kb, lda, n2, 0,
                          (int *)nullptr, tiny);
                RL_TRY((gemm<T, false, false>(m2, n2, kb, T(-1), P + (long long)kb * lda, lda, P + kb, lda, T(1),
                                             P + (long long)kb * lda + kb, lda, s)));
            }
        }
        if (K1 < n) {
            // the block's swaps in the columns left and right of it, then U12 and the
            // K = KB trailing update (tensor cores for FP32)
            RL_TRY(laswp<T>(A, lda, n, K0, K1, ipiv, K0, K1, s));
            const int N2 = n - K1;
            T *L11 = A + (long long)K0 * lda + K0;
            RL_TRY(tri_solve_dev<T>(L11, lda, KB, L11 + KB, lda, N2, 0, &sync.p->err, s, tiny));
            RL_TRY((gemm<T, false, false>(N2, N2, KB, T(-1), L11 + (long long)KB * lda, lda, L11 + KB, lda, T(1),
                                         L11 + (long long)KB * lda + KB, lda, s)));
        } else if (K0 > 0) {
            RL_TRY(laswp<T>(A, lda, K0, 0, 0, ipiv, K0, K1, s));  // the last block's swaps on the left
        }
    }
    int err = 0;
    RL_TRY_CUDA(cudaMemcpyAsync(&err, &sync.p->err, sizeof(int), cudaMemcpyDeviceToHost, s));
    RL_TRY_CUDA(cudaStreamSynchronize(s));
    return err;
}

// Blocked right-looking Cholesky: diagonal block by one CTA, L21 = A21 L11^-T, SYRK.
// FP32: 256-column blocks (outer_nb); L11^-1 comes from a triangular solve with the
// identity, L21 = A21 (L11^-1)^T and the lower-triangle SYRK A22 -= L21 L21^T (K = 256)
// run on the tensor cores. FP64: 64-column blocks, L21 by substitution, DFMA SYRK. The
// strict upper triangle is never written either way.
template <class T>
rl_status chol_factor_dev(T *A, long long lda, int n, cudaStream_t s, T tiny = Eps<T>::value) {
    NvtxRange nvtx_("rl.cholesky.factor");
    if (n <= 0) return RL_OK;
    if (n <= CTA_NMAX) return factor_small<T>(A, lda, n, 1, nullptr, s, tiny);
    if constexpr (outer_nb<T>() > 0) {
        constexpr int NBO = outer_nb<T>();
        DevBuf<T> Linv, T21;
        DevBuf<int> st;
        RL_TRY(Linv.alloc((size_t)NBO * NBO, s));
        RL_TRY(T21.alloc((size_t)(n - std::min(n, NBO)) * NBO, s));
        RL_TRY(st.alloc(1, s));
        RL_TRY_CUDA(cudaMemsetAsync(st.p, 0, sizeof(int), s));
        for (int K0 = 0; K0 < n; K0 += NBO) {
            const int KB = std::min(NBO, n - K0), m2 = n - K0 - KB;
            T *P = A + (long long)K0 * lda + K0;
            RL_TRY(factor_small<T>(P, lda, KB, 1, nullptr, s, tiny));
            if (m2 <= 0) continue;
            const long long kk = (long long)KB * KB;
            RL_LAUNCH(eye_kernel<T>, (int)((kk + 255) / 256), 256, 0, s, Linv.p, (long long)KB, KB, KB);
            RL_TRY(tri_solve_dev<T>(P, lda, KB, Linv.p, KB, KB, 1, st.p, s, tiny));
            T *A21 = P + (long long)KB * lda;
            RL_TRY((gemm<T, false, true>(m2, KB, KB, T(1), A21, lda, Linv.p, KB, T(0), T21.p, KB, s)));
            RL_TRY_CUDA(cudaMemcpy2DAsync(A21, lda * sizeof(T), T21.p, KB * sizeof(T), KB * sizeof(T), m2,
                                          cudaMemcpyDeviceToDevice, s));
            RL_TRY((gemm<T, false, true, true>(m2, m2, KB, T(-1), A21, lda, A21, lda, T(1), A21 + KB, lda, s)));
        }
        return read_status<T>(st.p, s);
    }
    constexpr int NB = PanelNB<T>::value;
    for (int k0 = 0; k0 < n; k0 += NB) {
        const int kb = std::min(NB, n - k0), mrows = n - k0;
        T *P = A + (long long)k0 * lda + k0;
        RL_TRY(factor_small<T>(P, lda, kb, 1, nullptr, s, tiny));
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

// Tm of a reflector block V (mrows x kb): partial Gram matrices, then the T recursion.
template <class T>
rl_status block_t_factor(const T *V, int mrows, int kb, const T *tau, T *part, int max_parts, T *Tm,
                         cudaStream_t s) {
    const int nparts = ceil_div(mrows, kGramRows);
    if (nparts > max_parts) return RL_ERR_INVALID_ARG;
    RL_LAUNCH(gram_partial_kernel<T>, nparts, 256, 0, s, V, mrows, kb, part);
    const size_t smem = 2 * 64 * 65 * sizeof(T);
    RL_TRY(set_smem(larft_kernel<T>, smem));
    RL_LAUNCH(larft_kernel<T>, 1, 256, smem, s, part, nparts, tau, kb, Tm);
    return RL_OK;
}

// Blocked Householder QR with compact-WY trailing updates; nrefl reflectors
// (min(m, n) for a plain QR; n for the augmented least-squares matrix).
template <class T>
rl_status qr_factor_dev(T *A, long long lda, int m, int n, int nrefl, T *tau, cudaStream_t s) {
    NvtxRange nvtx_("rl.qr.factor");
    if (nrefl <= 0) return RL_OK;
    constexpr int NB = PanelNB<T>::value;
    int Gmax, rp;
    panel_geometry<T>(m, Gmax, rp);
    if ((size_t)rp * (NB + 1) * sizeof(T) > 200 * 1024) return RL_ERR_INVALID_ARG;
    DevBuf<T> part, x0buf, V, Gp, Tm, W1, W2;
    DevBuf<PanelSync> sync;
    RL_TRY(part.alloc((size_t)2 * Gmax * (1 + NB), s));
    RL_TRY(x0buf.alloc(2, s));
    RL_TRY(sync.alloc(1, s));
    RL_TRY(V.alloc((size_t)m * NB, s));
    const int max_parts = ceil_div(m, kGramRows);
    RL_TRY(Gp.alloc((size_t)max_parts * 64 * 64, s));
    RL_TRY(Tm.alloc(NB * NB, s));
    RL_TRY(W1.alloc((size_t)NB * std::max(1, n), s));
    RL_TRY(W2.alloc((size_t)NB * std::max(1, n), s));
    auto pk = qr_panel_kernel<T>;
    RL_TRY(set_smem(pk, 200 * 1024));
    // Sticky error word, read once at the end (see lu_factor_dev).
    RL_TRY_CUDA(cudaMemsetAsync(sync.p, 0, sizeof(PanelSync), s));
    unsigned long long wns = wait_ns();
    for (int k0 = 0; k0 < nrefl; k0 += NB) {
        const int kb = std::min(NB, nrefl - k0), mrows = m - k0;
        int G, rows_per;
        panel_geometry<T>(mrows, G, rows_per);
        const size_t smem = ((size_t)rows_per * (NB + 1) + NB) * sizeof(T);
        T *P = A + (long long)k0 * lda + k0;
        T *tk = tau + k0;
        bool clustered = false;
        RL_TRY(qr_panel_cluster<T>(P, lda, mrows, kb, tk, s, clustered));
        if (!clustered) {
            if (k0 > 0) RL_TRY_CUDA(cudaMemsetAsync(&sync.p->ctr, 0, sizeof(unsigned), s));
            void *args[] = {&P, &lda, (void *)&mrows, (void *)&kb, &rows_per, &tk, &part.p, &x0buf.p, &sync.p, &wns};
            RL_TRY(launch_coop<T>((void *)pk, G, smem, args, s));
        }
        const int n2 = n - k0 - kb;
        if (n2 <= 0) continue;
        const long long mk = (long long)mrows * kb;
        RL_LAUNCH(extract_v_kernel<T>, (int)((mk + 255) / 256), 256, 0, s, P, lda, mrows, kb, V.p);
        RL_TRY(block_t_factor<T>(V.p, mrows, kb, tk, Gp.p, max_parts, Tm.p, s));
        T *A2 = P + kb;
        RL_TRY((gemm<T, true, false>(kb, n2, mrows, T(1), V.p, kb, A2, lda, T(0), W1.p, n2, s)));
        RL_TRY((gemm<T, true, false>(kb, n2, kb, T(1), Tm.p, kb, W1.p, n2, T(0), W2.p, n2, s)));
        RL_TRY((gemm<T, false, false>(mrows, n2, kb, T(-1), V.p, kb, W2.p, n2, T(1), A2, lda, s)));
    }
    int err = 0;
    RL_TRY_CUDA(cudaMemcpyAsync(&err, &sync.p->err, sizeof(int), cudaMemcpyDeviceToHost, s));
    RL_TRY_CUDA(cudaStreamSynchronize(s));
    return err;
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
    DevBuf<T> V, Gp, Tm, W1, W2;
    RL_TRY(V.alloc((size_t)m * NB, s));
    const int max_parts = ceil_div(m, kGramRows);
    RL_TRY(Gp.alloc((size_t)max_parts * 64 * 64, s));
    RL_TRY(Tm.alloc(NB * NB, s));
    RL_TRY(W1.alloc((size_t)NB * k, s));
    RL_TRY(W2.alloc((size_t)NB * k, s));
    for (int k0 = ((jmax - 1) / NB) * NB; k0 >= 0; k0 -= NB) {
        const int kb = std::min(NB, jmax - k0), mrows = m - k0, nc = k - k0;
        const T *P = QR + (long long)k0 * lda + k0;
        const long long mkb = (long long)mrows * kb;
        RL_LAUNCH(extract_v_kernel<T>, (int)((mkb + 255) / 256), 256, 0, s, P, lda, mrows, kb, V.p);
        RL_TRY(block_t_factor<T>(V.p, mrows, kb, tau + k0, Gp.p, max_parts, Tm.p, s));
        T *Q2 = Q + (long long)k0 * ldq + k0;
        RL_TRY((gemm<T, true, false>(kb, nc, mrows, T(1), V.p, kb, Q2, ldq, T(0), W1.p, nc, s)));
        RL_TRY((gemm<T, false, false>(kb, nc, kb, T(1), Tm.p, kb, W1.p, nc, T(0), W2.p, nc, s)));
        RL_TRY((gemm<T, false, false>(mrows, nc, kb, T(-1), V.p, kb, W2.p, nc, T(1), Q2, ldq, s)));
    }
    return RL_OK;
}

// X <- Q X (trans = false) or X <- Q^T X (trans = true) for the m x q matrix X (row
// stride ldx), Q = H_0 H_1 ... H_{p-1} from the compact QR (m x n, p = min(m, n)):
// HouseholderComposition::left_multiply_into (householder.rs:203-227) applies the
// reflectors from the last to the first, Q^T takes them from the first to the last.
// Per 64-reflector panel (compact WY, Q_i = I - V T V^T): X[k0:, :] -= V (op(T) (V^T X[k0:, :]))
// with op(T) = T for Q, T^T for Q^T.
template <class T>
rl_status qr_apply_q_dev(const T *QR, long long lda, int m, int n, const T *tau, int q, T *X, long long ldx, bool trans,
                         cudaStream_t s) {
    const int p = std::min(m, n);
    if (m <= 0 || q <= 0 || p <= 0) return RL_OK;
    constexpr int NB = PanelNB<T>::value;
    DevBuf<T> V, Gp, Tm, W1, W2;
    RL_TRY(V.alloc((size_t)m * NB, s));
    const int max_parts = ceil_div(m, kGramRows);
    RL_TRY(Gp.alloc((size_t)max_parts * 64 * 64, s));
    RL_TRY(Tm.alloc(NB * NB, s));
    RL_TRY(W1.alloc((size_t)NB * q, s));
    RL_TRY(W2.alloc((size_t)NB * q, s));
    const int last = ((p - 1) / NB) * NB;
    for (int i = 0; i <= last / NB; i++) {
        const int k0 = trans ? i * NB : last - i * NB;
        const int kb = std::min(NB, p - k0), mrows = m - k0;
        const T *P = QR + (long long)k0 * lda + k0;
        const long long mkb = (long long)mrows * kb;
        RL_LAUNCH(extract_v_kernel<T>, (int)((mkb + 255) / 256), 256, 0, s, P, lda, mrows, kb, V.p);
        RL_TRY(block_t_factor<T>(V.p, mrows, kb, tau + k0, Gp.p, max_parts, Tm.p, s));
        T *X2 = X + (long long)k0 * ldx;
        RL_TRY((gemm<T, true, false>(kb, q, mrows, T(1), V.p, kb, X2, ldx, T(0), W1.p, q, s)));
        if (trans)
            RL_TRY((gemm<T, true, false>(kb, q, kb, T(1), Tm.p, kb, W1.p, q, T(0), W2.p, q, s)));
        else
            RL_TRY((gemm<T, false, false>(kb, q, kb, T(1), Tm.p, kb, W1.p, q, T(0), W2.p, q, s)));
        RL_TRY((gemm<T, false, false>(mrows, q, kb, T(-1), V.p, kb, W2.p, q, T(1), X2, ldx, s)));
    }
    return RL_OK;
}

// Blocked triangular solve op(A) X = Y in place (A n x n, Y n x nrhs).
// mode 0: unit lower, 1: lower, 2: upper, 3: L^T with L lower. |d_ii| < eps is
// recorded as RL_ERR_DIV_BY_ZERO in *dstatus. A may be stored in a narrower type TA than
// the arithmetic type T for at most kSweepGroups x kSweepRhs right-hand sides (an FP32
// factor applied in FP64), kSweepRhs on a GPU shared with other workers.
template <class T, class TA>
rl_status tri_solve_dev(const TA *A, long long lda, int n, T *Y, long long ldy, int nrhs, int mode, int *dstatus,
                        cudaStream_t s, T tiny) {
    if (n <= 0 || nrhs <= 0) return RL_OK;
    constexpr int NB = 64;
    if (nrhs <= kSweepRhs && g_shared_gpu) {
        // Few right-hand sides on a shared GPU: per 64-row block a one-CTA diagonal solve
        // (warp per column) and a warp-per-row GEMV update, all short launches.
        const int wpb = 8, gridr = std::max(1, std::min(4 * num_sms(), ceil_div(n, wpb)));
        if (mode == 0 || mode == 1) {
            for (int b0 = 0; b0 < n; b0 += NB) {
                const int bs = std::min(NB, n - b0), rest = n - b0 - bs;
                T *Yb = Y + (long long)b0 * ldy;
                RL_LAUNCH((trsv_diag_kernel<T, TA>), 1, 256, 0, s, A + (long long)b0 * lda + b0, lda, bs, Yb, ldy, nrhs, mode,
                          dstatus, tiny);
                if (rest > 0)
                    RL_LAUNCH((gemv_update_kernel<T, TA>), std::min(gridr, ceil_div(rest, wpb)), 32 * wpb, 0, s,
                              A + (long long)(b0 + bs) * lda + b0, lda, rest, bs, Yb, ldy, Yb + (long long)bs * ldy,
                              nrhs, false);
            }
        } else {
            for (int b1 = n; b1 > 0; b1 -= NB) {
                const int b0 = std::max(0, b1 - NB), bs = b1 - b0;
                T *Yb = Y + (long long)b0 * ldy;
                RL_LAUNCH((trsv_diag_kernel<T, TA>), 1, 256, 0, s, A + (long long)b0 * lda + b0, lda, bs, Yb, ldy, nrhs, mode,
                          dstatus, tiny);
                if (b0 > 0) {
                    if (mode == 2)
                        RL_LAUNCH((gemv_update_kernel<T, TA>), std::min(gridr, ceil_div(b0, wpb)), 32 * wpb, 0, s, A + b0, lda,
                                  b0, bs, Yb, ldy, Y, nrhs, false);
                    else
                        RL_LAUNCH((gemv_update_kernel<T, TA>), ceil_div(b0, 256), 256, 0, s, A + (long long)b0 * lda, lda, b0,
                                  bs, Yb, ldy, Y, nrhs, true);
                }
            }
        }
        return RL_OK;
    }
    if (sweep_groups(nrhs) > 0 && !g_shared_gpu) {
        // Up to kSweepGroups x kSweepRhs right-hand sides: the whole solve in one launch
        // (trsv_sweep_kernel, groups of kSweepRhs columns side by side). The blocked form
        // below costs two launches per 64-row block, a 64-step chain on a few CTAs and a
        // GEMM whose tiles would be mostly empty.
        const int nb = ceil_div(n, kSweepRows), words = sweep_ctl_words(n, nrhs);
        DevBuf<int> ctl;
        RL_TRY(ctl.alloc(words, s));
        RL_TRY_CUDA(cudaMemsetAsync(ctl.p, 0, sizeof(int) * words, s));
        // one right-hand side: the 1-wide instance (the 8-wide one would issue 8 FMAs per
        // element, 7 of them predicated off, each a full issue of the FP64 pipe for T = double)
        const dim3 grid(std::min(nb, kSweepCtas), sweep_groups(nrhs));
        if (nrhs == 1)
            RL_LAUNCH((trsv_sweep_kernel<T, TA, 1>), grid, 256, 0, s, A, lda, n, Y, ldy, nrhs, mode, ctl.p, dstatus, tiny,
                      wait_ns(), (int)tune(RL_TUNE_TEST_WITHHOLD_SWEEP_BLOCK), (const T *)nullptr);
        else
            RL_LAUNCH((trsv_sweep_kernel<T, TA>), grid, 256, 0, s, A, lda, n, Y, ldy, nrhs, mode, ctl.p, dstatus, tiny,
                      wait_ns(), (int)tune(RL_TUNE_TEST_WITHHOLD_SWEEP_BLOCK), (const T *)nullptr);
        return RL_OK;
    }
    if constexpr (!std::is_same<T, TA>::value) {
        return RL_ERR_INVALID_ARG;  // mixed storage: few right-hand sides only
    } else {
        const int gr = ceil_div(nrhs, kTrsmCols);
        if (mode == 0 || mode == 1) {
            for (int b0 = 0; b0 < n; b0 += NB) {
                const int bs = std::min(NB, n - b0);
                const T *D = A + (long long)b0 * lda + b0;
                T *Yb = Y + (long long)b0 * ldy;
                RL_LAUNCH(trsm_diag_kernel<T>, gr, 128, 0, s, D, lda, bs, Yb, ldy, nrhs, mode, dstatus, tiny);
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
                RL_LAUNCH(trsm_diag_kernel<T>, gr, 128, 0, s, D, lda, bs, Yb, ldy, nrhs, mode, dstatus, tiny);
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
}

// Inverses of op(A)'s 64 x 64 diagonal blocks, formed in T (ceil(n / 64) row-major
// 64 x 64 blocks in Dinv; diag_inverse_kernel).
template <class T, class TA>
rl_status diag_inverse(const TA *A, long long lda, int n, int mode, T *Dinv, int *dstatus, cudaStream_t s, T tiny) {
    if (n <= 0) return RL_OK;
    RL_LAUNCH((diag_inverse_kernel<T, TA>), ceil_div(n, kSweepRows), 64, 0, s, A, lda, n, mode, Dinv, dstatus, tiny);
    return RL_OK;
}

// op(A) Y = Y' for at most kSweepGroups x kSweepRhs right-hand sides in one sweep launch
// whose block solves are products with the diagonal blocks' inverses Dinv
// (diag_inverse). ctl: sweep_ctl_words(n, nrhs) zeroed ints (each group's ticket and
// block flags). More right-hand sides, or a GPU shared with other streams of this
// library (the serving workers, see tri_solve_dev), take tri_solve_dev's substitution
// paths instead.
template <class T, class TA>
rl_status tri_solve_inv_dev(const TA *A, long long lda, int n, const T *Dinv, T *Y, long long ldy, int nrhs, int mode,
                            int *dstatus, cudaStream_t s, T tiny, int *ctl) {
    if (sweep_groups(nrhs) == 0 || g_shared_gpu)
        return tri_solve_dev<T, TA>(A, lda, n, Y, ldy, nrhs, mode, dstatus, s, tiny);
    if (n <= 0 || nrhs <= 0) return RL_OK;
    const int nb = ceil_div(n, kSweepRows);
    const dim3 grid(std::min(nb, kSweepCtas), sweep_groups(nrhs));
    if (nrhs == 1)
        RL_LAUNCH((trsv_sweep_kernel<T, TA, 1>), grid, 256, 0, s, A, lda, n, Y, ldy, nrhs, mode, ctl, dstatus, tiny,
                  wait_ns(), (int)tune(RL_TUNE_TEST_WITHHOLD_SWEEP_BLOCK), Dinv);
    else
        RL_LAUNCH((trsv_sweep_kernel<T, TA>), grid, 256, 0, s, A, lda, n, Y, ldy, nrhs, mode, ctl, dstatus, tiny,
                  wait_ns(), (int)tune(RL_TUNE_TEST_WITHHOLD_SWEEP_BLOCK), Dinv);
    return RL_OK;
}

static __global__ void ipiv_to_perm_kernel(const int *ipiv, int n, uint64_t *perm, uint64_t *scratch) {
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

inline rl_status check_perm(size_t n, const uint64_t *perm) {
    std::vector<unsigned char> seen(n, 0);
    for (size_t i = 0; i < n; i++) {
        if (perm[i] >= n || seen[perm[i]]) return RL_ERR_INVALID_PERMUTATION;
        seen[perm[i]] = 1;
    }
    return RL_OK;
}

inline bool fits_int(size_t v) { return v <= (size_t)INT32_MAX; }

}  // namespace rl
