// Tiled SIMT GEMM for sm_103a, used for Matrix * Matrix and for the trailing-matrix
// updates of the blocked factorisations:
//     C = alpha * op(A) * op(B) + beta * C,   row-major, op = identity or transpose.
// FP32 uses FFMA (74 TFLOP/s on GB300); FP64 uses DFMA (GB300's FP64 rate is the same
// ~1 TFLOP/s through DFMA and through DMMA, so the SIMT form loses nothing and keeps one
// code path). Tiles are double-buffered through shared memory; every thread owns a
// TM x TN register tile split into 4x4 quadrants to keep shared-memory reads
// conflict-free.
#pragma once

#include <type_traits>

#include "common.cuh"
#include "gemm_tc.cuh"

namespace rl {

template <class T>
struct GemmCfg;
template <>
struct GemmCfg<float> {
    static constexpr int BM = 128, BN = 128, BK = 8, TM = 8, TN = 8;
};
template <>
struct GemmCfg<double> {
    static constexpr int BM = 64, BN = 64, BK = 8, TM = 4, TN = 4;
};

template <class T>
__device__ __forceinline__ void lds4(const T *p, T (&o)[4]);
template <>
__device__ __forceinline__ void lds4<float>(const float *p, float (&o)[4]) {
    float4 v = *reinterpret_cast<const float4 *>(p);
    o[0] = v.x, o[1] = v.y, o[2] = v.z, o[3] = v.w;
}
template <>
__device__ __forceinline__ void lds4<double>(const double *p, double (&o)[4]) {
    double2 v0 = reinterpret_cast<const double2 *>(p)[0];
    double2 v1 = reinterpret_cast<const double2 *>(p)[1];
    o[0] = v0.x, o[1] = v0.y, o[2] = v1.x, o[3] = v1.y;
}

// op(A) is m x k: A[i * lda + p] (TA = false) or A[p * lda + i] (TA = true).
// op(B) is k x n: B[p * ldb + j] (TB = false) or B[j * ldb + p] (TB = true).
// LOWER = true computes only the tiles that touch the lower triangle (i >= j) and only
// writes elements with i >= j (the SYRK form used by Cholesky).
template <class T, bool TA, bool TB, bool LOWER>
__global__ void __launch_bounds__((GemmCfg<T>::BM / GemmCfg<T>::TM) * (GemmCfg<T>::BN / GemmCfg<T>::TN))
    gemm_kernel(int m, int n, int k, T alpha, const T *__restrict__ A, long long lda, const T *__restrict__ B,
                long long ldb, T beta, T *__restrict__ C, long long ldc, int kslice, long long zstride) {
    constexpr int BM = GemmCfg<T>::BM, BN = GemmCfg<T>::BN, BK = GemmCfg<T>::BK;
    constexpr int TM = GemmCfg<T>::TM, TN = GemmCfg<T>::TN;
    constexpr int NTX = BN / TN, NTY = BM / TM, NT = NTX * NTY;
    constexpr int SM_ = TM / 4, SN_ = TN / 4;  // quadrants per thread
    constexpr int A_PER = BM * BK / NT, B_PER = BK * BN / NT;
    static_assert(A_PER >= 1 && B_PER >= 1, "tile too small for the block");

    __shared__ __align__(16) T As[2][BK][BM];
    __shared__ __align__(16) T Bs[2][BK][BN];

    if (gridDim.z > 1) {  // split K: slice z of the reduction into its own partial C
        const int kz = blockIdx.z * kslice;
        k = max(0, min(kslice, k - kz));
        A += TA ? (long long)kz * lda : kz;
        B += TB ? kz : (long long)kz * ldb;
        C += blockIdx.z * zstride;
    }
    const int tid = threadIdx.x;
    const int tx = tid % NTX, ty = tid / NTX;
    const int row0 = blockIdx.y * BM, col0 = blockIdx.x * BN;
    if (LOWER && col0 > row0 + BM - 1) return;  // tile strictly above the diagonal

    T acc[TM][TN];
#pragma unroll
    for (int i = 0; i < TM; i++)
#pragma unroll
        for (int j = 0; j < TN; j++) acc[i][j] = T(0);

    T ra[A_PER], rb[B_PER];

    auto load_tile = [&](int k0) {
#pragma unroll
        for (int e = 0; e < A_PER; e++) {
            int idx = tid + e * NT;
            int i, p;
            if (TA) {  // consecutive threads along i (contiguous in memory)
                i = idx % BM;
                p = idx / BM;
            } else {  // consecutive threads along p
                p = idx % BK;
                i = idx / BK;
            }
            int gi = row0 + i, gp = k0 + p;
            T v = T(0);
            if (gi < m && gp < k) v = TA ? A[(long long)gp * lda + gi] : A[(long long)gi * lda + gp];
            ra[e] = v;
        }
#pragma unroll
        for (int e = 0; e < B_PER; e++) {
            int idx = tid + e * NT;
            int j, p;
            if (TB) {
                p = idx % BK;
                j = idx / BK;
            } else {
                j = idx % BN;
                p = idx / BN;
            }
            int gj = col0 + j, gp = k0 + p;
            T v = T(0);
            if (gj < n && gp < k) v = TB ? B[(long long)gj * ldb + gp] : B[(long long)gp * ldb + gj];
            rb[e] = v;
        }
    };
    auto store_tile = [&](int buf) {
#pragma unroll
        for (int e = 0; e < A_PER; e++) {
            int idx = tid + e * NT;
            int i, p;
            if (TA) {
                i = idx % BM;
                p = idx / BM;
            } else {
                p = idx % BK;
                i = idx / BK;
            }
            As[buf][p][i] = ra[e];
        }
#pragma unroll
        for (int e = 0; e < B_PER; e++) {
            int idx = tid + e * NT;
            int j, p;
            if (TB) {
                p = idx % BK;
                j = idx / BK;
            } else {
                j = idx % BN;
                p = idx / BN;
            }
            Bs[buf][p][j] = rb[e];
        }
    };

    const int ktiles = (k + BK - 1) / BK;
    if (ktiles > 0) {
        load_tile(0);
        store_tile(0);
    }
    __syncthreads();
    for (int kt = 0; kt < ktiles; kt++) {
        const int buf = kt & 1;
        if (kt + 1 < ktiles) load_tile((kt + 1) * BK);
#pragma unroll
        for (int p = 0; p < BK; p++) {
            T a[TM], b[TN];
#pragma unroll
            for (int s = 0; s < SM_; s++) {
                T q[4];
                lds4<T>(&As[buf][p][s * (BM / SM_) + ty * 4], q);
#pragma unroll
                for (int r = 0; r < 4; r++) a[s * 4 + r] = q[r];
            }
#pragma unroll
            for (int s = 0; s < SN_; s++) {
                T q[4];
                lds4<T>(&Bs[buf][p][s * (BN / SN_) + tx * 4], q);
#pragma unroll
                for (int r = 0; r < 4; r++) b[s * 4 + r] = q[r];
            }
#pragma unroll
            for (int i = 0; i < TM; i++)
#pragma unroll
                for (int j = 0; j < TN; j++) acc[i][j] = fma(a[i], b[j], acc[i][j]);
        }
        if (kt + 1 < ktiles) store_tile(buf ^ 1);
        __syncthreads();
    }

#pragma unroll
    for (int i = 0; i < TM; i++) {
        const int gi = row0 + (i / 4) * (BM / SM_) + ty * 4 + (i % 4);
        if (gi >= m) continue;
#pragma unroll
        for (int j = 0; j < TN; j++) {
            const int gj = col0 + (j / 4) * (BN / SN_) + tx * 4 + (j % 4);
            if (gj >= n) continue;
            if (LOWER && gj > gi) continue;
            T *cp = C + (long long)gi * ldc + gj;
            T v = alpha * acc[i][j];
            if (beta != T(0)) v = fma(beta, *cp, v);
            *cp = v;
        }
    }
}

// Launches C = alpha * op(A) op(B) + beta * C on `stream`. FP32 products with at least
// a 128 x 128 tile's worth of C and K >= 256 go to the tcgen05 kernel (gemm_tc.cuh).
// A product with fewer tiles than SMs and a long K (the V^T A2 and V^T V products of a
// Householder block, K = the panel height) is split along K into partial tiles that
// run at once, then added in slice order.
template <class T, bool TA, bool TB, bool LOWER = false>
rl_status gemm(int m, int n, int k, T alpha, const T *A, long long lda, const T *B, long long ldb, T beta, T *C,
               long long ldc, cudaStream_t stream) {
    if (m <= 0 || n <= 0) return RL_OK;
    constexpr int BM = GemmCfg<T>::BM, BN = GemmCfg<T>::BN, BK = GemmCfg<T>::BK;
    constexpr int NT = (BM / GemmCfg<T>::TM) * (BN / GemmCfg<T>::TN);
    dim3 grid((n + BN - 1) / BN, (m + BM - 1) / BM);
    const int tiles = (int)(grid.x * grid.y), sms = num_sms();
    if constexpr (std::is_same<T, float>::value) {  // FP32 with enough work: tensor cores (3xTF32)
        if (sgemm_tc_eligible(m, n, k)) {
            const int tc_tiles = ceil_div(n, tc::BN) * ceil_div(m, tc::BM);
            int ks = 1;
            if (!LOWER && tc_tiles < sms / 2 && k >= 1024) ks = std::min({16, ceil_div(sms, tc_tiles), k / 256});
            return sgemm_tc<TA, TB>(m, n, k, alpha, A, lda, B, ldb, beta, C, ldc, LOWER, stream, ks);
        }
    }
    int ksplit = 1;
    if (!LOWER && tiles < sms && k >= 1024) ksplit = std::min({16, ceil_div(2 * sms, tiles), k / 256});
    if (ksplit > 1) {
        const int kslice = ceil_div(ceil_div(k, ksplit), BK) * BK;
        ksplit = ceil_div(k, kslice);
        const long long zstride = (long long)m * n;
        DevBuf<T> part;
        RL_TRY(part.alloc((size_t)ksplit * zstride, stream));
        grid.z = ksplit;
        RL_LAUNCH((gemm_kernel<T, TA, TB, LOWER>), grid, NT, 0, stream, m, n, k, T(1), A, lda, B, ldb, T(0), part.p, (long long)n,
                  kslice, zstride);
        RL_LAUNCH(splitk_reduce_kernel<T>, std::min(4 * sms, ceil_div(zstride, 256)), 256, 0, stream, m, n, ksplit, alpha,
                  part.p, beta, C, ldc);
        return RL_OK;
    }
    RL_LAUNCH((gemm_kernel<T, TA, TB, LOWER>), grid, NT, 0, stream, m, n, k, alpha, A, lda, B, ldb, beta, C, ldc, k,
              0ll);
    return RL_OK;
}

}  // namespace rl
