// FP32 GEMM on the 5th-generation tensor cores with FP32 accuracy (3xTF32):
//
//     C = alpha * A * B + beta * C,  A (m x k), B (k x n), C (m x n), row-major.
//
// Every operand x is split once into hi = tf32(x) (round to nearest) and lo = x - hi
// (split_rows_kernel for A, split_transpose_kernel for B, which also transposes B to
// K-major), and each product is accumulated as a_lo b_hi + a_hi b_lo + a_hi b_hi in FP32
// in tensor memory (the a_lo b_lo term is below FP32 rounding).
//
// sgemm_tma_kernel: one CTA (4 warps) per 128 x 128 tile of C, accumulator in 128
// columns of tensor memory. K advances in chunks of 32 through a 3-stage ring of shared
// memory, each stage holding the four 128 x 32 operand tiles (A_hi, A_lo, B_hi, B_lo),
// loaded by TMA with the 128-byte swizzle the MMA descriptors expect. Warp 0 lane 0
// produces (waits for a stage to be empty, arms its mbarrier with the byte count, issues
// the four tensor copies), warp 1 lane 0 issues the 12 MMAs of each chunk (4 k-steps x
// 3 products, kind::tf32, M = N = 128, K = 8) and commits them to the stage's empty
// barrier, and finally to a done barrier that the four warps wait on before reading the
// accumulator back with tcgen05.ld (warp w owns rows 32w .. 32w + 31). Every mbarrier wait
// is bounded; on expiry the CTA records RL_ERR_TIMEOUT, writes NaN over its tile, frees
// its tensor memory and returns.
#pragma once

#include <cuda.h>
#include <cudaTypedefs.h>

#include <cstdint>
#include <mutex>

#include "common.cuh"

namespace rl {
namespace tc {

constexpr int BM = 128, BN = 128, BK = 32, STAGES = 3;
constexpr int TILE_BYTES = BM * BK * 4;        // one 128 x 32 FP32 operand tile: 16 KB
constexpr int STAGE_BYTES = 4 * TILE_BYTES;    // A_hi, A_lo, B_hi, B_lo: 64 KB
constexpr int SMEM_BYTES = STAGES * STAGE_BYTES + 1024 + 256;  // + alignment slack + barriers
constexpr int THREADS = 128;
constexpr int TMEM_COLS = 128;

__device__ __forceinline__ uint32_t smem_u32(const void *p) { return (uint32_t)__cvta_generic_to_shared(p); }

// Shared-memory matrix descriptor for a K-major operand in the 128-byte swizzle layout
// (8-row groups 1024 bytes apart; the start address moves by 32 bytes per K = 8 step
// inside the 128-byte swizzle atom).
__device__ __forceinline__ uint64_t smem_desc_sw128(uint32_t addr) {
    uint64_t d = 0;
    d |= (uint64_t)((addr >> 4) & 0x3FFFu);
    d |= (uint64_t)1 << 16;             // leading byte offset (unused for swizzled K-major)
    d |= (uint64_t)(1024 >> 4) << 32;   // stride byte offset: 8 rows x 128 bytes
    d |= (uint64_t)1 << 46;             // descriptor version of this architecture
    d |= (uint64_t)2 << 61;             // layout: 128-byte swizzle
    return d;
}

// Instruction descriptor of kind::tf32: D F32, A and B TF32, both K-major, N, M.
__host__ __device__ constexpr uint32_t idesc_tf32(int M, int N) {
    return (1u << 4) | (2u << 7) | (2u << 10) | ((uint32_t)(N >> 3) << 17) | ((uint32_t)(M >> 4) << 24);
}

__device__ __forceinline__ float tf32_rna(float x) {
    uint32_t r;
    asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(r) : "f"(x));
    return __uint_as_float(r);
}

__device__ __forceinline__ void mbar_init(uint64_t *bar, unsigned count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}

__device__ __forceinline__ void mbar_expect_tx(uint64_t *bar, unsigned bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes)
                 : "memory");
}

// Wait for the given phase parity, bounded by `limit` ns of %globaltimer (try_wait may
// itself suspend the thread for a hardware-defined time, so a poll count would not bound
// the wall time); false on expiry.
__device__ __forceinline__ bool mbar_wait(uint64_t *bar, unsigned parity, unsigned long long limit) {
    const uint32_t a = smem_u32(bar);
    unsigned long long t0, t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t0));
    for (;;) {
        uint32_t done;
        asm volatile(
            "{\n\t.reg .pred p;\n\t"
            "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
            "selp.u32 %0, 1, 0, p;\n\t}"
            : "=r"(done)
            : "r"(a), "r"(parity)
            : "memory");
        if (done) return true;
        asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
        if (t - t0 > limit) return false;
    }
}

// 2D tensor copy global -> shared (x = the K coordinate, y = the row), completing on bar.
__device__ __forceinline__ void tma_load_2d(void *dst, const CUtensorMap *map, int x, int y, uint64_t *bar) {
    asm volatile(
        "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], [%4];" ::"r"(
            smem_u32(dst)),
        "l"(reinterpret_cast<uint64_t>(map)), "r"(x), "r"(y), "r"(smem_u32(bar))
        : "memory");
}

__device__ __forceinline__ void mma_tf32(uint32_t d_tmem, uint64_t a_desc, uint64_t b_desc, uint32_t idesc,
                                         uint32_t accumulate) {
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "setp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n\t}" ::"r"(d_tmem),
        "l"(a_desc), "l"(b_desc), "r"(idesc), "r"(accumulate)
        : "memory");
}

__device__ __forceinline__ void mma_commit(uint64_t *bar) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_u32(bar))
                 : "memory");
}

__device__ __forceinline__ void tmem_ld16(uint32_t taddr, float (&v)[16]) {
    uint32_t r[16];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
          "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
        : "r"(taddr));
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
    for (int i = 0; i < 16; i++) v[i] = __uint_as_float(r[i]);
}

}  // namespace tc

// hi/lo of A (rows x k, row stride ldx) into rows x kp buffers (kp = k rounded up to 32,
// zero beyond k).
static __global__ void split_rows_kernel(const float *__restrict__ X, long long ldx, int rows, int k, int kp,
                                         float *__restrict__ hi, float *__restrict__ lo) {
    const long long total = (long long)rows * kp;
    for (long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x; e < total; e += (long long)gridDim.x * blockDim.x) {
        const int r = (int)(e / kp), c = (int)(e - (long long)r * kp);
        const float x = c < k ? X[(long long)r * ldx + c] : 0.f;
        const float h = tc::tf32_rna(x);
        hi[e] = h;
        lo[e] = x - h;
    }
}

// hi/lo of B^T: B is k x n (row stride ldb); outputs are n x kp (K-major), zero beyond k.
// 32 x 32 tiles through shared memory; block (32, 8).
static __global__ void split_transpose_kernel(const float *__restrict__ B, long long ldb, int k, int n, int kp,
                                              float *__restrict__ hi, float *__restrict__ lo) {
    __shared__ float t[32][33];
    const int tx = threadIdx.x, ty = threadIdx.y;
    const int n0 = blockIdx.x * 32, k0 = blockIdx.y * 32;
#pragma unroll
    for (int j = 0; j < 4; j++) {
        const int kk = k0 + ty + 8 * j, nn = n0 + tx;
        t[ty + 8 * j][tx] = (kk < k && nn < n) ? B[(long long)kk * ldb + nn] : 0.f;
    }
    __syncthreads();
#pragma unroll
    for (int j = 0; j < 4; j++) {
        const int nn = n0 + ty + 8 * j, kk = k0 + tx;
        if (nn < n) {
            const float x = t[tx][ty + 8 * j];
            const float h = tc::tf32_rna(x);
            hi[(long long)nn * kp + kk] = h;
            lo[(long long)nn * kp + kk] = x - h;
        }
    }
}

static __global__ void __launch_bounds__(tc::THREADS, 1)
    sgemm_tma_kernel(const __grid_constant__ CUtensorMap tAh, const __grid_constant__ CUtensorMap tAl,
                     const __grid_constant__ CUtensorMap tBh, const __grid_constant__ CUtensorMap tBl, int m, int n,
                     int kp, float alpha, float beta, float *__restrict__ C, long long ldc, int lower, int *err,
                     int kc_per, long long zstride, unsigned long long wait_ns) {
    using namespace tc;
    // lower: only the elements on or below the diagonal are written (the SYRK form);
    // tiles wholly above it do nothing
    if (lower && (int)(blockIdx.x * BN) >= (int)(blockIdx.y * BM) + BM) return;
    extern __shared__ unsigned char smem_raw[];
    unsigned char *smem =
        reinterpret_cast<unsigned char *>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
    uint64_t *full = reinterpret_cast<uint64_t *>(smem + STAGES * STAGE_BYTES);
    uint64_t *empty = full + STAGES;
    uint64_t *done = empty + STAGES;
    uint32_t *tmem_slot = reinterpret_cast<uint32_t *>(done + 1);
    __shared__ int s_fail;
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int row0 = blockIdx.y * BM, col0 = blockIdx.x * BN;
    // split K: slice z covers the K chunks [c_begin, c_begin + nk) into its own partial C
    const int c_begin = blockIdx.z * kc_per;
    const int nk = max(0, min(kp / BK, c_begin + kc_per) - c_begin);
    C += blockIdx.z * zstride;

    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(tmem_slot)),
                     "r"(TMEM_COLS)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    if (tid == 0) {
        s_fail = 0;
        for (int s = 0; s < STAGES; s++) {
            mbar_init(&full[s], 1);
            mbar_init(&empty[s], 1);
        }
        mbar_init(done, 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    const uint32_t tmem = *tmem_slot;

    int issued = 0;  // producer: chunks whose loads were issued
    if (warp == 0 && lane == 0) {  // producer
        for (int c = 0; c < nk; c++) {
            const int s = c % STAGES, use = c / STAGES;
            if (use > 0 && !mbar_wait(&empty[s], (use - 1) & 1, wait_ns)) {
                s_fail = 1;
                break;
            }
            unsigned char *st = smem + s * STAGE_BYTES;
            mbar_expect_tx(&full[s], STAGE_BYTES);
            const int x = (c_begin + c) * BK;
            tma_load_2d(st, &tAh, x, row0, &full[s]);
            tma_load_2d(st + TILE_BYTES, &tAl, x, row0, &full[s]);
            tma_load_2d(st + 2 * TILE_BYTES, &tBh, x, col0, &full[s]);
            tma_load_2d(st + 3 * TILE_BYTES, &tBl, x, col0, &full[s]);
            issued = c + 1;
        }
    } else if (warp == 1 && lane == 0) {  // MMA issuer
        constexpr uint32_t idesc = idesc_tf32(BM, BN);
        for (int c = 0; c < nk; c++) {
            const int s = c % STAGES, use = c / STAGES;
            if (!mbar_wait(&full[s], use & 1, wait_ns)) {
                s_fail = 1;
                break;
            }
            asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
            const uint32_t base = smem_u32(smem + s * STAGE_BYTES);
#pragma unroll
            for (int ks = 0; ks < BK / 8; ks++) {
                const uint32_t o = ks * 32;
                const uint64_t ah = smem_desc_sw128(base + o), al = smem_desc_sw128(base + TILE_BYTES + o);
                const uint64_t bh = smem_desc_sw128(base + 2 * TILE_BYTES + o),
                               bl = smem_desc_sw128(base + 3 * TILE_BYTES + o);
                mma_tf32(tmem, al, bh, idesc, (c > 0 || ks > 0) ? 1u : 0u);
                mma_tf32(tmem, ah, bl, idesc, 1u);
                mma_tf32(tmem, ah, bh, idesc, 1u);
            }
            mma_commit(&empty[s]);
        }
        mma_commit(done);
    }
    __syncwarp();
    bool ok = nk == 0 || mbar_wait(done, 0, wait_ns);  // every MMA issued (also after a failure) has completed
    ok = __syncthreads_and(ok && !s_fail) != 0;
    if (!ok && warp == 0 && lane == 0) {
        // Drain: the last load issued on each stage must land before this CTA's shared
        // memory is given up (a wait that runs out here leaves nothing else to do).
        for (int c = max(0, issued - STAGES); c < issued; c++) mbar_wait(&full[c % STAGES], (c / STAGES) & 1, wait_ns);
    }
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    const int r = row0 + warp * 32 + lane;
#pragma unroll 1
    for (int c0 = 0; c0 < BN; c0 += 16) {
        float v[16];
        if (ok && nk > 0) {
            tc::tmem_ld16(tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)c0, v);
        } else {
#pragma unroll
            for (int j = 0; j < 16; j++) v[j] = ok ? 0.f : __int_as_float(0x7fc00000);
        }
        if (r < m) {
            float *dst = C + (long long)r * ldc + col0 + c0;
#pragma unroll
            for (int j = 0; j < 16; j++) {
                if (col0 + c0 + j < n && !(lower && col0 + c0 + j > r)) {
                    float out = alpha * v[j];
                    if (ok && beta != 0.f) out = fmaf(beta, dst[j], out);
                    dst[j] = out;
                }
            }
        }
    }
    if (!ok && tid == 0) atomicCAS(err, 0, RL_ERR_TIMEOUT);
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    if (warp == 0)
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(TMEM_COLS) : "memory");
}

// Sticky timeout word of the tensor-core GEMM (one per translation unit that launches it).
static __device__ int g_sgemm_tc_err;

// Shapes worth the tensor cores: at least half a 128 x 128 tile of C in each direction
// and K >= 256. Below that K the per-call split, tensor-map set-up and a pipeline that
// never fills cost more than the SIMT kernel saves (the K = 64 trailing updates of the
// blocked factorisations measured slower on this path).
inline bool sgemm_tc_eligible(int m, int n, int k) {
    return m >= 64 && n >= 64 && (long long)m * n >= 128 * 128 && k >= 256;
}

// cuTensorMapEncodeTiled from the driver, looked up once.
inline PFN_cuTensorMapEncodeTiled_v12000 tensor_map_encoder() {
    static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
    static std::once_flag once;
    std::call_once(once, [] {
        void *p = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) ==
                cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(p);
        cudaGetLastError();
    });
    return fn;
}

// A rows x kp FP32 matrix (row stride kp) as 128 x 32 tiles with the 128-byte swizzle.
inline rl_status make_tile_map(CUtensorMap &map, const float *base, int rows, int kp) {
    auto enc = tensor_map_encoder();
    if (!enc) return RL_ERR_CUDA;
    const cuuint64_t dims[2] = {(cuuint64_t)kp, (cuuint64_t)rows};
    const cuuint64_t strides[1] = {(cuuint64_t)kp * sizeof(float)};
    const cuuint32_t box[2] = {(cuuint32_t)tc::BK, (cuuint32_t)tc::BM};
    const cuuint32_t estr[2] = {1, 1};
    const CUresult r = enc(&map, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 2, const_cast<float *>(base), dims, strides, box, estr,
                           CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B,
                           CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    return r == CUDA_SUCCESS ? RL_OK : RL_ERR_CUDA;
}

// C = alpha * sum_z P[z] + beta * C (m x n; P[z] packed with row stride n), in z order.
template <class T>
__global__ void splitk_reduce_kernel(int m, int n, int nz, T alpha, const T *__restrict__ P, T beta, T *__restrict__ C,
                                     long long ldc) {
    const long long total = (long long)m * n;
    for (long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x; e < total; e += (long long)gridDim.x * blockDim.x) {
        T sum = T(0);
        for (int z = 0; z < nz; z++) sum += P[z * total + e];
        const int i = (int)(e / n), j = (int)(e - (long long)i * n);
        T *cp = C + (long long)i * ldc + j;
        T v = alpha * sum;
        if (beta != T(0)) v = fma(beta, *cp, v);
        *cp = v;
    }
}

// C = alpha op(A) op(B) + beta C on the tensor cores (3xTF32); any strides, any
// alignment. op(A) = A (m x k, A[i * lda + p]) or A^T (A[p * lda + i]); op(B) = B (k x n,
// B[p * ldb + j]) or B^T (B[j * ldb + p]). The split kernels repack both operands K-major.
// ksplit > 1 (not with `lower`) runs K in that many slices at once into partial tiles,
// added in slice order afterwards: for products with few output tiles and a long K.
template <bool TA, bool TB>
rl_status sgemm_tc(int m, int n, int k, float alpha, const float *A, long long lda, const float *B, long long ldb,
                   float beta, float *C, long long ldc, bool lower, cudaStream_t s, int ksplit = 1) {
    static const cudaError_t attr =
        cudaFuncSetAttribute(sgemm_tma_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, tc::SMEM_BYTES);
    RL_TRY_CUDA(attr);
    const int kp = (k + tc::BK - 1) / tc::BK * tc::BK;
    DevBuf<float> Ah, Al, Bh, Bl;
    RL_TRY(Ah.alloc((size_t)m * kp, s));
    RL_TRY(Al.alloc((size_t)m * kp, s));
    RL_TRY(Bh.alloc((size_t)n * kp, s));
    RL_TRY(Bl.alloc((size_t)n * kp, s));
    auto split_rows = [&](const float *X, long long ldx, int rows, float *hi, float *lo) -> rl_status {
        const long long t = (long long)rows * kp;
        RL_LAUNCH(split_rows_kernel, (int)std::min<long long>(8LL * num_sms(), (t + 255) / 256), 256, 0, s, X, ldx,
                  rows, k, kp, hi, lo);
        return RL_OK;
    };
    auto split_t = [&](const float *X, long long ldx, int rows, float *hi, float *lo) -> rl_status {
        RL_LAUNCH(split_transpose_kernel, dim3((rows + 31) / 32, kp / 32), dim3(32, 8), 0, s, X, ldx, k, rows, kp, hi,
                  lo);
        return RL_OK;
    };
    RL_TRY(TA ? split_t(A, lda, m, Ah.p, Al.p) : split_rows(A, lda, m, Ah.p, Al.p));
    RL_TRY(TB ? split_rows(B, ldb, n, Bh.p, Bl.p) : split_t(B, ldb, n, Bh.p, Bl.p));
    CUtensorMap mAh, mAl, mBh, mBl;
    RL_TRY(make_tile_map(mAh, Ah.p, m, kp));
    RL_TRY(make_tile_map(mAl, Al.p, m, kp));
    RL_TRY(make_tile_map(mBh, Bh.p, n, kp));
    RL_TRY(make_tile_map(mBl, Bl.p, n, kp));
    int *err = nullptr;
    RL_TRY_CUDA(cudaGetSymbolAddress(reinterpret_cast<void **>(&err), g_sgemm_tc_err));
    dim3 grid((n + tc::BN - 1) / tc::BN, (m + tc::BM - 1) / tc::BM);
    const int nkc = kp / tc::BK;
    if (ksplit > 1 && !lower) {
        const int kc_per = (nkc + ksplit - 1) / ksplit;
        grid.z = (nkc + kc_per - 1) / kc_per;
        const long long zstride = (long long)m * n;
        DevBuf<float> part;
        RL_TRY(part.alloc((size_t)grid.z * zstride, s));
        RL_LAUNCH(sgemm_tma_kernel, grid, tc::THREADS, tc::SMEM_BYTES, s, mAh, mAl, mBh, mBl, m, n, kp, 1.f, 0.f, part.p,
                  (long long)n, 0, err, kc_per, zstride, wait_ns());
        RL_LAUNCH(splitk_reduce_kernel<float>, (int)std::min<long long>(4LL * num_sms(), (zstride + 255) / 256), 256, 0, s,
                  m, n, (int)grid.z, alpha, part.p, beta, C, ldc);
        return RL_OK;
    }
    RL_LAUNCH(sgemm_tma_kernel, grid, tc::THREADS, tc::SMEM_BYTES, s, mAh, mAl, mBh, mBl, m, n, kp, alpha, beta, C,
              ldc, lower ? 1 : 0, err, nkc, 0ll, wait_ns());
    return RL_OK;
}

// Reads and clears the sticky timeout word (synchronises the stream).
inline rl_status sgemm_tc_status(cudaStream_t s) {
    int *err = nullptr;
    RL_TRY_CUDA(cudaGetSymbolAddress(reinterpret_cast<void **>(&err), g_sgemm_tc_err));
    int h = 0;
    RL_TRY_CUDA(cudaMemcpyAsync(&h, err, sizeof(int), cudaMemcpyDeviceToHost, s));
    RL_TRY_CUDA(cudaStreamSynchronize(s));
    if (h) RL_TRY_CUDA(cudaMemsetAsync(err, 0, sizeof(int), s));
    return h ? RL_ERR_TIMEOUT : RL_OK;
}

}  // namespace rl
