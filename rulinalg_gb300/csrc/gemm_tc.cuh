// FP32 GEMM on the 5th-generation tensor cores (tcgen05, TF32 inputs, FP32 accumulation
// in tensor memory) with FP32 accuracy from the 3xTF32 split: every operand x is held as
// hi = tf32(x) (round to nearest) and lo = x - hi, and each product as
// a_lo b_hi + a_hi b_lo + a_hi b_hi (the a_lo b_lo term is below FP32 rounding).
//
//     C = alpha * A * B + beta * C,  A (m x k), B (k x n), C (m x n), row-major.
//
// One CTA (4 warps) computes a 128 x 128 tile of C in 128 columns of tensor memory.
// K advances in chunks of 32: all threads load the chunk of A and B from global memory,
// split it and store hi and lo into shared memory in the no-swizzle K-major "core
// matrix" layout (8 rows x 16 bytes per core matrix; core matrices 128 bytes apart along
// K and 256 bytes apart along M/N), one thread issues the 12 MMAs of the chunk
// (4 k-steps of 8 x 3 products) and commits them to the chunk's mbarrier. Two chunk
// buffers alternate, so the next chunk's loads overlap the current chunk's MMAs; a buffer
// is rewritten only after its mbarrier reports the MMAs that read it complete. The
// epilogue reads the accumulator back with tcgen05.ld (warp w owns rows 32w..32w+31).
// Every mbarrier wait is bounded; on expiry the CTA records RL_ERR_TIMEOUT, skips the
// epilogue, frees its tensor memory and returns.
#pragma once

#include <cstdint>

#include "common.cuh"

namespace rl {
namespace tc {

constexpr int BM = 128, BN = 128, BK = 32;
constexpr int KSTEP = 8;                       // K of one kind::tf32 MMA
constexpr int NSTEP = BK / KSTEP;              // MMA k-steps per chunk
constexpr int OPER_BYTES = BM * KSTEP * 4;     // one operand k-step tile (128 rows x 8): 4 KB
constexpr int CHUNK_BYTES = NSTEP * OPER_BYTES;  // one operand chunk: 16 KB
constexpr int STAGE_BYTES = 4 * CHUNK_BYTES;   // A_hi, A_lo, B_hi, B_lo: 64 KB
constexpr int SMEM_BYTES = 2 * STAGE_BYTES + 64;
constexpr int THREADS = 128;
constexpr int TMEM_COLS = 128;
constexpr unsigned long long kWaitLimit = 1ull << 26;  // polls of an mbarrier before giving up

__device__ __forceinline__ uint32_t smem_u32(const void *p) { return (uint32_t)__cvta_generic_to_shared(p); }

// Shared-memory matrix descriptor: no swizzle, K-major, leading (K) and stride (M/N)
// byte offsets between core matrices.
__device__ __forceinline__ uint64_t smem_desc(uint32_t addr, uint32_t lbo, uint32_t sbo) {
    uint64_t d = 0;
    d |= (uint64_t)((addr >> 4) & 0x3FFFu);
    d |= (uint64_t)((lbo >> 4) & 0x3FFFu) << 16;
    d |= (uint64_t)((sbo >> 4) & 0x3FFFu) << 32;
    d |= (uint64_t)1 << 46;  // descriptor version of this architecture
    return d;                // base offset 0, layout type 0 (no swizzle)
}

// Instruction descriptor of kind::tf32: D F32, A and B TF32, both K-major, N, M.
__host__ __device__ constexpr uint32_t idesc_tf32(int M, int N) {
    return (1u << 4) | (2u << 7) | (2u << 10) | ((uint32_t)(N >> 3) << 17) | ((uint32_t)(M >> 4) << 24);
}

// Byte offset of element (row r, k) inside one 128 x 8 k-step tile.
__device__ __forceinline__ uint32_t tile_off(int r, int k) {
    return (uint32_t)((r >> 3) * 256 + (k >> 2) * 128 + (r & 7) * 16 + (k & 3) * 4);
}

__device__ __forceinline__ float tf32_rna(float x) {
    uint32_t r;
    asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(r) : "f"(x));
    return __uint_as_float(r);
}

__device__ __forceinline__ void mbar_init(uint64_t *bar, unsigned count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}

// Bounded wait for the given phase parity; false on expiry.
__device__ __forceinline__ bool mbar_wait(uint64_t *bar, unsigned parity) {
    const uint32_t a = smem_u32(bar);
    for (unsigned long long i = 0; i < kWaitLimit; i++) {
        uint32_t done;
        asm volatile(
            "{\n\t.reg .pred p;\n\t"
            "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
            "selp.u32 %0, 1, 0, p;\n\t}"
            : "=r"(done)
            : "r"(a), "r"(parity)
            : "memory");
        if (done) return true;
    }
    return false;
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

// A and B rows must start 16-byte aligned (lda, ldb multiples of 4, A and B aligned).
static __global__ void __launch_bounds__(tc::THREADS, 1)
    sgemm_tc_kernel(int m, int n, int k, float alpha, const float *__restrict__ A, long long lda,
                    const float *__restrict__ B, long long ldb, float beta, float *__restrict__ C, long long ldc,
                    int *err) {
    using namespace tc;
    extern __shared__ __align__(1024) unsigned char smem[];
    uint64_t *bar = reinterpret_cast<uint64_t *>(smem + 2 * STAGE_BYTES);  // 2 mbarriers
    uint32_t *tmem_slot = reinterpret_cast<uint32_t *>(smem + 2 * STAGE_BYTES + 16);
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int row0 = blockIdx.y * BM, col0 = blockIdx.x * BN;

    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(tmem_slot)),
                     "r"(TMEM_COLS)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    if (tid == 0) {
        mbar_init(&bar[0], 1);
        mbar_init(&bar[1], 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    const uint32_t tmem = *tmem_slot;
    constexpr uint32_t idesc = idesc_tf32(BM, BN);
    bool ok = true;

    const int nchunks = (k + BK - 1) / BK;
    for (int c = 0; c < nchunks && ok; c++) {
        const int s = c & 1;
        unsigned char *st = smem + s * STAGE_BYTES;
        if (c >= 2) ok = mbar_wait(&bar[s], ((c - 2) >> 1) & 1);  // the MMAs that read this stage
        if (!__syncthreads_and(ok)) {
            ok = false;
            break;
        }
        const int k0 = c * BK;
        // A chunk: 128 rows x 32 k, float4 along k (one core-matrix row per float4)
#pragma unroll
        for (int e = 0; e < (BM * BK / 4) / THREADS; e++) {
            const int idx = tid + e * THREADS, r = idx >> 3, kq = (idx & 7) * 4;
            const int gr = row0 + r, gk = k0 + kq;
            float4 v = make_float4(0.f, 0.f, 0.f, 0.f);
            if (gr < m) {
                const float *src = A + (long long)gr * lda + gk;
                if (gk + 3 < k)
                    v = *reinterpret_cast<const float4 *>(src);
                else {
                    if (gk < k) v.x = src[0];
                    if (gk + 1 < k) v.y = src[1];
                    if (gk + 2 < k) v.z = src[2];
                }
            }
            const float h0 = tf32_rna(v.x), h1 = tf32_rna(v.y), h2 = tf32_rna(v.z), h3 = tf32_rna(v.w);
            const uint32_t off = (kq >> 3) * OPER_BYTES + tile_off(r, kq & 7);
            *reinterpret_cast<float4 *>(st + off) = make_float4(h0, h1, h2, h3);
            *reinterpret_cast<float4 *>(st + CHUNK_BYTES + off) =
                make_float4(v.x - h0, v.y - h1, v.z - h2, v.w - h3);
        }
        // B chunk: 32 k x 128 n, float4 along n (four rows of the K-major B tile)
#pragma unroll
        for (int e = 0; e < (BK * BN / 4) / THREADS; e++) {
            const int idx = tid + e * THREADS, kk = idx >> 5, nq = (idx & 31) * 4;
            const int gk = k0 + kk, gn = col0 + nq;
            float4 v = make_float4(0.f, 0.f, 0.f, 0.f);
            if (gk < k) {
                const float *src = B + (long long)gk * ldb + gn;
                if (gn + 3 < n)
                    v = *reinterpret_cast<const float4 *>(src);
                else {
                    if (gn < n) v.x = src[0];
                    if (gn + 1 < n) v.y = src[1];
                    if (gn + 2 < n) v.z = src[2];
                }
            }
            const float x[4] = {v.x, v.y, v.z, v.w};
            unsigned char *bh = st + 2 * CHUNK_BYTES + (kk >> 3) * OPER_BYTES;
            unsigned char *bl = st + 3 * CHUNK_BYTES + (kk >> 3) * OPER_BYTES;
#pragma unroll
            for (int q = 0; q < 4; q++) {
                const float h = tf32_rna(x[q]);
                const uint32_t off = tile_off(nq + q, kk & 7);
                *reinterpret_cast<float *>(bh + off) = h;
                *reinterpret_cast<float *>(bl + off) = x[q] - h;
            }
        }
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");  // make the stores visible to the MMAs
        __syncthreads();
        if (tid == 0) {
            asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
            const uint32_t base = smem_u32(st);
#pragma unroll
            for (int ks = 0; ks < NSTEP; ks++) {
                const uint32_t o = ks * OPER_BYTES;
                const uint64_t ah = smem_desc(base + o, 128, 256), al = smem_desc(base + CHUNK_BYTES + o, 128, 256);
                const uint64_t bh = smem_desc(base + 2 * CHUNK_BYTES + o, 128, 256),
                               bl = smem_desc(base + 3 * CHUNK_BYTES + o, 128, 256);
                mma_tf32(tmem, al, bh, idesc, (c > 0 || ks > 0) ? 1u : 0u);
                mma_tf32(tmem, ah, bl, idesc, 1u);
                mma_tf32(tmem, ah, bh, idesc, 1u);
            }
            mma_commit(&bar[s]);
        }
    }
    // all MMAs done: the last chunk's commit covers every earlier MMA of this thread
    if (ok && nchunks > 0) ok = mbar_wait(&bar[(nchunks - 1) & 1], ((nchunks - 1) >> 1) & 1);
    ok = __syncthreads_and(ok) != 0;
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    if (ok) {
        const int r = row0 + warp * 32 + lane;
#pragma unroll 1
        for (int c0 = 0; c0 < BN; c0 += 16) {
            float v[16];
            tc::tmem_ld16(tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)c0, v);
            if (r < m) {
                float *dst = C + (long long)r * ldc + col0 + c0;
#pragma unroll
                for (int j = 0; j < 16; j++) {
                    if (col0 + c0 + j < n) {
                        float out = alpha * (nchunks > 0 ? v[j] : 0.f);
                        if (beta != 0.f) out = fmaf(beta, dst[j], out);
                        dst[j] = out;
                    }
                }
            }
        }
    } else if (tid == 0) {
        atomicCAS(err, 0, RL_ERR_TIMEOUT);
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    if (warp == 0)
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(TMEM_COLS) : "memory");
}

}  // namespace rl

namespace rl {

// Sticky timeout word of the tensor-core GEMM (one per translation unit that launches it).
static __device__ int g_sgemm_tc_err;

inline bool sgemm_tc_eligible(int m, int n, int k, const float *A, long long lda, const float *B, long long ldb) {
    return m >= 128 && n >= 128 && k >= tc::BK && lda % 4 == 0 && ldb % 4 == 0 &&
           reinterpret_cast<uintptr_t>(A) % 16 == 0 && reinterpret_cast<uintptr_t>(B) % 16 == 0;
}

// C = alpha A B + beta C on the tensor cores (3xTF32); the caller checks eligibility.
inline rl_status sgemm_tc(int m, int n, int k, float alpha, const float *A, long long lda, const float *B, long long ldb,
                          float beta, float *C, long long ldc, cudaStream_t s) {
    static const cudaError_t attr =
        cudaFuncSetAttribute(sgemm_tc_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, tc::SMEM_BYTES);
    RL_TRY_CUDA(attr);
    int *err = nullptr;
    RL_TRY_CUDA(cudaGetSymbolAddress(reinterpret_cast<void **>(&err), g_sgemm_tc_err));
    const dim3 grid((n + tc::BN - 1) / tc::BN, (m + tc::BM - 1) / tc::BM);
    RL_LAUNCH(sgemm_tc_kernel, grid, tc::THREADS, tc::SMEM_BYTES, s, m, n, k, alpha, A, lda, B, ldb, beta, C, ldc,
              err);
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
