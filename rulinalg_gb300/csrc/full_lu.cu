// FullPivLu: LU with complete pivoting (src/matrix/decomposition/lu.rs:303-599).
//
// One cooperative persistent launch runs all n elimination steps. Each step is a single
// pass over the trailing block with one grid barrier after it:
//   * the pivot of the step is the largest |a| of the trailing block with the first one in
//     row-major order winning ties (select_pivot, lu.rs:364-382); every CTA reduces the
//     per-CTA candidates of the previous pass itself, so all agree without another barrier;
//   * the row and column swaps are not moved through memory: the pass reads the current
//     trailing block (ping-pong buffer `cur`) through the swaps and writes the next one to
//     the other buffer, while the pivot row (final U row k) and the multiplier column
//     (final L column k) go straight to A, and the swaps of the finished parts (rows k, r
//     left of the block, columns k, c above it) are applied in A;
//   * the elimination uses the reference's operations (gaussian_elimination,
//     lu.rs:603-616): the multiplier by division and a - m * u with the product rounded
//     before the subtraction (no FMA), so the factors and both permutations are
//     bit-identical to the reference's for any input, ties included;
//   * each pass also finds its CTA's candidate for the next step's pivot, into the half
//     of the candidate arrays the step's parity selects (a CTA may write step k + 1's
//     candidates while another still reads step k's).
// A zero pivot ends the elimination as the reference's `break` does, leaving the
// remaining trailing block in A as it stands.
#include <vector>

#include "dense_ops.cuh"

namespace rl {
namespace {

constexpr int kFpThreads = 256;

template <class T>
__device__ __forceinline__ T mul_rn(T a, T b);
template <>
__device__ __forceinline__ double mul_rn<double>(double a, double b) { return __dmul_rn(a, b); }
template <>
__device__ __forceinline__ float mul_rn<float>(float a, float b) { return __fmul_rn(a, b); }
template <class T>
__device__ __forceinline__ T sub_rn(T a, T b);
template <>
__device__ __forceinline__ double sub_rn<double>(double a, double b) { return __dsub_rn(a, b); }
template <>
__device__ __forceinline__ float sub_rn<float>(float a, float b) { return __fsub_rn(a, b); }

// Candidates are (key, row-major index) pairs. The key of v is |v|'s bit pattern, which
// orders like |v| for non-NaN values, so the comparisons run on the integer units; a
// NaN is never a candidate (|NaN| > x is false in the reference's scan). The larger key
// wins, the smaller index on ties.
template <class T>
struct AbsKey;
template <>
struct AbsKey<double> {
    static __device__ __forceinline__ unsigned long long of(double v, bool &nan) {
        const unsigned long long k = (unsigned long long)__double_as_longlong(v) & 0x7fffffffffffffffULL;
        nan = k > 0x7ff0000000000000ULL;
        return k;
    }
};
template <>
struct AbsKey<float> {
    static __device__ __forceinline__ unsigned long long of(float v, bool &nan) {
        const unsigned k = __float_as_uint(v) & 0x7fffffffu;
        nan = k > 0x7f800000u;
        return k;
    }
};

constexpr long long kNone = LLONG_MAX;

template <class T>
__device__ __forceinline__ void cand_take(unsigned long long &bk, long long &bi, T v, long long i) {
    bool nan;
    const unsigned long long k = AbsKey<T>::of(v, nan);
    if (!nan && (k > bk || (k == bk && i < bi))) {
        bk = k;
        bi = i;
    }
}

__device__ __forceinline__ void cand_combine(unsigned long long &bk, long long &bi, unsigned long long k2, long long i2) {
    if (i2 != kNone && (bi == kNone || k2 > bk || (k2 == bk && i2 < bi))) {
        bk = k2;
        bi = i2;
    }
}

// Block-wide candidate; every thread gets it. Uses sk / si [warps].
__device__ void block_cand(unsigned long long &bk, long long &bi, unsigned long long *sk, long long *si) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1)
        cand_combine(bk, bi, __shfl_xor_sync(0xffffffffu, bk, o), __shfl_xor_sync(0xffffffffu, bi, o));
    __syncthreads();
    if (lane == 0) {
        sk[warp] = bk;
        si[warp] = bi;
    }
    __syncthreads();
    bk = sk[0];
    bi = si[0];
    for (int w = 1; w < kFpThreads / 32; w++) cand_combine(bk, bi, sk[w], si[w]);
}

constexpr int kFpRowsChunk = 256;  // multipliers staged in shared memory per round
constexpr int kFpUnroll = 8;       // columns per lane with their loads issued together

// One launch, grid-wide barriers between the steps (cooperative launch). Rows of the
// trailing block go to CTAs round-robin (row k + 1 + g + m G to CTA g); a CTA forms its
// rows' multipliers thread-per-row (one division per row, not one per lane), then its
// warps eliminate one row each at a time, the loads of kFpUnroll columns per lane in
// flight together.
template <class T>
__global__ void __launch_bounds__(kFpThreads) full_piv_lu_kernel(T *A, long long lda, int n, T *W0, T *W1,
                                                                 long long ldw, int *piv_r, int *piv_c,
                                                                 unsigned long long *cand_k, long long *cand_i,
                                                                 PanelSync *sync, int *steps,
                                                                 unsigned long long wait_ns) {
    __shared__ unsigned long long sk[kFpThreads / 32];
    __shared__ long long si[kFpThreads / 32];
    __shared__ T s_l[kFpRowsChunk];
    const int G = gridDim.x, g = blockIdx.x;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int gw = g * (kFpThreads / 32) + warp, nw = G * (kFpThreads / 32);
    unsigned phase = 0;
    // candidates of the whole matrix for step 0
    {
        unsigned long long bk = 0;
        long long bi = kNone;
        for (int i = gw; i < n; i += nw)
            for (int j = lane; j < n; j += 32) cand_take(bk, bi, W0[(long long)i * ldw + j], (long long)i * n + j);
        block_cand(bk, bi, sk, si);
        if (threadIdx.x == 0) {
            cand_k[g] = bk;  // half 0: read by step 0
            cand_i[g] = bi;
        }
    }
    if (!grid_barrier(&sync->ctr, (unsigned)(G * (++phase)), &sync->err, wait_ns)) return;
    int k = 0;
    for (; k < n; k++) {
        T *cur = (k & 1) ? W1 : W0, *nxt = (k & 1) ? W0 : W1;
        // the step's pivot, the same in every CTA
        unsigned long long bk = 0;
        long long bi = kNone;
        const int half = (k & 1) * G;
        for (int q = threadIdx.x; q < G; q += kFpThreads)
            cand_combine(bk, bi, ((volatile unsigned long long *)cand_k)[half + q],
                         ((volatile long long *)cand_i)[half + q]);
        block_cand(bk, bi, sk, si);
        int r = k, c = k;
        const T akk = cur[(long long)k * ldw + k];
        if (bi != kNone && !isnan(akk)) {
            r = (int)(bi / n);
            c = (int)(bi - (long long)r * n);
        }
        const T pv = cur[(long long)r * ldw + c];
        if (absT(pv) == T(0)) break;  // lu.rs:408-410 (a NaN pivot goes on, as there)
        if (g == 0 && threadIdx.x == 0) {
            piv_r[k] = r;
            piv_c[k] = c;
        }
        // swaps of the finished parts: rows k, r left of the block, columns k, c above it
        if (r != k)
            for (int j = gw * 32 + lane; j < k; j += nw * 32) {
                const T t = A[(long long)k * lda + j];
                A[(long long)k * lda + j] = A[(long long)r * lda + j];
                A[(long long)r * lda + j] = t;
            }
        if (c != k)
            for (int i = gw * 32 + lane; i < k; i += nw * 32) {
                const T t = A[(long long)i * lda + k];
                A[(long long)i * lda + k] = A[(long long)i * lda + c];
                A[(long long)i * lda + c] = t;
            }
        // the pivot row: final U row k, read through the swaps (row r, columns swapped)
        const T *__restrict__ prow = cur + (long long)r * ldw;
        if (gw == 0)
            for (int j = k + lane; j < n; j += 32) A[(long long)k * lda + j] = prow[j == k ? c : (j == c ? k : j)];
        // this CTA's rows below the pivot: multiplier into A's column k, eliminated row
        // into nxt, candidates for the next step
        bk = 0;
        bi = kNone;
        const int first = k + 1 + g;
        const int cnt = first < n ? (n - first + G - 1) / G : 0;
        for (int m0 = 0; m0 < cnt; m0 += kFpRowsChunk) {
            const int mc = min(kFpRowsChunk, cnt - m0);
            for (int t = threadIdx.x; t < mc; t += kFpThreads) {
                const int i = first + (m0 + t) * G;
                const int src = i == r ? k : i;  // row i after the swap of rows k and r
                const T l = cur[(long long)src * ldw + c] / pv;
                s_l[t] = l;
                A[(long long)i * lda + k] = l;
            }
            __syncthreads();
            for (int t = warp; t < mc; t += kFpThreads / 32) {
                const int i = first + (m0 + t) * G;
                const int src = i == r ? k : i;
                const T *__restrict__ row = cur + (long long)src * ldw;
                T *__restrict__ out = nxt + (long long)i * ldw;
                const T l = s_l[t];
                for (int j0 = k + 1; j0 < n; j0 += 32 * kFpUnroll) {
                    T a[kFpUnroll], u[kFpUnroll];
#pragma unroll
                    for (int q = 0; q < kFpUnroll; q++) {
                        const int j = j0 + lane + 32 * q;
                        const int sj = j == c ? k : j;  // column j after the swap of columns k and c
                        a[q] = j < n ? row[sj] : T(0);
                        u[q] = j < n ? prow[sj] : T(0);
                    }
#pragma unroll
                    for (int q = 0; q < kFpUnroll; q++) {
                        const int j = j0 + lane + 32 * q;
                        if (j < n) {
                            const T v = sub_rn(a[q], mul_rn(l, u[q]));
                            out[j] = v;
                            cand_take(bk, bi, v, (long long)i * n + j);
                        }
                    }
                }
            }
            __syncthreads();  // s_l is refilled by the next round
        }
        block_cand(bk, bi, sk, si);
        if (threadIdx.x == 0) {
            cand_k[G - half + g] = bk;  // the other half: read by step k + 1
            cand_i[G - half + g] = bi;
        }
        if (!grid_barrier(&sync->ctr, (unsigned)(G * (++phase)), &sync->err, wait_ns)) return;
    }
    // after a break the trailing block stays as it stands (in the current buffer)
    if (k < n) {
        const T *cur = (k & 1) ? W1 : W0;
        for (int i = k + gw; i < n; i += nw)
            for (int j = k + lane; j < n; j += 32) A[(long long)i * lda + j] = cur[(long long)i * ldw + j];
    }
    if (g == 0 && threadIdx.x == 0) *steps = k;
}

// Factor the device matrix A (n x n, row stride lda) in place; piv_r / piv_c receive the
// pivot row and column of each step, *steps the number of steps taken (< n after a zero
// pivot). Synchronises the stream.
template <class T>
rl_status full_lu_dev(T *A, long long lda, int n, int *piv_r, int *piv_c, int &steps, cudaStream_t s) {
    NvtxRange nvtx_("rl.full_lu.factor");
    steps = 0;
    if (n <= 0) return RL_OK;
    auto kern = full_piv_lu_kernel<T>;
    int per_sm = 0;
    RL_TRY_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, kFpThreads, 0));
    const long long want = ((long long)n * n + 8LL * kFpThreads - 1) / (8LL * kFpThreads);
    // at most RL_TUNE_FULLPIV_CTAS_PER_SM (3) CTAs per SM: each step ends in a grid
    // barrier and reads every CTA's candidate, and the elimination is bound by the FP64
    // pipe, not by loads in flight
    const int cap = (int)tune(RL_TUNE_FULLPIV_CTAS_PER_SM);
    const int G = (int)std::max<long long>(
        1, std::min<long long>(want, (long long)std::max(1, std::min(per_sm, cap)) * num_sms()));
    DevBuf<T> W0, W1;
    DevBuf<unsigned long long> cv;
    DevBuf<long long> ci;
    DevBuf<PanelSync> sync;
    DevBuf<int> dsteps;
    RL_TRY(W0.alloc((size_t)n * n, s));
    RL_TRY(W1.alloc((size_t)n * n, s));
    RL_TRY(cv.alloc(2 * (size_t)G, s));
    RL_TRY(ci.alloc(2 * (size_t)G, s));
    RL_TRY(sync.alloc(1, s));
    RL_TRY(dsteps.alloc(1, s));
    RL_TRY_CUDA(cudaMemsetAsync(sync.p, 0, sizeof(PanelSync), s));
    RL_TRY_CUDA(cudaMemcpy2DAsync(W0.p, n * sizeof(T), A, lda * sizeof(T), n * sizeof(T), n, cudaMemcpyDeviceToDevice,
                                  s));
    long long ldw = n;
    unsigned long long wns = wait_ns();
    void *args[] = {&A, &lda, &n, &W0.p, &W1.p, &ldw, &piv_r, &piv_c, &cv.p, &ci.p, &sync.p, &dsteps.p, &wns};
    RL_TRY(launch_coop<T>((void *)kern, G, 0, args, s));
    int h[2] = {0, 0};
    RL_TRY_CUDA(cudaMemcpyAsync(&h[0], dsteps.p, sizeof(int), cudaMemcpyDeviceToHost, s));
    RL_TRY_CUDA(cudaMemcpyAsync(&h[1], &sync.p->err, sizeof(int), cudaMemcpyDeviceToHost, s));
    RL_TRY_CUDA(cudaStreamSynchronize(s));
    if (h[1]) return h[1];
    steps = h[0];
    return RL_OK;
}

// The stored form of a swap sequence (PermutationMatrix::swap_rows per step, then
// inverse(), lu.rs:415-429).
void stored_perm(size_t n, const int *piv, int steps, uint64_t *out) {
    std::vector<uint64_t> p(n);
    for (size_t i = 0; i < n; i++) p[i] = i;
    for (int k = 0; k < steps; k++) std::swap(p[k], p[piv[k]]);
    for (size_t i = 0; i < n; i++) out[p[i]] = i;
}

bool valid_perm(size_t n, const uint64_t *perm) {
    std::vector<unsigned char> seen(n, 0);
    for (size_t i = 0; i < n; i++) {
        if (perm[i] >= n || seen[perm[i]]) return false;
        seen[perm[i]] = 1;
    }
    return true;
}

template <class T>
rl_status full_lu_decompose_host(size_t n, T *a, size_t lda, uint64_t *p, uint64_t *q) {
    if (n == 0) return RL_OK;
    if (!a || !p || !q || lda < n || n > (size_t)INT32_MAX) return RL_ERR_INVALID_ARG;
    RL_TRY(ensure_device());
    cudaStream_t s = cudaStreamPerThread;
    DevBuf<T> dA;
    DevBuf<int> dpr, dpc;
    RL_TRY(dA.alloc(n * n, s));
    RL_TRY(dpr.alloc(n, s));
    RL_TRY(dpc.alloc(n, s));
    RL_TRY(copy_h2d(dA.p, n, a, lda, n, n, s));
    int steps = 0;
    RL_TRY(full_lu_dev<T>(dA.p, (long long)n, (int)n, dpr.p, dpc.p, steps, s));
    std::vector<int> pr(n), pc(n);
    RL_TRY(copy_d2h(a, lda, dA.p, n, n, n, s));
    RL_TRY_CUDA(cudaMemcpyAsync(pr.data(), dpr.p, n * sizeof(int), cudaMemcpyDeviceToHost, s));
    RL_TRY_CUDA(cudaMemcpyAsync(pc.data(), dpc.p, n * sizeof(int), cudaMemcpyDeviceToHost, s));
    RL_TRY_CUDA(cudaStreamSynchronize(s));
    stored_perm(n, pr.data(), steps, p);
    stored_perm(n, pc.data(), steps, q);
    return RL_OK;
}

// x = Q U^-1 L^-1 P b per column (lu.rs:480-486): permute (y[p[i]] = b[i]), unit-lower
// and upper solves (DivByZero for |u_ii| < epsilon), then x[i] = y[q[i]]. The last step
// deliberately differs from the reference, which writes x[q[i]] = y[i] (`&self.q * x`,
// lu.rs:485): with A = (L U)[p][:, q] (the reconstruction of lu.rs:903-907) the solution
// is the gather, and the scatter agrees with it only when q is its own inverse (as in
// the reference's 4 x 4 tests); otherwise the reference returns a wrong x.
template <class T>
rl_status full_lu_solve_host(size_t n, size_t nrhs, const T *lu, size_t lda, const uint64_t *p, const uint64_t *q,
                             T *b, size_t ldb) {
    if (n == 0 || nrhs == 0) return RL_OK;
    if (!lu || !p || !q || !b || lda < n || ldb < nrhs || n > (size_t)INT32_MAX || nrhs > (size_t)INT32_MAX)
        return RL_ERR_INVALID_ARG;
    if (!valid_perm(n, p) || !valid_perm(n, q)) return RL_ERR_INVALID_PERMUTATION;
    std::vector<uint64_t> qinv(n);  // x[i] = y[q[i]] is the scatter x[qinv[j]] = y[j]
    for (size_t i = 0; i < n; i++) qinv[q[i]] = i;
    RL_TRY(ensure_device());
    cudaStream_t s = cudaStreamPerThread;
    DevBuf<T> dF, dB, dY;
    DevBuf<uint64_t> dp, dq;
    DevBuf<int> st;
    RL_TRY(dF.alloc(n * n, s));
    RL_TRY(dB.alloc(n * nrhs, s));
    RL_TRY(dY.alloc(n * nrhs, s));
    RL_TRY(dp.alloc(n, s));
    RL_TRY(dq.alloc(n, s));
    RL_TRY(st.alloc(1, s));
    RL_TRY_CUDA(cudaMemsetAsync(st.p, 0, sizeof(int), s));
    RL_TRY(copy_h2d(dF.p, n, lu, lda, n, n, s));
    RL_TRY(copy_h2d(dB.p, nrhs, b, ldb, n, nrhs, s));
    RL_TRY_CUDA(cudaMemcpyAsync(dp.p, p, n * sizeof(uint64_t), cudaMemcpyHostToDevice, s));
    RL_TRY_CUDA(cudaMemcpyAsync(dq.p, qinv.data(), n * sizeof(uint64_t), cudaMemcpyHostToDevice, s));
    const long long tot = (long long)n * nrhs;
    const int g = (int)((tot + 255) / 256);  // one thread per element
    RL_LAUNCH(permute_rows_kernel<T>, g, 256, 0, s, dB.p, (long long)nrhs, dY.p, (long long)nrhs, (int)n, (int)nrhs,
              dp.p);
    RL_TRY(tri_solve_dev<T>(dF.p, (long long)n, (int)n, dY.p, (long long)nrhs, (int)nrhs, 0, st.p, s));
    RL_TRY(tri_solve_dev<T>(dF.p, (long long)n, (int)n, dY.p, (long long)nrhs, (int)nrhs, 2, st.p, s));
    const rl_status r = read_status<T>(st.p, s);
    if (r != RL_OK) return r;
    RL_LAUNCH(permute_rows_kernel<T>, g, 256, 0, s, dY.p, (long long)nrhs, dB.p, (long long)nrhs, (int)n, (int)nrhs,
              dq.p);
    RL_TRY(copy_d2h(b, ldb, dB.p, nrhs, n, nrhs, s));
    RL_TRY_CUDA(cudaStreamSynchronize(s));
    return RL_OK;
}

}  // namespace
}  // namespace rl

using namespace rl;

extern "C" {

rl_status rl_sfull_lu_decompose(size_t n, float *a, size_t lda, uint64_t *p, uint64_t *q) {
    return full_lu_decompose_host<float>(n, a, lda, p, q);
}
rl_status rl_dfull_lu_decompose(size_t n, double *a, size_t lda, uint64_t *p, uint64_t *q) {
    return full_lu_decompose_host<double>(n, a, lda, p, q);
}
rl_status rl_sfull_lu_solve(size_t n, size_t nrhs, const float *lu, size_t lda, const uint64_t *p, const uint64_t *q,
                            float *b, size_t ldb) {
    return full_lu_solve_host<float>(n, nrhs, lu, lda, p, q, b, ldb);
}
rl_status rl_dfull_lu_solve(size_t n, size_t nrhs, const double *lu, size_t lda, const uint64_t *p, const uint64_t *q,
                            double *b, size_t ldb) {
    return full_lu_solve_host<double>(n, nrhs, lu, lda, p, q, b, ldb);
}

}  // extern "C"
