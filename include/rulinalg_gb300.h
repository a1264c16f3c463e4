/*
 * rulinalg_gb300: C ABI of the GB300 (sm_103a) implementation of rulinalg's dense
 * hot path: `Mul` for Matrix<f32>/Matrix<f64> (GEMM) and the factor-and-solve
 * routines PartialPivLu, Cholesky and HouseholderQr with their solve/det/inverse.
 *
 * Conventions (all entry points):
 *  - Matrices are row-major exactly like rulinalg's Matrix<T> (src/matrix/mod.rs:45-49)
 *    and MatrixSlice (src/matrix/mod.rs:58-64): element (i, j) at ptr[i * ld + j], where
 *    `ld` is the row stride (>= number of columns).
 *  - Plain entry points take HOST pointers (a Rust Vec<T>'s buffer); the library copies
 *    to the GPU, computes there and copies back. `_dev` entry points take DEVICE pointers
 *    and a cudaStream_t passed as `void *` (NULL = the calling thread's default stream)
 *    and are asynchronous unless stated otherwise.
 *  - Permutations are the reference's stored form: a uint64_t per row, "row i -> perm[i]"
 *    (PermutationMatrix{perm: Vec<usize>}, src/matrix/permutation_matrix.rs:102-111).
 *  - Every function returns an rl_status. There is no CPU fallback: without a usable
 *    GPU every compute entry point returns RL_ERR_NO_DEVICE.
 *  - Thread safety: every call may come from any host thread; host-pointer calls run on
 *    the per-thread default stream and block until their result is on the host.
 */
#ifndef RULINALG_GB300_H
#define RULINALG_GB300_H

#include <stddef.h>
#include <stdint.h>

#if defined(__GNUC__)
#define RL_API __attribute__((visibility("default")))
#else
#define RL_API
#endif

#ifdef __cplusplus
extern "C" {
#endif

/* Status codes. 1..6 map one to one onto rulinalg's ErrorKind (src/error.rs:21-34);
 * RL_ERR_SHAPE is returned where the reference panics on a dimension assert!
 * (e.g. src/matrix/mat_mul.rs:21, src/matrix/decomposition/lu.rs:165,232). */
typedef int rl_status;
#define RL_OK 0
#define RL_ERR_INVALID_ARG 1
#define RL_ERR_DECOMP_FAILURE 2
#define RL_ERR_ALGEBRA_FAILURE 3
#define RL_ERR_DIV_BY_ZERO 4
#define RL_ERR_SCALAR_CONVERSION 5
#define RL_ERR_INVALID_PERMUTATION 6
#define RL_ERR_SHAPE 16
#define RL_ERR_CUDA 32
#define RL_ERR_NO_DEVICE 33
#define RL_ERR_OUT_OF_MEMORY 34
#define RL_ERR_TIMEOUT 35
#define RL_ERR_NOT_CONVERGED 36
#define RL_ERR_BUSY 37 /* the serving loop's queue is full (backpressure); submit again later */

/* Human-readable text for a status (static storage). */
RL_API const char *rl_status_string(rl_status status);
/* ABI version: major * 10000 + minor * 100 + patch. */
RL_API int rl_version(void);
/* RL_OK when a CUDA device of compute capability 10.3 is usable by this process. */
RL_API rl_status rl_device_check(void);
/* Number of kernel launches this library has issued in this process (all threads). */
RL_API uint64_t rl_launch_count(void);

/* -------------------------------------------------------------------- tunables -- */
/* Process-wide settings of the library (no counterpart in the reference, which has no
 * launch shapes or device waits). rl_tune_set stores a value for the calls that start
 * after it (a batched plan takes its launch shape and upload chunks when it is created,
 * and its wait limit when its launch sequence is recorded); rl_tune_get reads it back.
 * The batched autotuner (rulinalg_gb300/autotune.py) writes the RL_TUNE_BATCH_* and
 * RL_TUNE_UPLOAD_CHUNKS values it selects. Out-of-range values return
 * RL_ERR_INVALID_ARG and change nothing. */
#define RL_TUNE_WAIT_TIMEOUT_NS 1     /* limit of every device-side wait, ns: [1e6, 1e10], default 1e9 */
#define RL_TUNE_PANEL_CLUSTER_MAX 2   /* largest thread-block cluster of the blocked LU / QR panels: [0, 16],
                                         default 16 (capped by the device); 0: always the cooperative grid */
#define RL_TUNE_BATCH_CTAS_PER_SM 3   /* CTAs per SM of the batched launch: [0, 8], 0 (default): the
                                         kernel's occupancy; larger values are capped by it */
#define RL_TUNE_BATCH_WARP_COST 4     /* systems of cost n^3 (x2 for LU) up to this take the one-warp path in
                                         a largest-first batch: [0, 32768], default 32768 */
#define RL_TUNE_UPLOAD_CHUNKS 5       /* chunks of the host path's overlapped upload: [1, 256], default 32 */
#define RL_TUNE_MIXED_REFINE_STEPS 6   /* single-system mixed solves: iterative-refinement steps before
                                         GMRES-IR takes over: [1, 30], default 30 (LAPACK dsgesv's limit) */
#define RL_TUNE_LU_OUTER_NB 7         /* FP32 blocked LU (n > 512): width of the outer column blocks whose
                                         trailing update is one K = width GEMM on the tensor cores: [-1, 4096],
                                         rounded down to a multiple of 64; 0..63: one level, every 64-column
                                         panel updates the whole trailing matrix; -1 (default): one level for
                                         n < 6144, 1024-column blocks from there (measured best on GB300) */
#define RL_TUNE_MIXED_SWEEP_INV 8     /* single-system mixed solves, up to 128 right-hand sides: the refinement's
                                         FP32 triangular sweeps apply each 64 x 64 diagonal block as its
                                         precomputed inverse (a product) instead of a 64-step substitution:
                                         [0, 1], default 1 (1-7% faster at n = 4096-16384, same refinement
                                         steps within one) */
#define RL_TUNE_PANEL_LOOKAHEAD 9     /* blocked LU panels on a cluster: column j + 1's pivot search and
                                         push overlap the rest of column j's elimination (bit-identical
                                         factors; measured not faster on GB300): [0, 1], default 0 */
#define RL_TUNE_FULLPIV_CTAS_PER_SM 10 /* FullPivLu's cooperative launch: CTAs per SM, [1, 3], default 3 (each
                                          elimination step ends in a grid barrier over all of them) */
#define RL_TUNE_TEST_WITHHOLD_CHUNK 100 /* tests only: the host batched path never sets this chunk's arrival
                                           flag, so its wait runs out (RL_ERR_TIMEOUT): [-1, 255], default -1 */
#define RL_TUNE_TEST_WITHHOLD_SWEEP_BLOCK 101 /* tests only: the one-launch triangular sweep never
                                                 publishes this 64-row block: [-1, 2^30], default -1 */
RL_API rl_status rl_tune_set(int key, int64_t value);
RL_API rl_status rl_tune_get(int key, int64_t *value);

/* ------------------------------------------------------------------------ GEMM -- */
/* C = A * B with A m x k, B k x n, C m x n; alpha = 1, beta = 0.
 * Replaces the matrixmultiply::{sgemm,dgemm} calls of mat_mul_general!
 * (src/matrix/mat_mul.rs:33-43 and :57-67): rsa/rsb are the row strides that
 * `row_stride()` supplies there, rsc = n for a new Matrix. */
RL_API rl_status rl_sgemm(size_t m, size_t k, size_t n, const float *a, size_t rsa, const float *b, size_t rsb,
                   float *c, size_t rsc);
RL_API rl_status rl_dgemm(size_t m, size_t k, size_t n, const double *a, size_t rsa, const double *b, size_t rsb,
                   double *c, size_t rsc);
RL_API rl_status rl_sgemm_dev(size_t m, size_t k, size_t n, const float *a, size_t rsa, const float *b, size_t rsb,
                       float *c, size_t rsc, void *stream);
RL_API rl_status rl_dgemm_dev(size_t m, size_t k, size_t n, const double *a, size_t rsa, const double *b,
                       size_t rsb, double *c, size_t rsc, void *stream);

/* ---------------------------------------------------------------- PartialPivLu -- */
/* PartialPivLu::decompose (src/matrix/decomposition/lu.rs:163-194): A (n x n, in place)
 * becomes the compact LU (unit L strictly below the diagonal, U on and above it) and
 * perm receives the stored permutation p with P A = L U. Pivoting takes the first
 * largest |a[i,k]|; a pivot with |p| < epsilon returns RL_ERR_DIV_BY_ZERO. */
RL_API rl_status rl_slu_decompose(size_t n, float *a, size_t lda, uint64_t *perm);
RL_API rl_status rl_dlu_decompose(size_t n, double *a, size_t lda, uint64_t *perm);
/* PartialPivLu::solve (lu.rs:231-244) for nrhs right-hand sides at once: B is n x nrhs
 * (row-major, row stride ldb; nrhs = 1, ldb = 1 is a Vector<T>) and is overwritten by X.
 * RL_ERR_DIV_BY_ZERO when |u_ii| < epsilon (src/matrix/mod.rs:333-336). */
RL_API rl_status rl_slu_solve(size_t n, size_t nrhs, const float *lu, size_t lda, const uint64_t *perm, float *b,
                       size_t ldb);
RL_API rl_status rl_dlu_solve(size_t n, size_t nrhs, const double *lu, size_t lda, const uint64_t *perm, double *b,
                       size_t ldb);
/* PartialPivLu::inverse (lu.rs:251-285). */
RL_API rl_status rl_slu_inverse(size_t n, const float *lu, size_t lda, const uint64_t *perm, float *inv, size_t ldi);
RL_API rl_status rl_dlu_inverse(size_t n, const double *lu, size_t lda, const uint64_t *perm, double *inv,
                         size_t ldi);
/* PartialPivLu::det (lu.rs:291-300): prod(diag U) * det(P). */
RL_API rl_status rl_slu_det(size_t n, const float *lu, size_t lda, const uint64_t *perm, float *det);
RL_API rl_status rl_dlu_det(size_t n, const double *lu, size_t lda, const uint64_t *perm, double *det);

/* ------------------------------------------------------------------- FullPivLu -- */
/* FullPivLu::decompose (src/matrix/decomposition/lu.rs:385-430): complete pivoting, A (n
 * x n, in place) becomes the compact LU and p, q receive the stored row and column
 * permutations (P A Q = L U, the reference's stored forms, lu.rs:425-429). Each pivot is
 * the largest |a| of the trailing block, the first in row-major order on ties
 * (select_pivot, lu.rs:364-382); a zero pivot ends the elimination (the reference's
 * `break`, never an error). The elimination uses the reference's operations (multiplier
 * by division, a - m * u without FMA), so LU, p and q are bit-identical to the
 * reference's on every input. */
RL_API rl_status rl_sfull_lu_decompose(size_t n, float *a, size_t lda, uint64_t *p, uint64_t *q);
RL_API rl_status rl_dfull_lu_decompose(size_t n, double *a, size_t lda, uint64_t *p, uint64_t *q);
/* FullPivLu::solve (lu.rs:480-486) for nrhs right-hand sides: B (n x nrhs, row stride
 * ldb) is overwritten by X = Q U^-1 L^-1 P B; |u_ii| < epsilon returns RL_ERR_DIV_BY_ZERO
 * (back_substitution, src/matrix/mod.rs:333-336), an invalid p or q
 * RL_ERR_INVALID_PERMUTATION. One deliberate difference: the reference applies q by
 * scatter (x[q[i]] = y[i], `&self.q * x` at lu.rs:485), which solves A x = b only when q
 * is its own inverse; this applies it by gather (x[i] = y[q[i]]), the solution for the
 * factorisation A = (L U)[p][:, q] that the reference's own tests reconstruct. */
RL_API rl_status rl_sfull_lu_solve(size_t n, size_t nrhs, const float *lu, size_t lda, const uint64_t *p,
                                   const uint64_t *q, float *b, size_t ldb);
RL_API rl_status rl_dfull_lu_solve(size_t n, size_t nrhs, const double *lu, size_t lda, const uint64_t *p,
                                   const uint64_t *q, double *b, size_t ldb);

/* -------------------------------------------------------------------- Cholesky -- */
/* Cholesky::decompose (src/matrix/decomposition/cholesky.rs:116-169): the lower triangle
 * of A (in place) becomes L with A = L L^T; the strict upper triangle is neither read nor
 * written. |d| < epsilon or d < 0 on the diagonal returns RL_ERR_DECOMP_FAILURE. */
RL_API rl_status rl_scholesky_decompose(size_t n, float *a, size_t lda);
RL_API rl_status rl_dcholesky_decompose(size_t n, double *a, size_t lda);
/* Cholesky::solve (cholesky.rs:194-202) for n x nrhs B, overwritten by X. */
RL_API rl_status rl_scholesky_solve(size_t n, size_t nrhs, const float *l, size_t ldl, float *b, size_t ldb);
RL_API rl_status rl_dcholesky_solve(size_t n, size_t nrhs, const double *l, size_t ldl, double *b, size_t ldb);
/* Cholesky::inverse (cholesky.rs:209-234) and Cholesky::det (cholesky.rs:175-180). */
RL_API rl_status rl_scholesky_inverse(size_t n, const float *l, size_t ldl, float *inv, size_t ldi);
RL_API rl_status rl_dcholesky_inverse(size_t n, const double *l, size_t ldl, double *inv, size_t ldi);
RL_API rl_status rl_scholesky_det(size_t n, const float *l, size_t ldl, float *det);
RL_API rl_status rl_dcholesky_det(size_t n, const double *l, size_t ldl, double *det);

/* --------------------------------------------------------------- HouseholderQr -- */
/* HouseholderQr::decompose (src/matrix/decomposition/qr.rs:180-223): A (m x n, in place)
 * becomes R on and above the diagonal and the Householder vectors v_j (implicit leading
 * 1) below it; tau receives min(m, n) scale factors. Infallible in the reference. */
RL_API rl_status rl_sqr_decompose(size_t m, size_t n, float *a, size_t lda, float *tau);
RL_API rl_status rl_dqr_decompose(size_t m, size_t n, double *a, size_t lda, double *tau);
/* HouseholderComposition::first_k_columns (householder.rs:235-268): the first k columns
 * of Q (m x k) from the compact storage; k = m is QR::unpack's Q (qr.rs:278-296), k = n
 * is unpack_thin's Q1 (qr.rs:250-275). */
RL_API rl_status rl_sqr_first_k_columns(size_t m, size_t n, const float *qr, size_t lda, const float *tau, size_t k,
                                 float *q, size_t ldq);
RL_API rl_status rl_dqr_first_k_columns(size_t m, size_t n, const double *qr, size_t lda, const double *tau,
                                 size_t k, double *q, size_t ldq);
/* HouseholderComposition::left_multiply_into (householder.rs:203-227): X <- Q X for the
 * m x q matrix X (row stride ldx), Q = H_0 H_1 ... H_{p-1} of the compact storage from
 * rl_*qr_decompose (m x n, p = min(m, n) reflectors, tau as there), the reflectors
 * applied from the last to the first, without forming Q. */
RL_API rl_status rl_sqr_q_apply(size_t m, size_t n, const float *qr, size_t lda, const float *tau, size_t q, float *x,
                                size_t ldx);
RL_API rl_status rl_dqr_q_apply(size_t m, size_t n, const double *qr, size_t lda, const double *tau, size_t q,
                                double *x, size_t ldx);
/* X <- Q^T X, the reflectors from the first to the last: the q1^T * b step of the
 * least-squares composition (qr.rs:250-275 unpack_thin, then &Matrix * &Vector,
 * src/matrix/impl_ops.rs:298-314, on the transpose) without forming Q. */
RL_API rl_status rl_sqr_q_apply_t(size_t m, size_t n, const float *qr, size_t lda, const float *tau, size_t q,
                                  float *x, size_t ldx);
RL_API rl_status rl_dqr_q_apply_t(size_t m, size_t n, const double *qr, size_t lda, const double *tau, size_t q,
                                  double *x, size_t ldx);
/* BaseMatrix::solve_u_triangular (src/matrix/base/mod.rs:1015-1024, back_substitution
 * src/matrix/mod.rs:318-357) and solve_l_triangular (base/mod.rs:1058-1067,
 * forward_substitution src/matrix/mod.rs:363-398): T X = B for an n x n triangle (the
 * other triangle's values are ignored), B n x nrhs overwritten by X; |t_ii| < epsilon returns
 * RL_ERR_DIV_BY_ZERO as the reference's Err(DivByZero). */
RL_API rl_status rl_strsv_upper(size_t n, size_t nrhs, const float *u, size_t ldu, float *b, size_t ldb);
RL_API rl_status rl_dtrsv_upper(size_t n, size_t nrhs, const double *u, size_t ldu, double *b, size_t ldb);
RL_API rl_status rl_strsv_lower(size_t n, size_t nrhs, const float *l, size_t ldl, float *b, size_t ldb);
RL_API rl_status rl_dtrsv_lower(size_t n, size_t nrhs, const double *l, size_t ldl, double *b, size_t ldb);
/* Least squares min ||A x - b||_2 for m >= n (no routine in the reference; it is the
 * composition unpack_thin -> q1^T b -> r1.solve_u_triangular, qr.rs:250-275,
 * src/matrix/base/mod.rs:1015-1024). A is consumed, b has m entries, x receives n.
 * RL_ERR_DIV_BY_ZERO when |r_ii| < epsilon. */
RL_API rl_status rl_sqr_least_squares(size_t m, size_t n, float *a, size_t lda, const float *b, float *x);
RL_API rl_status rl_dqr_least_squares(size_t m, size_t n, double *a, size_t lda, const double *b, double *x);

/* ---------------------------------------------------- Matrix::solve/inverse/det -- */
/* Matrix::solve (src/matrix/impl_mat.rs:354-356): decompose + solve; A is consumed. */
RL_API rl_status rl_smatrix_solve(size_t n, float *a, size_t lda, float *b);
RL_API rl_status rl_dmatrix_solve(size_t n, double *a, size_t lda, double *b);
/* Matrix::inverse (impl_mat.rs:386-388). A is consumed. */
RL_API rl_status rl_smatrix_inverse(size_t n, float *a, size_t lda, float *inv, size_t ldi);
RL_API rl_status rl_dmatrix_inverse(size_t n, double *a, size_t lda, double *inv, size_t ldi);
/* Matrix::det (impl_mat.rs:407-427): closed forms for diagonal, 2x2 and 3x3, else
 * PartialPivLu with a decomposition failure mapped to 0. A is consumed. */
RL_API rl_status rl_smatrix_det(size_t n, float *a, size_t lda, float *det);
RL_API rl_status rl_dmatrix_det(size_t n, double *a, size_t lda, double *det);

/* ------------------------------------------------------------- batched solves -- */
/* Thousands of independent systems A_i x_i = b_i (n_i <= 512, any mix of sizes and of
 * PartialPivLu / Cholesky) solved in one launch. The reference has no batched routine:
 * this replaces a caller's loop of `PartialPivLu::decompose(a)?.solve(b)`
 * (lu.rs:163-244) or `Cholesky::decompose(a)?.solve(b)` (cholesky.rs:116-202).
 *
 * Packed layout: system i's matrix occupies n_i * n_i elements (row-major, row stride
 * n_i) starting at a[a_offset[i]]; its right-hand side and solution occupy n_i elements
 * at b[b_offset[i]] and x[b_offset[i]] (rl_batch_plan_layout gives the offsets).
 *
 * Precision of a plan:
 *   RL_PREC_FP64  f64 systems, factor and solve in FP64 (the plain GPU path).
 *   RL_PREC_MIXED f64 systems, factor in FP32, FP64 iterative refinement (residual,
 *                 update and backward-error stopping test in FP64) to f64 accuracy;
 *                 systems whose FP32 factor fails or whose refinement stalls are
 *                 refactored in FP64 in the same launch sequence (iters = -1).
 *   RL_PREC_FP32  f32 systems (Matrix<f32>), factor and solve in FP32.
 * Per system: info (rl_status: DivByZero / DecompFailure as the reference would
 * return), iters (refinement steps) and berr = ||b - A x||_inf /
 * (||A||_inf ||x||_inf + ||b||_inf) computed in FP64. iters/berr may be NULL. */
#define RL_KIND_LU 0
#define RL_KIND_CHOLESKY 1
#define RL_PREC_FP64 0
#define RL_PREC_MIXED 1
#define RL_PREC_FP32 2
typedef struct rl_batch_plan rl_batch_plan;
RL_API rl_status rl_batch_plan_create(rl_batch_plan **plan, size_t count, const int32_t *n, const uint8_t *kind,
                               int precision);
RL_API rl_status rl_batch_plan_destroy(rl_batch_plan *plan);
RL_API rl_status rl_batch_plan_layout(const rl_batch_plan *plan, int64_t *a_offset, int64_t *b_offset, int64_t *a_total,
                               int64_t *b_total);
/* Device pointers; asynchronous on `stream`; the launch sequence is captured once as a
 * CUDA graph per set of pointers and replayed. */
RL_API rl_status rl_dbatch_solve_dev(rl_batch_plan *plan, const double *a, const double *b, double *x, int32_t *info,
                              int32_t *iters, double *berr, void *stream);
RL_API rl_status rl_sbatch_solve_dev(rl_batch_plan *plan, const float *a, const float *b, float *x, int32_t *info,
                              int32_t *iters, double *berr, void *stream);
/* Host pointers: copy in, solve, copy out; blocking. */
RL_API rl_status rl_dbatch_solve(rl_batch_plan *plan, const double *a, const double *b, double *x, int32_t *info,
                          int32_t *iters, double *berr);
RL_API rl_status rl_sbatch_solve(rl_batch_plan *plan, const float *a, const float *b, float *x, int32_t *info,
                          int32_t *iters, double *berr);

/* ---------------------------------------------- mixed-precision single systems -- */
/* One (typically large) f64 system A X = B, n x n, nrhs columns (row-major, strides).
 * The replaced reference call is `PartialPivLu::decompose(a)?.solve(b)` (lu.rs:163-244)
 * or `Cholesky::decompose(a)?.solve(b)` (cholesky.rs:116-202) per column.
 * rl_dsolve_mixed*: FP32 factor on the GPU (kind = RL_KIND_LU / RL_KIND_CHOLESKY), FP64
 * residual, update and backward-error stopping test (||r|| <= sqrt(n) u ||A|| ||x||);
 * when plain refinement stalls or diverges, GMRES-IR (restarted FP64 GMRES
 * left-preconditioned by the FP32 factors); when that fails too, or the FP32 factor
 * breaks down, an FP64 refactor. rl_dsolve_fp64_dev: the plain all-FP64 GPU solve.
 * info (may be NULL) reports the refinement steps, GMRES iterations, the path taken and
 * the max normwise backward error over the columns. The _dev forms take device
 * pointers and synchronise the stream (the host reads the stopping test). */
#define RL_PATH_REFINEMENT 0
#define RL_PATH_GMRES 1
#define RL_PATH_FP64 2
typedef struct rl_solve_info {
    int32_t iters;
    int32_t gmres_iters;
    int32_t path;
    int32_t reserved;
    double berr;
} rl_solve_info;
RL_API rl_status rl_dsolve_mixed_dev(size_t n, size_t nrhs, int kind, const double *a, size_t lda, const double *b,
                                     size_t ldb, double *x, size_t ldx, rl_solve_info *info, void *stream);
RL_API rl_status rl_dsolve_mixed(size_t n, size_t nrhs, int kind, const double *a, size_t lda, const double *b,
                                 size_t ldb, double *x, size_t ldx, rl_solve_info *info);
RL_API rl_status rl_dsolve_fp64_dev(size_t n, size_t nrhs, int kind, const double *a, size_t lda, const double *b,
                                    size_t ldb, double *x, size_t ldx, rl_solve_info *info, void *stream);

/* Resident factorisations for repeated solves with new right-hand sides. The replaced
 * reference pattern is one `PartialPivLu::decompose(a)?` / `Cholesky::decompose(a)?`
 * (lu.rs:163-194, cholesky.rs:116-169) followed by many `solve(b)` calls (lu.rs:231-244,
 * cholesky.rs:194-202); here the factor stays on the device. rl_factor_create copies the
 * device matrix A (n x n, row stride lda) and factors it in FP32 (mixed precision, as
 * rl_dsolve_mixed); rl_factor_solve gives f64-accurate X for device B (n x nrhs) with
 * FP64 refinement / GMRES-IR, building and keeping the FP64 factor if a solve needs it.
 * Device pointers; both synchronise `stream` (the host reads the stopping test). Solves
 * against one factor from several threads are serialised. */
typedef struct rl_factor rl_factor;
RL_API rl_status rl_factor_create(rl_factor **factor, int kind, size_t n, const double *a, size_t lda, void *stream);
RL_API rl_status rl_factor_solve(rl_factor *factor, size_t nrhs, const double *b, size_t ldb, double *x, size_t ldx,
                                 rl_solve_info *info, void *stream);
RL_API rl_status rl_factor_destroy(rl_factor *factor);

/* Least squares min ||A x - b||_2 (m >= n, one right-hand side) in mixed precision: the
 * f64 result of HouseholderQr::decompose(a) and the composition Q^T b, R x = (Q^T b)[0:n]
 * (qr.rs:171-275; rl_dqr_least_squares is the all-FP64 drop-in). Householder QR of the
 * FP32 copy of A, then the corrected semi-normal equations refined in FP64 until the
 * correction is below 4u ||x|| (or stalls below 1e3 u ||x||, the floor left by the FP64
 * residual when b is far from range(A)); anything else falls back to FP64 QR. info->berr is ||A^T r|| / (||A|| (||A|| ||x|| +
 * ||b||)) with inf-norms. The _dev form takes device pointers and synchronises the
 * stream. */
RL_API rl_status rl_dlstsq_mixed_dev(size_t m, size_t n, const double *a, size_t lda, const double *b, double *x,
                                     rl_solve_info *info, void *stream);
RL_API rl_status rl_dlstsq_mixed(size_t m, size_t n, const double *a, size_t lda, const double *b, double *x,
                                 rl_solve_info *info);

/* ---------------------------------------------------------------------- serving -- */
/* A request loop in front of the GPU solvers (no counterpart in the reference, which is
 * a single-threaded library): clients submit requests from any thread and wait on
 * tickets; worker threads with their own CUDA streams batch the small LU / Cholesky
 * requests that are waiting into one mixed-precision launch (continuous batching), run
 * the others alone, keep factors resident on request (re-solves with new right-hand
 * sides reuse them), and admit work only while its device-memory footprint fits the
 * budget. Answers are f64-accurate (backward error as for RL_PREC_MIXED); QR least
 * squares is FP64 Householder QR of [A | b]. Host buffers a, b, x must stay valid until
 * the ticket completes. */
#define RL_REQ_LU 0
#define RL_REQ_CHOLESKY 1
#define RL_REQ_LSTSQ 2
#define RL_REQ_RESOLVE 3
typedef struct rl_server rl_server;
typedef struct rl_server_config {
    size_t hbm_budget_bytes; /* 0: 80% of the free device memory after start-up */
    int workers;             /* worker threads / CUDA streams (0: 8); worker 0 serves only batchable requests */
    int max_batch;           /* systems per batched launch (0: 4096) */
    int small_n;             /* largest n sent to the batched kernel (0: 512) */
    int max_pending;         /* requests submitted but not finished, at most (0: no limit); beyond it
                                rl_server_submit returns RL_ERR_BUSY and counts a rejection */
} rl_server_config;
typedef struct rl_request {
    int kind;        /* RL_REQ_* */
    int retain;      /* LU / Cholesky: keep the factor resident; its handle comes back in rl_result.factor */
    uint64_t factor; /* RL_REQ_RESOLVE: handle of a resident factor */
    size_t m, n;     /* A is m x n (m = n, or 0, except for least squares) */
    const double *a; /* host, row-major m x n (unused for RL_REQ_RESOLVE) */
    const double *b; /* host, m entries */
    double *x;       /* host, n entries, written on completion */
} rl_request;
typedef struct rl_result {
    rl_status status;
    int32_t iters;     /* refinement steps */
    int32_t path;      /* RL_PATH_* */
    int32_t reserved;
    double berr;       /* normwise backward error (0 for least squares) */
    uint64_t factor;   /* resident factor handle (retain / re-solve) */
    double queue_us;   /* submit -> a worker took it */
    double latency_us; /* submit -> result on the host */
} rl_result;
typedef struct rl_server_stats {
    uint64_t submitted, completed, failed, batches, batched_requests;
    uint64_t bytes_in_use, bytes_peak, bytes_budget, resident_factors;
    double p50_us, p99_us, mean_us, solves_per_s;
    uint64_t rejected; /* submissions refused with RL_ERR_BUSY */
} rl_server_stats;
RL_API rl_status rl_server_create(const rl_server_config *cfg, rl_server **server);
/* Non-blocking; RL_ERR_OUT_OF_MEMORY when the request can never fit the budget, RL_ERR_BUSY
 * when max_pending requests are already in the server. */
RL_API rl_status rl_server_submit(rl_server *server, const rl_request *req, uint64_t *ticket);
/* Blocks until the ticket completes (timeout_s < 0: no limit); the ticket is consumed. */
RL_API rl_status rl_server_wait(rl_server *server, uint64_t ticket, double timeout_s, rl_result *result);
RL_API rl_status rl_server_release_factor(rl_server *server, uint64_t factor);
RL_API rl_status rl_server_stats_get(rl_server *server, rl_server_stats *stats);
RL_API rl_status rl_server_reset_stats(rl_server *server);
/* Load replay: submits reqs[i] at arrival_s[i] seconds after the call (a Poisson trace,
 * say), then waits for all of them; results[i] receives each outcome (status
 * RL_ERR_BUSY for a request refused by backpressure). */
RL_API rl_status rl_server_replay(rl_server *server, size_t count, const double *arrival_s, const rl_request *reqs,
                                  rl_result *results);
/* Drains the admitted requests, releases resident factors and stops the workers. */
RL_API rl_status rl_server_destroy(rl_server *server);

/* ------------------------------------------------- solve without any allocation -- */
/* No counterpart in the reference. For callers that cannot allocate device memory (a
 * serving process that reserves all GPU memory at start-up and forbids allocation
 * afterwards, or a host framework whose own pool owns the device memory): one f64 system
 * A x = b with n <= 512, solved like an RL_PREC_MIXED batch of one (FP32 factor, FP64
 * refinement, FP64 refactor fallback; kind = RL_KIND_LU or RL_KIND_CHOLESKY). Device
 * pointers; asynchronous on `stream`; A is n x n row-major (row stride n). info / iters /
 * berr receive one value each (iters, berr may be NULL).
 * All scratch memory is one fixed array inside the library (about 3 MiB, held on every
 * GPU that loads the library until the process exits); no cudaMalloc or other
 * allocation happens. n > 512 returns RL_ERR_INVALID_ARG. The first call on a device
 * looks up the array's device address (cudaGetSymbolAddress) and sets the kernels'
 * shared-memory limits, so make that first call before any stream capture. Calls share
 * the array: calls that overlap on the GPU race on it and must be ordered by the caller
 * (for example by issuing them on one stream). */
RL_API rl_status rl_dsolve_mixed_noalloc_dev(size_t n, int kind, const double *a, const double *b, double *x,
                                             int32_t *info, int32_t *iters, double *berr, void *stream);

#ifdef __cplusplus
}
#endif
#endif /* RULINALG_GB300_H */
