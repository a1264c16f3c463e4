/*
 * Type-generic body of the oracle. Included twice by rulinalg_oracle.c, once with
 * T=double/SFX=d and once with T=float/SFX=s. Test infrastructure only: a CPU
 * restatement of rulinalg 0.4.2's algorithms, operation by operation, so that the
 * CUDA library can be checked against it. Nothing in the product links this.
 *
 * Layout convention throughout: row-major, element (i, j) at a[i * lda + j], exactly
 * like rulinalg's Matrix<T>{rows, cols, data} (src/matrix/mod.rs:45-49) and
 * MatrixSlice{ptr, rows, cols, row_stride} (src/matrix/mod.rs:58-64).
 *
 * Floating point: the file is compiled with -ffp-contract=off and without fast-math,
 * because rustc never fuses a*b+c into an FMA; every expression below keeps the
 * reference's evaluation order.
 */
#define CAT2(a, b) a##_##b
#define CAT(a, b) CAT2(a, b)
#define FN(name) CAT(name, SFX)

/* utils::dot (src/utils.rs:20-51): eight partial sums over blocks of 8, combined as
 * s + p0 + p4, + p1 + p5, + p2 + p6, + p3 + p7, then a sequential scalar tail. */
T FN(or_dot)(size_t len, const T *u, const T *v) {
    T s = 0, p0 = 0, p1 = 0, p2 = 0, p3 = 0, p4 = 0, p5 = 0, p6 = 0, p7 = 0;
    size_t i = 0;
    while (len - i >= 8) {
        p0 = p0 + u[i + 0] * v[i + 0];
        p1 = p1 + u[i + 1] * v[i + 1];
        p2 = p2 + u[i + 2] * v[i + 2];
        p3 = p3 + u[i + 3] * v[i + 3];
        p4 = p4 + u[i + 4] * v[i + 4];
        p5 = p5 + u[i + 5] * v[i + 5];
        p6 = p6 + u[i + 6] * v[i + 6];
        p7 = p7 + u[i + 7] * v[i + 7];
        i += 8;
    }
    s = s + p0 + p4;
    s = s + p1 + p5;
    s = s + p2 + p6;
    s = s + p3 + p7;
    for (; i < len; i++) s = s + u[i] * v[i];
    return s;
}

/* Generic-T GEMM path of mat_mul_general! (src/matrix/mat_mul.rs:77-92): i-k-j loop,
 * new_data[i*r+j] = new_data[i*r+j] + a[i,k] * b[k,j], starting from zero. The f32/f64
 * branches of the reference call the external matrixmultiply crate (^0.1.13,
 * Cargo.toml:19), whose summation order is not in the reference tree; this loop stands
 * in for it and GEMM parity is therefore normwise. */
void FN(or_gemm)(size_t p, size_t q, size_t r, const T *a, size_t lda, const T *b, size_t ldb, T *c,
                 size_t ldc) {
    for (size_t i = 0; i < p; i++)
        for (size_t j = 0; j < r; j++) c[i * ldc + j] = 0;
    for (size_t i = 0; i < p; i++)
        for (size_t k = 0; k < q; k++) {
            const T aik = a[i * lda + k];
            for (size_t j = 0; j < r; j++) c[i * ldc + j] = c[i * ldc + j] + aik * b[k * ldb + j];
        }
}

/* &Matrix * &Vector (src/matrix/impl_ops.rs:298-314): one utils::dot per row. */
void FN(or_matvec)(size_t m, size_t n, const T *a, size_t lda, const T *x, T *y) {
    for (size_t i = 0; i < m; i++) y[i] = FN(or_dot)(n, a + i * lda, x);
}

/* Euclidean norm of a matrix (src/norm/mod.rs:108-119): sum over rows of dot(row,row),
 * then sqrt, i.e. the Frobenius norm with rulinalg's summation order. */
T FN(or_norm_frobenius)(size_t m, size_t n, const T *a, size_t lda) {
    T s = 0;
    for (size_t i = 0; i < m; i++) s = s + FN(or_dot)(n, a + i * lda, a + i * lda);
    return SQRT(s);
}

/* ---------------------------------------------------------------- PartialPivLu -- */

/* gaussian_elimination (src/matrix/decomposition/lu.rs:603-616): multiplier by division,
 * then lu[i,j] = lu[i,j] - mult * lu[index,j] (no FMA). */
static void FN(gaussian_elimination)(size_t n, T *lu, size_t lda, size_t index) {
    const T piv_val = lu[index * lda + index];
    for (size_t i = index + 1; i < n; i++) {
        const T mult = lu[i * lda + index] / piv_val;
        lu[i * lda + index] = mult;
        for (size_t j = index + 1; j < n; j++)
            lu[i * lda + j] = lu[i * lda + j] - mult * lu[index * lda + j];
    }
}

/* PartialPivLu::decompose (src/matrix/decomposition/lu.rs:163-194).
 * Pivot search: start from the diagonal, take a later row only if |a[i,k]| > |max|
 * strictly (the first maximum wins). Failure: |max| < epsilon -> DivByZero. The swaps
 * are applied to the whole row (src/matrix/base/mod.rs:1394-1418) and to the
 * permutation (src/matrix/permutation_matrix.rs:132-134); the stored permutation is the
 * inverse of the accumulated one (lu.rs:192, permutation_matrix.rs:137-148).
 * perm_out (optional) receives that stored form. gap_out (optional) receives, per
 * step, (|max| - |second largest|) / |max| among the candidates: the margin by which
 * the pivot choice is unique. Returns RL_OK or RL_ERR_DIV_BY_ZERO (then perm_out is
 * untouched and `a` holds the partial factorisation, as the consumed matrix would). */
int FN(or_lu_decompose)(size_t n, T *a, size_t lda, uint64_t *perm_out, T *gap_out) {
    uint64_t *p = (uint64_t *)malloc(((n) + 1) * sizeof(uint64_t));
    for (size_t i = 0; i < n; i++) p[i] = i;
    for (size_t index = 0; index < n; index++) {
        size_t curr_max_idx = index;
        T curr_max = a[index * lda + index];
        for (size_t i = index + 1; i < n; i++) {
            if (ABS(a[i * lda + index]) > ABS(curr_max)) {
                curr_max = a[i * lda + index];
                curr_max_idx = i;
            }
        }
        if (gap_out) {
            T second = 0;
            for (size_t i = index; i < n; i++)
                if (i != curr_max_idx && ABS(a[i * lda + index]) > second) second = ABS(a[i * lda + index]);
            gap_out[index] = ABS(curr_max) > 0 ? (ABS(curr_max) - second) / ABS(curr_max) : 0;
        }
        if (ABS(curr_max) < EPS) {
            free(p);
            return RL_ERR_DIV_BY_ZERO;
        }
        if (curr_max_idx != index) {
            for (size_t j = 0; j < n; j++) {
                T t = a[index * lda + j];
                a[index * lda + j] = a[curr_max_idx * lda + j];
                a[curr_max_idx * lda + j] = t;
            }
            uint64_t t = p[index];
            p[index] = p[curr_max_idx];
            p[curr_max_idx] = t;
        }
        FN(gaussian_elimination)(n, a, lda, index);
    }
    if (perm_out) /* inverse: inv[perm[i]] = i */
        for (size_t i = 0; i < n; i++) perm_out[p[i]] = i;
    free(p);
    return RL_OK;
}

/* lu_forward_substitution (lu.rs:624-642): unit lower L, sequential fold
 * sum = sum + l[i,j] * x[j] for j < i, then x[i] = x[i] - sum. */
static void FN(lu_forward_substitution)(size_t n, const T *lu, size_t lda, T *x) {
    for (size_t i = 1; i < n; i++) {
        T adj = 0;
        for (size_t j = 0; j < i; j++) adj = adj + lu[i * lda + j] * x[j];
        x[i] = x[i] - adj;
    }
}

/* back_substitution (src/matrix/mod.rs:318-357): from the last row up,
 * DivByZero if |u_ii| < epsilon, x[i] = (x[i] - dot(u[i, i+1..], x[i+1..])) / u_ii. */
int FN(or_back_substitution)(size_t n, const T *u, size_t ldu, T *x) {
    for (size_t ii = n; ii-- > 0;) {
        const T divisor = u[ii * ldu + ii];
        if (ABS(divisor) < EPS) return RL_ERR_DIV_BY_ZERO;
        const T d = FN(or_dot)(n - ii - 1, u + ii * ldu + ii + 1, x + ii + 1);
        x[ii] = (x[ii] - d) / divisor;
    }
    return RL_OK;
}

/* forward_substitution (src/matrix/mod.rs:363-398): DivByZero if |l_ii| < epsilon,
 * x[i] = (x[i] - dot(l[i, 0..i], x[0..i])) / l_ii. */
int FN(or_forward_substitution)(size_t n, const T *l, size_t ldl, T *x) {
    for (size_t i = 0; i < n; i++) {
        const T divisor = l[i * ldl + i];
        if (ABS(divisor) < EPS) return RL_ERR_DIV_BY_ZERO;
        const T d = FN(or_dot)(i, l + i * ldl, x);
        x[i] = (x[i] - d) / divisor;
    }
    return RL_OK;
}

/* PartialPivLu::solve (lu.rs:231-244): y = P b with buffer[perm[i]] = b[i]
 * (permutation_matrix.rs:369-382), then unit-lower forward and upper back substitution.
 * b is overwritten by x. */
int FN(or_lu_solve)(size_t n, const T *lu, size_t lda, const uint64_t *perm, T *b) {
    T *y = (T *)malloc(((n) + 1) * sizeof(T));
    for (size_t i = 0; i < n; i++) y[perm[i]] = b[i];
    FN(lu_forward_substitution)(n, lu, lda, y);
    int st = FN(or_back_substitution)(n, lu, lda, y);
    if (st == RL_OK) memcpy(b, y, n * sizeof(T));
    free(y);
    return st;
}

/* PartialPivLu::inverse (lu.rs:251-285): one solve per unit vector e_i, written to
 * column i. */
int FN(or_lu_inverse)(size_t n, const T *lu, size_t lda, const uint64_t *perm, T *inv, size_t ldi) {
    T *e = (T *)malloc(((n) + 1) * sizeof(T));
    for (size_t i = 0; i < n; i++) {
        for (size_t j = 0; j < n; j++) e[j] = 0;
        e[i] = 1;
        int st = FN(or_lu_solve)(n, lu, lda, perm, e);
        if (st != RL_OK) {
            free(e);
            return st;
        }
        for (size_t j = 0; j < n; j++) inv[j * ldi + i] = e[j];
    }
    free(e);
    return RL_OK;
}

/* PartialPivLu::det (lu.rs:291-300): fold(1, x * y) over diag(U), times det(P) from
 * the permutation's parity (permutation_matrix.rs:216-260). */
T FN(or_lu_det)(size_t n, const T *lu, size_t lda, const uint64_t *perm) {
    T u_det = 1;
    for (size_t i = 0; i < n; i++) u_det = u_det * lu[i * lda + i];
    T p_det = or_perm_parity_odd(n, perm) ? (T)0 - (T)1 : (T)1;
    return p_det * u_det;
}

/* Matrix::det (src/matrix/impl_mat.rs:407-427): diagonal matrices fold their diagonal,
 * 2x2 and 3x3 use closed forms, everything else goes through PartialPivLu and maps a
 * decomposition failure to zero. `a` is consumed (overwritten). */
T FN(or_matrix_det)(size_t n, T *a, size_t lda) {
    int is_diag = 1;
    for (size_t i = 0; i < n && is_diag; i++)
        for (size_t j = 0; j < n; j++)
            if (i != j && a[i * lda + j] != 0) {
                is_diag = 0;
                break;
            }
#define A_(i, j) a[(i) * lda + (j)]
    if (is_diag) {
        T d = 1;
        for (size_t i = 0; i < n; i++) d = d * A_(i, i);
        return d;
    } else if (n == 2) {
        return (A_(0, 0) * A_(1, 1)) - (A_(0, 1) * A_(1, 0));
    } else if (n == 3) {
        return (A_(0, 0) * A_(1, 1) * A_(2, 2)) + (A_(0, 1) * A_(1, 2) * A_(2, 0)) +
               (A_(0, 2) * A_(1, 0) * A_(2, 1)) - (A_(0, 0) * A_(1, 2) * A_(2, 1)) -
               (A_(0, 1) * A_(1, 0) * A_(2, 2)) - (A_(0, 2) * A_(1, 1) * A_(2, 0));
    }
#undef A_
    uint64_t *perm = (uint64_t *)malloc(((n) + 1) * sizeof(uint64_t));
    T d = 0;
    if (FN(or_lu_decompose)(n, a, lda, perm, NULL) == RL_OK) d = FN(or_lu_det)(n, a, lda, perm);
    free(perm);
    return d;
}

/* ------------------------------------------------------------------ FullPivLu -- */

/* FullPivLu::decompose (src/matrix/decomposition/lu.rs:385-430) with select_pivot
 * (lu.rs:364-382): at step `index` the pivot is the largest |a| of the trailing block,
 * scanned row by row from (index, index) with a strict > (the first maximum in row-major
 * order wins; a NaN never wins); a zero pivot ends the elimination (`break`, never an
 * error). Whole rows and whole columns are swapped (src/matrix/base/mod.rs:1394-1418,
 * :1446-1463), the swaps recorded in p and q (permutation_matrix.rs:132-134), then
 * gaussian_elimination (lu.rs:603-616). p_out / q_out (optional) receive the stored
 * forms, the inverses of the accumulated permutations (lu.rs:425-429); piv_r / piv_c
 * (optional) the pivot row and column of each step, -1 from a break on. */
void FN(or_full_lu_decompose)(size_t n, T *a, size_t lda, uint64_t *p_out, uint64_t *q_out, int64_t *piv_r,
                              int64_t *piv_c) {
    uint64_t *p = (uint64_t *)malloc(((n) + 1) * sizeof(uint64_t));
    uint64_t *q = (uint64_t *)malloc(((n) + 1) * sizeof(uint64_t));
    for (size_t i = 0; i < n; i++) p[i] = q[i] = i;
    for (size_t i = 0; i < n; i++) {
        if (piv_r) piv_r[i] = -1;
        if (piv_c) piv_c[i] = -1;
    }
    for (size_t index = 0; index < n; index++) {
        size_t pr = index, pc = index;
        T pv = a[index * lda + index];
        for (size_t row = index; row < n; row++)
            for (size_t col = index; col < n; col++) {
                const T val = a[row * lda + col];
                if (ABS(val) > ABS(pv)) {
                    pv = val;
                    pr = row;
                    pc = col;
                }
            }
        if (ABS(pv) == 0) break;
        if (piv_r) piv_r[index] = (int64_t)pr;
        if (piv_c) piv_c[index] = (int64_t)pc;
        if (pr != index)
            for (size_t j = 0; j < n; j++) {
                const T t = a[index * lda + j];
                a[index * lda + j] = a[pr * lda + j];
                a[pr * lda + j] = t;
            }
        if (pc != index)
            for (size_t i = 0; i < n; i++) {
                const T t = a[i * lda + index];
                a[i * lda + index] = a[i * lda + pc];
                a[i * lda + pc] = t;
            }
        uint64_t t = p[index];
        p[index] = p[pr];
        p[pr] = t;
        t = q[index];
        q[index] = q[pc];
        q[pc] = t;
        FN(gaussian_elimination)(n, a, lda, index);
    }
    if (p_out)
        for (size_t i = 0; i < n; i++) p_out[p[i]] = i;
    if (q_out)
        for (size_t i = 0; i < n; i++) q_out[q[i]] = i;
    free(p);
    free(q);
}

/* FullPivLu::solve (lu.rs:480-486) as the reference writes it: y = P b (buffer[p[i]] =
 * b[i], permutation_matrix.rs:369-382), unit-lower forward and upper back substitution
 * (DivByZero when |u_ii| < epsilon), then `&self.q * x` the same way with q
 * (b[q[i]] = y[i]). That last scatter solves A x = b only when q is its own inverse; the
 * tests compare the GPU (which gathers, b[i] = y[q[i]]) with the corrected composition. */
int FN(or_full_lu_solve)(size_t n, const T *lu, size_t lda, const uint64_t *p, const uint64_t *q, T *b) {
    T *y = (T *)malloc(((n) + 1) * sizeof(T));
    for (size_t i = 0; i < n; i++) y[p[i]] = b[i];
    FN(lu_forward_substitution)(n, lu, lda, y);
    const int st = FN(or_back_substitution)(n, lu, lda, y);
    if (st == RL_OK)
        for (size_t i = 0; i < n; i++) b[q[i]] = y[i];
    free(y);
    return st;
}

/* ------------------------------------------------------------------- Cholesky -- */

/* Cholesky::decompose (src/matrix/decomposition/cholesky.rs:116-169), GVL 4.2.5 gaxpy
 * form: for column j, a[k,j] -= dot(a[k,0..j], a[j,0..j]) for k >= j; the diagonal d is
 * checked (|d| < epsilon or d < 0 -> DecompFailure) and column j from the diagonal down
 * is divided by sqrt(d). The strict upper triangle is never read or written. */
int FN(or_chol_decompose)(size_t n, T *a, size_t lda) {
    for (size_t j = 0; j < n; j++) {
        if (j > 0) {
            for (size_t k = j; k < n; k++) {
                const T kj = FN(or_dot)(j, a + k * lda, a + j * lda);
                a[k * lda + j] = a[k * lda + j] - kj;
            }
        }
        const T diagonal = a[j * lda + j];
        if (ABS(diagonal) < EPS) return RL_ERR_DECOMP_FAILURE;
        if (diagonal < 0) return RL_ERR_DECOMP_FAILURE;
        const T divisor = SQRT(diagonal);
        for (size_t k = j; k < n; k++) a[k * lda + j] = a[k * lda + j] / divisor;
    }
    return RL_OK;
}

/* transpose_back_substitution (cholesky.rs:329-361): solves L^T x = b in column-AXPY
 * form: x[i] /= l_ii, then x[j] = x[j] - x[i] * l[i,j] for j < i. */
int FN(or_transpose_back_substitution)(size_t n, const T *l, size_t ldl, T *x) {
    for (size_t ii = n; ii-- > 0;) {
        const T diagonal = l[ii * ldl + ii];
        if (ABS(diagonal) < EPS) return RL_ERR_DIV_BY_ZERO;
        x[ii] = x[ii] / diagonal;
        for (size_t j = 0; j < ii; j++) x[j] = x[j] - x[ii] * l[ii * ldl + j];
    }
    return RL_OK;
}

/* Cholesky::solve (cholesky.rs:194-202). b is overwritten by x. */
int FN(or_chol_solve)(size_t n, const T *l, size_t ldl, T *b) {
    int st = FN(or_forward_substitution)(n, l, ldl, b);
    if (st != RL_OK) return st;
    return FN(or_transpose_back_substitution)(n, l, ldl, b);
}

/* Cholesky::det (cholesky.rs:175-180): (prod of diag(L))^2. */
T FN(or_chol_det)(size_t n, const T *l, size_t ldl) {
    T d = 1;
    for (size_t i = 0; i < n; i++) d = d * l[i * ldl + i];
    return d * d;
}

/* Cholesky::inverse (cholesky.rs:209-234): one solve per unit vector. */
int FN(or_chol_inverse)(size_t n, const T *l, size_t ldl, T *inv, size_t ldi) {
    T *e = (T *)malloc(((n) + 1) * sizeof(T));
    for (size_t i = 0; i < n; i++) {
        for (size_t j = 0; j < n; j++) e[j] = 0;
        e[i] = 1;
        int st = FN(or_chol_solve)(n, l, ldl, e);
        if (st != RL_OK) {
            free(e);
            return st;
        }
        for (size_t j = 0; j < n; j++) inv[j * ldi + i] = e[j];
    }
    free(e);
    return RL_OK;
}

/* ------------------------------------------------------------- HouseholderQr -- */

/* HouseholderReflection::compute (src/matrix/decomposition/householder.rs:32-89), in
 * place on x (length m): sigma = dot(x[1..], x[1..]); sigma == 0 -> tau = 0 and x is left
 * as it is; otherwise |x| = sqrt(x0*x0 + sigma), v0 = x0 + |x| if x0 > 0 else x0 - |x|,
 * tau = 2*v0*v0 / (v0*v0 + sigma), x[0] = v0 and every element is divided by v0. */
T FN(or_house_compute)(size_t m, T *x) {
    if (m == 0) return 0;
    const T sigma = FN(or_dot)(m - 1, x + 1, x + 1);
    const T x0 = x[0];
    if (sigma == 0) return 0;
    const T x_norm = SQRT(x0 * x0 + sigma);
    const T v0 = x0 > 0 ? x0 + x_norm : x0 - x_norm;
    const T two = 2;
    const T tau = two * v0 * v0 / (v0 * v0 + sigma);
    x[0] = v0;
    for (size_t i = 0; i < m; i++) x[i] = x[i] / v0;
    return tau;
}

/* buffered_left_multiply_into (householder.rs:100-130): u = A^T v via transpose_gemv
 * (src/internal_utils.rs:28-45: y = 0, then y += v[j] * row_j for every row, i.e.
 * y[c] = y[c] + v[j] * a[j,c]) and A <- A - tau v u^T via ger (internal_utils.rs:67-83:
 * row_i[c] = row_i[c] + (alpha * v[i]) * u[c] with alpha = -tau). A is m x n. */
void FN(or_house_apply)(size_t m, size_t n, T *a, size_t lda, const T *v, T tau, T *u) {
    for (size_t c = 0; c < n; c++) u[c] = 0;
    for (size_t j = 0; j < m; j++) {
        const T s = v[j];
        for (size_t c = 0; c < n; c++) u[c] = u[c] + s * a[j * lda + c];
    }
    const T alpha = -tau;
    for (size_t i = 0; i < m; i++) {
        const T s = alpha * v[i];
        for (size_t c = 0; c < n; c++) a[i * lda + c] = a[i * lda + c] + s * u[c];
    }
}

/* HouseholderQr::decompose (src/matrix/decomposition/qr.rs:180-223), GVL Alg. 5.2.1:
 * for j < min(m, n) the reflector of column j (rows j..m) is computed, applied to the
 * bottom-right block, and its v[1..] stored below the diagonal (store_in_col,
 * householder.rs:151-162). tau has min(m, n) entries. */
void FN(or_qr_decompose)(size_t m, size_t n, T *a, size_t lda, T *tau) {
    const size_t p = m < n ? m : n;
    T *v = (T *)malloc(((m) + 1) * sizeof(T));
    T *u = (T *)malloc(((n) + 1) * sizeof(T));
    for (size_t j = 0; j < p; j++) {
        T *blk = a + j * lda + j;
        const size_t mj = m - j, nj = n - j;
        for (size_t i = 0; i < mj; i++) v[i] = blk[i * lda];
        const T t = FN(or_house_compute)(mj, v);
        FN(or_house_apply)(mj, nj, blk, lda, v, t, u);
        for (size_t i = 1; i < mj; i++) blk[i * lda] = v[i];
        tau[j] = t;
    }
    free(v);
    free(u);
}

/* HouseholderComposition::first_k_columns (householder.rs:235-268): start from the
 * first k columns of the m x m identity and apply reflectors j = min(p, k)-1 .. 0 to the
 * block [j.., j..], each reflector loaded from column j of the storage with an implicit
 * leading 1 (load_house_from_col, householder.rs:271-284). qr is m x n, q is m x k. */
void FN(or_qr_first_k_columns)(size_t m, size_t n, const T *qr, size_t lda, const T *tau, size_t k, T *q,
                               size_t ldq) {
    const size_t p = m < n ? m : n;
    const size_t jmax = p < k ? p : k;
    for (size_t i = 0; i < m; i++)
        for (size_t c = 0; c < k; c++) q[i * ldq + c] = (i == c) ? 1 : 0;
    T *v = (T *)malloc(((m) + 1) * sizeof(T));
    T *u = (T *)malloc(((k) + 1) * sizeof(T));
    for (size_t jj = jmax; jj-- > 0;) {
        const size_t mj = m - jj;
        for (size_t i = 0; i < mj; i++) v[i] = qr[(jj + i) * lda + jj];
        v[0] = 1;
        FN(or_house_apply)(mj, k - jj, q + jj * ldq + jj, ldq, v, tau[jj], u);
    }
    free(v);
    free(u);
}

/* HouseholderComposition::left_multiply_into (householder.rs:203-227): X <- Q X for an
 * m x q matrix X, reflectors applied from the last to the first. */
void FN(or_qr_q_left_multiply)(size_t m, size_t n, const T *qr, size_t lda, const T *tau, size_t q, T *x,
                               size_t ldx) {
    const size_t p = m < n ? m : n;
    T *v = (T *)malloc(((m) + 1) * sizeof(T));
    T *u = (T *)malloc(((q) + 1) * sizeof(T));
    for (size_t jj = p; jj-- > 0;) {
        const size_t mj = m - jj;
        for (size_t i = 0; i < mj; i++) v[i] = qr[(jj + i) * lda + jj];
        v[0] = 1;
        FN(or_house_apply)(mj, q, x + jj * ldx, ldx, v, tau[jj], u);
    }
    free(v);
    free(u);
}

/* X <- Q^T X: the same reflectors as or_qr_q_left_multiply (buffered_left_multiply_into,
 * householder.rs:100-130, each loaded by load_house_from_col, :271-284) applied from the
 * first to the last. The reference has no such method; Q^T X is what the least-squares
 * composition computes as q1^T * b (qr.rs:250-275 then impl_ops.rs:298-314). */
void FN(or_qr_qt_left_multiply)(size_t m, size_t n, const T *qr, size_t lda, const T *tau, size_t q, T *x,
                                size_t ldx) {
    const size_t p = m < n ? m : n;
    T *v = (T *)malloc(((m) + 1) * sizeof(T));
    T *u = (T *)malloc(((q) + 1) * sizeof(T));
    for (size_t jj = 0; jj < p; jj++) {
        const size_t mj = m - jj;
        for (size_t i = 0; i < mj; i++) v[i] = qr[(jj + i) * lda + jj];
        v[0] = 1;
        FN(or_house_apply)(mj, q, x + jj * ldx, ldx, v, tau[jj], u);
    }
    free(v);
    free(u);
}

/* Least squares through the reference's public API (no such routine exists in the
 * reference): ThinQR {q1, r1} = HouseholderQr::decompose(A).unpack_thin()
 * (qr.rs:250-275, m > n), c = q1^T * b via &Matrix * &Vector (impl_ops.rs:298-314, one
 * utils::dot per row of the transposed q1), x = r1.solve_u_triangular(c)
 * (src/matrix/base/mod.rs:1015-1024 -> back_substitution). a (m x n, m > n) is consumed;
 * x receives n values. */
int FN(or_qr_lstsq)(size_t m, size_t n, T *a, size_t lda, const T *b, T *x) {
    T *tau = (T *)malloc(((n) + 1) * sizeof(T));
    T *q1 = (T *)malloc(((m * n) + 1) * sizeof(T));
    T *q1t = (T *)malloc(((m * n) + 1) * sizeof(T));
    T *r1 = (T *)malloc(((n * n) + 1) * sizeof(T));
    FN(or_qr_decompose)(m, n, a, lda, tau);
    FN(or_qr_first_k_columns)(m, n, a, lda, tau, n, q1, n);
    for (size_t i = 0; i < n; i++)
        for (size_t j = 0; j < n; j++) r1[i * n + j] = j >= i ? a[i * lda + j] : 0;
    for (size_t i = 0; i < m; i++)
        for (size_t j = 0; j < n; j++) q1t[j * m + i] = q1[i * n + j];
    FN(or_matvec)(n, m, q1t, m, b, x);
    int st = FN(or_back_substitution)(n, r1, n, x);
    free(tau);
    free(q1);
    free(q1t);
    free(r1);
    return st;
}

/* ------------------------------------------------- threaded variants (tests) -- */
/* For the configurations' full sizes (n = 1024 .. 4096) the tests split the work of the
 * functions above over POSIX threads. Each element of the result sees exactly the
 * operations of the single-threaded function, in the same order (the threads only
 * partition rows, or right-hand-side columns), so the results are bit-identical to it. */

typedef struct {
    size_t p, q, r, lda, ldb, ldc, lo, hi;
    const T *a, *b;
    T *c;
} FN(or_gemm_job);

static void *FN(or_gemm_worker)(void *arg) {
    FN(or_gemm_job) *j = (FN(or_gemm_job) *)arg;
    FN(or_gemm)(j->hi - j->lo, j->q, j->r, j->a + j->lo * j->lda, j->lda, j->b, j->ldb, j->c + j->lo * j->ldc,
                j->ldc);
    return NULL;
}

/* or_gemm with the rows of C split over `threads` threads (i-k-j per row as there). */
void FN(or_gemm_mt)(size_t p, size_t q, size_t r, const T *a, size_t lda, const T *b, size_t ldb, T *c, size_t ldc,
                    int threads) {
    if (threads < 1) threads = 1;
    if (threads > 256) threads = 256;
    if ((size_t)threads > p) threads = p ? (int)p : 1;
    pthread_t th[256];
    FN(or_gemm_job) jobs[256];
    for (int t = 0; t < threads; t++) {
        FN(or_gemm_job) j = {p, q, r, lda, ldb, ldc, p * (size_t)t / (size_t)threads,
                             p * (size_t)(t + 1) / (size_t)threads, a, b, c};
        jobs[t] = j;
    }
    for (int t = 1; t < threads; t++) pthread_create(&th[t], NULL, FN(or_gemm_worker), &jobs[t]);
    FN(or_gemm_worker)(&jobs[0]);
    for (int t = 1; t < threads; t++) pthread_join(th[t], NULL);
}

typedef struct {
    size_t n, lda;
    T *a;
    uint64_t *p;
    T *gap;
    int tid, threads, status;
    volatile int *stop;
    pthread_barrier_t *bar;
} FN(or_lu_job);

/* One thread of or_lu_decompose_mt: thread 0 runs the pivot search, the failure check
 * and the row swap of each step (lu.rs:169-190) exactly as or_lu_decompose does; after a
 * barrier every thread eliminates its contiguous share of the rows below the pivot with
 * gaussian_elimination's operations (lu.rs:603-616); a second barrier ends the step. */
static void *FN(or_lu_worker)(void *arg) {
    FN(or_lu_job) *j = (FN(or_lu_job) *)arg;
    const size_t n = j->n, lda = j->lda;
    T *a = j->a;
    for (size_t index = 0; index < n; index++) {
        if (j->tid == 0) {
            size_t curr_max_idx = index;
            T curr_max = a[index * lda + index];
            for (size_t i = index + 1; i < n; i++) {
                if (ABS(a[i * lda + index]) > ABS(curr_max)) {
                    curr_max = a[i * lda + index];
                    curr_max_idx = i;
                }
            }
            if (j->gap) {
                T second = 0;
                for (size_t i = index; i < n; i++)
                    if (i != curr_max_idx && ABS(a[i * lda + index]) > second) second = ABS(a[i * lda + index]);
                j->gap[index] = ABS(curr_max) > 0 ? (ABS(curr_max) - second) / ABS(curr_max) : 0;
            }
            if (ABS(curr_max) < EPS) {
                *j->stop = 1;
                j->status = RL_ERR_DIV_BY_ZERO;
            } else if (curr_max_idx != index) {
                for (size_t c = 0; c < n; c++) {
                    T t = a[index * lda + c];
                    a[index * lda + c] = a[curr_max_idx * lda + c];
                    a[curr_max_idx * lda + c] = t;
                }
                uint64_t t = j->p[index];
                j->p[index] = j->p[curr_max_idx];
                j->p[curr_max_idx] = t;
            }
        }
        pthread_barrier_wait(j->bar);
        if (*j->stop) break;
        const size_t rows = n - index - 1;
        const size_t lo = index + 1 + rows * (size_t)j->tid / (size_t)j->threads;
        const size_t hi = index + 1 + rows * (size_t)(j->tid + 1) / (size_t)j->threads;
        const T piv_val = a[index * lda + index];
        for (size_t i = lo; i < hi; i++) {
            const T mult = a[i * lda + index] / piv_val;
            a[i * lda + index] = mult;
            for (size_t c = index + 1; c < n; c++) a[i * lda + c] = a[i * lda + c] - mult * a[index * lda + c];
        }
        pthread_barrier_wait(j->bar);
    }
    return NULL;
}

/* or_lu_decompose with the elimination rows of every step split over `threads`
 * threads; bit-identical to it (same pivots, same factors, same status). */
int FN(or_lu_decompose_mt)(size_t n, T *a, size_t lda, uint64_t *perm_out, T *gap_out, int threads) {
    if (threads < 1) threads = 1;
    if (threads > 256) threads = 256;
    if (threads == 1 || n < 64) return FN(or_lu_decompose)(n, a, lda, perm_out, gap_out);
    uint64_t *p = (uint64_t *)malloc(((n) + 1) * sizeof(uint64_t));
    for (size_t i = 0; i < n; i++) p[i] = i;
    pthread_t th[256];
    FN(or_lu_job) jobs[256];
    pthread_barrier_t bar;
    volatile int stop = 0;
    pthread_barrier_init(&bar, NULL, (unsigned)threads);
    for (int t = 0; t < threads; t++) {
        FN(or_lu_job) j = {n, lda, a, p, gap_out, t, threads, RL_OK, &stop, &bar};
        jobs[t] = j;
    }
    for (int t = 1; t < threads; t++) pthread_create(&th[t], NULL, FN(or_lu_worker), &jobs[t]);
    FN(or_lu_worker)(&jobs[0]);
    for (int t = 1; t < threads; t++) pthread_join(th[t], NULL);
    pthread_barrier_destroy(&bar);
    const int st = jobs[0].status;
    if (st == RL_OK && perm_out)
        for (size_t i = 0; i < n; i++) perm_out[p[i]] = i;
    free(p);
    return st;
}

typedef struct {
    size_t n, lda, nrhs, ldb, lo, hi;
    const T *lu;
    const uint64_t *perm;
    T *b;
    int status;
} FN(or_solve_job);

static void *FN(or_lu_solve_worker)(void *arg) {
    FN(or_solve_job) *j = (FN(or_solve_job) *)arg;
    T *col = (T *)malloc(((j->n) + 1) * sizeof(T));
    j->status = RL_OK;
    for (size_t c = j->lo; c < j->hi; c++) {
        for (size_t i = 0; i < j->n; i++) col[i] = j->b[i * j->ldb + c];
        const int st = j->perm ? FN(or_lu_solve)(j->n, j->lu, j->lda, j->perm, col)
                               : FN(or_chol_solve)(j->n, j->lu, j->lda, col);
        if (st != RL_OK) {
            j->status = st;
            break;
        }
        for (size_t i = 0; i < j->n; i++) j->b[i * j->ldb + c] = col[i];
    }
    free(col);
    return NULL;
}

/* PartialPivLu::solve (perm != NULL) or Cholesky::solve (perm == NULL) applied to each
 * column of the n x nrhs row-major B (overwritten by X), columns split over threads. */
int FN(or_solve_columns_mt)(size_t n, const T *lu, size_t lda, const uint64_t *perm, size_t nrhs, T *b, size_t ldb,
                            int threads) {
    if (threads < 1) threads = 1;
    if (threads > 256) threads = 256;
    if ((size_t)threads > nrhs) threads = nrhs ? (int)nrhs : 1;
    pthread_t th[256];
    FN(or_solve_job) jobs[256];
    for (int t = 0; t < threads; t++) {
        FN(or_solve_job) j = {n, lda, nrhs, ldb, nrhs * (size_t)t / (size_t)threads,
                              nrhs * (size_t)(t + 1) / (size_t)threads, lu, perm, b, RL_OK};
        jobs[t] = j;
    }
    for (int t = 1; t < threads; t++) pthread_create(&th[t], NULL, FN(or_lu_solve_worker), &jobs[t]);
    FN(or_lu_solve_worker)(&jobs[0]);
    for (int t = 1; t < threads; t++) pthread_join(th[t], NULL);
    for (int t = 0; t < threads; t++)
        if (jobs[t].status != RL_OK) return jobs[t].status;
    return RL_OK;
}

#undef FN
#undef CAT
#undef CAT2
