/*
 * rulinalg oracle: a CPU restatement of rulinalg 0.4.2's dense hot path (GEMM,
 * PartialPivLu, Cholesky, HouseholderQr and the substitutions they use), written in
 * plain C. It is TEST INFRASTRUCTURE: only the tests, the smoke check and the CPU
 * baseline leg of the benchmark load it, and only to check or time against it. The
 * CUDA library never links or calls it.
 *
 * Every function cites the reference file:line it follows. The reference itself is
 * Rust and cannot be built here, so the restatement is pinned by the reference's own
 * known-answer tests (tests/golden/).
 *
 * Build: see oracle/Makefile (-O2 -ffp-contract=off, no fast-math).
 */
#define _POSIX_C_SOURCE 200809L
#include <math.h>
#include <float.h>
#include <pthread.h>
#include <stdatomic.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#include "../include/rulinalg_gb300.h"

/* PermutationMatrix::parity (src/matrix/permutation_matrix.rs:216-234) through
 * permute_by_swap (permutation_matrix.rs:479-509): every cycle is resolved by swaps,
 * and each swap flips the parity. Returns 1 for odd. */
int or_perm_parity_odd(size_t n, const uint64_t *perm_in) {
    uint64_t *perm = (uint64_t *)malloc(((n) + 1) * sizeof(uint64_t));
    memcpy(perm, perm_in, n * sizeof(uint64_t));
    int odd = 0;
    for (size_t i = 0; i < n; i++) {
        uint64_t target = perm[i];
        while (i != target) {
            uint64_t new_target = perm[target];
            odd = !odd;
            perm[target] = target;
            target = new_target;
        }
        perm[i] = i;
    }
    free(perm);
    return odd;
}

/* validate_permutation (permutation_matrix.rs:438-470): every entry in [0, n) and
 * unique. Returns RL_OK or RL_ERR_INVALID_PERMUTATION. */
int or_perm_validate(size_t n, const uint64_t *perm) {
    unsigned char *seen = (unsigned char *)calloc(n ? n : 1, 1);
    int st = RL_OK;
    for (size_t i = 0; i < n; i++) {
        if (perm[i] >= n || seen[perm[i]]) {
            st = RL_ERR_INVALID_PERMUTATION;
            break;
        }
        seen[perm[i]] = 1;
    }
    free(seen);
    return st;
}

#define T double
#define SFX d
#define ABS fabs
#define SQRT sqrt
#define EPS DBL_EPSILON
#include "oracle_impl.h"
#undef T
#undef SFX
#undef ABS
#undef SQRT
#undef EPS

#define T float
#define SFX s
#define ABS fabsf
#define SQRT sqrtf
#define EPS FLT_EPSILON
#include "oracle_impl.h"
#undef T
#undef SFX
#undef ABS
#undef SQRT
#undef EPS

/* Helpers for the tests and the CPU baseline: a batch of independent systems solved
 * one after another with the reference algorithms above (the reference has no batched
 * routine; a caller loops). kind[i] = 0: PartialPivLu decompose + solve; 1: Cholesky.
 * a and b are packed, a_off/b_off give each system's start. a is consumed. info[i]
 * receives the status. nthreads > 1 splits the systems over POSIX threads. */

typedef struct {
    size_t lo, hi;
    _Atomic size_t *next; /* shared work counter: systems are taken one at a time */
    const int32_t *n;
    const uint8_t *kind;
    const int64_t *a_off, *b_off;
    double *a, *b;
    int32_t *info;
} or_batch_job;

static void *or_batch_worker(void *arg) {
    or_batch_job *j = (or_batch_job *)arg;
    uint64_t *perm = NULL;
    size_t cap = 0;
    for (;;) {
        const size_t i = atomic_fetch_add(j->next, 1);
        if (i >= j->hi) break;
        size_t n = (size_t)j->n[i];
        double *a = j->a + j->a_off[i];
        double *b = j->b + j->b_off[i];
        int st;
        if (j->kind[i] == 1) {
            st = or_chol_decompose_d(n, a, n);
            if (st == RL_OK) st = or_chol_solve_d(n, a, n, b);
        } else {
            if (n > cap) {
                free(perm);
                cap = n;
                perm = (uint64_t *)malloc(cap * sizeof(uint64_t));
            }
            st = or_lu_decompose_d(n, a, n, perm, NULL);
            if (st == RL_OK) st = or_lu_solve_d(n, a, n, perm, b);
        }
        j->info[i] = st;
    }
    free(perm);
    return NULL;
}

void or_batch_solve_d(size_t count, const int32_t *n, const uint8_t *kind, const int64_t *a_off, double *a,
                      const int64_t *b_off, double *b, int32_t *info, int nthreads) {
    if (nthreads < 1) nthreads = 1;
    if (nthreads > 256) nthreads = 256;
    pthread_t th[256];
    or_batch_job jobs[256];
    _Atomic size_t next = 0; /* the threads take systems one at a time from a shared counter */
    for (int t = 0; t < nthreads; t++) {
        jobs[t].lo = 0;
        jobs[t].hi = count;
        jobs[t].next = &next;
        jobs[t].n = n;
        jobs[t].kind = kind;
        jobs[t].a_off = a_off;
        jobs[t].b_off = b_off;
        jobs[t].a = a;
        jobs[t].b = b;
        jobs[t].info = info;
    }
    if (nthreads == 1) {
        or_batch_worker(&jobs[0]);
        return;
    }
    for (int t = 0; t < nthreads; t++) pthread_create(&th[t], NULL, or_batch_worker, &jobs[t]);
    for (int t = 0; t < nthreads; t++) pthread_join(th[t], NULL);
}
