// Mixed-precision solve of single (large) systems: FP32 factor on the GPU, FP64
// residual / update / backward-error stopping test, GMRES-IR when plain refinement
// stalls (FP64 GMRES left-preconditioned by the FP32 factors), FP64 refactor when that
// fails too. Plus the plain FP64 GPU solve used as its baseline.
#include <mutex>

#include "mixed_ops.cuh"

namespace rl {
namespace {

void fill_info(rl_solve_info *info, const SolveOut &o) {
    if (!info) return;
    info->iters = o.iters;
    info->gmres_iters = o.gmres;
    info->path = o.path;
    info->reserved = 0;
    info->berr = o.berr;
}

rl_status check_args(size_t n, size_t nrhs, int kind, const void *a, size_t lda, const void *b, size_t ldb, const void *x,
                     size_t ldx) {
    if (kind != RL_KIND_LU && kind != RL_KIND_CHOLESKY) return RL_ERR_INVALID_ARG;
    if (n == 0 || nrhs == 0) return RL_OK;
    if (!a || !b || !x || lda < n || ldb < nrhs || ldx < nrhs || n > (size_t)INT32_MAX || nrhs > (size_t)INT32_MAX)
        return RL_ERR_INVALID_ARG;
    return RL_OK;
}

}  // namespace
}  // namespace rl

using namespace rl;

// A resident factorisation: MixedFactor owns its device copy of A (FP64, for the
// residuals), the FP32 factor and, once a solve needed it, the FP64 factor.
struct rl_factor {
    MixedFactor f;
    std::mutex mu;  // solves against one factor are serialised (the FP64 factor is built lazily)
};

extern "C" {

rl_status rl_factor_create(rl_factor **out, int kind, size_t n, const double *a, size_t lda, void *stream) {
    if (!out || (kind != RL_KIND_LU && kind != RL_KIND_CHOLESKY)) return RL_ERR_INVALID_ARG;
    *out = nullptr;
    if (n == 0 || !a || lda < n || n > (size_t)INT32_MAX) return RL_ERR_INVALID_ARG;
    RL_TRY(ensure_device());
    cudaStream_t s = resolve_stream(stream);
    auto *h = new rl_factor();
    const rl_status st = h->f.factor(a, (long long)lda, (int)n, kind, true, s);
    if (st != RL_OK) {
        cudaStreamSynchronize(s);
        delete h;
        return st;
    }
    *out = h;
    return RL_OK;
}

rl_status rl_factor_solve(rl_factor *h, size_t nrhs, const double *b, size_t ldb, double *x, size_t ldx,
                          rl_solve_info *info, void *stream) {
    if (!h) return RL_ERR_INVALID_ARG;
    SolveOut o;
    if (nrhs == 0) {
        fill_info(info, o);
        return RL_OK;
    }
    if (!b || !x || ldb < nrhs || ldx < nrhs || nrhs > (size_t)INT32_MAX) return RL_ERR_INVALID_ARG;
    std::lock_guard<std::mutex> lk(h->mu);
    RL_TRY(h->f.solve(b, (long long)ldb, x, (long long)ldx, (int)nrhs, o, resolve_stream(stream)));
    fill_info(info, o);
    return RL_OK;
}

rl_status rl_factor_destroy(rl_factor *h) {
    if (!h) return RL_OK;
    {
        std::lock_guard<std::mutex> lk(h->mu);
        cudaStreamSynchronize(h->f.home);
        h->f.release();
    }
    delete h;
    return RL_OK;
}

rl_status rl_dsolve_mixed_dev(size_t n, size_t nrhs, int kind, const double *a, size_t lda, const double *b, size_t ldb,
                              double *x, size_t ldx, rl_solve_info *info, void *stream) {
    RL_TRY(check_args(n, nrhs, kind, a, lda, b, ldb, x, ldx));
    SolveOut o;
    if (n == 0 || nrhs == 0) {
        fill_info(info, o);
        return RL_OK;
    }
    RL_TRY(ensure_device());
    RL_TRY(solve_mixed(a, (long long)lda, (int)n, kind, b, (long long)ldb, x, (long long)ldx, (int)nrhs, o,
                       resolve_stream(stream)));
    fill_info(info, o);
    return RL_OK;
}

rl_status rl_dsolve_fp64_dev(size_t n, size_t nrhs, int kind, const double *a, size_t lda, const double *b, size_t ldb,
                             double *x, size_t ldx, rl_solve_info *info, void *stream) {
    RL_TRY(check_args(n, nrhs, kind, a, lda, b, ldb, x, ldx));
    SolveOut o;
    o.path = RL_PATH_FP64;
    if (n == 0 || nrhs == 0) {
        fill_info(info, o);
        return RL_OK;
    }
    RL_TRY(ensure_device());
    cudaStream_t s = resolve_stream(stream);
    RL_TRY(solve_fp64(a, (long long)lda, (int)n, kind, b, (long long)ldb, x, (long long)ldx, (int)nrhs, s));
    if (info) RL_TRY(backward_error_dev(a, (long long)lda, (int)n, x, (long long)ldx, b, (long long)ldb, (int)nrhs, o.berr, s));
    fill_info(info, o);
    return RL_OK;
}

rl_status rl_dsolve_mixed(size_t n, size_t nrhs, int kind, const double *a, size_t lda, const double *b, size_t ldb,
                          double *x, size_t ldx, rl_solve_info *info) {
    RL_TRY(check_args(n, nrhs, kind, a, lda, b, ldb, x, ldx));
    if (n == 0 || nrhs == 0) {
        fill_info(info, SolveOut());
        return RL_OK;
    }
    RL_TRY(ensure_device());
    cudaStream_t s = cudaStreamPerThread;
    DevBuf<double> dA, dB, dX;
    RL_TRY(dA.alloc(n * n, s));
    RL_TRY(dB.alloc(n * nrhs, s));
    RL_TRY(dX.alloc(n * nrhs, s));
    RL_TRY(copy_h2d(dA.p, n, a, lda, n, n, s));
    RL_TRY(copy_h2d(dB.p, nrhs, b, ldb, n, nrhs, s));
    SolveOut o;
    RL_TRY(solve_mixed(dA.p, (long long)n, (int)n, kind, dB.p, (long long)nrhs, dX.p, (long long)nrhs, (int)nrhs, o, s));
    RL_TRY(copy_d2h(x, ldx, dX.p, nrhs, n, nrhs, s));
    RL_TRY_CUDA(cudaStreamSynchronize(s));
    fill_info(info, o);
    return RL_OK;
}

rl_status rl_dlstsq_mixed_dev(size_t m, size_t n, const double *a, size_t lda, const double *b, double *x,
                              rl_solve_info *info, void *stream) {
    if (m < n) return RL_ERR_SHAPE;
    if (n == 0) {
        fill_info(info, SolveOut());
        return RL_OK;
    }
    if (!a || !b || !x || lda < n || m > (size_t)INT32_MAX) return RL_ERR_INVALID_ARG;
    RL_TRY(ensure_device());
    SolveOut o;
    RL_TRY(lstsq_mixed(a, (long long)lda, (int)m, (int)n, b, x, o, resolve_stream(stream)));
    fill_info(info, o);
    return RL_OK;
}

rl_status rl_dlstsq_mixed(size_t m, size_t n, const double *a, size_t lda, const double *b, double *x,
                          rl_solve_info *info) {
    if (m < n) return RL_ERR_SHAPE;
    if (n == 0) {
        fill_info(info, SolveOut());
        return RL_OK;
    }
    if (!a || !b || !x || lda < n || m > (size_t)INT32_MAX) return RL_ERR_INVALID_ARG;
    RL_TRY(ensure_device());
    cudaStream_t s = cudaStreamPerThread;
    DevBuf<double> dA, dB, dX;
    RL_TRY(dA.alloc(m * n, s));
    RL_TRY(dB.alloc(m, s));
    RL_TRY(dX.alloc(n, s));
    RL_TRY(copy_h2d(dA.p, n, a, lda, m, n, s));
    RL_TRY_CUDA(cudaMemcpyAsync(dB.p, b, m * sizeof(double), cudaMemcpyHostToDevice, s));
    SolveOut o;
    RL_TRY(lstsq_mixed(dA.p, (long long)n, (int)m, (int)n, dB.p, dX.p, o, s));
    RL_TRY_CUDA(cudaMemcpyAsync(x, dX.p, n * sizeof(double), cudaMemcpyDeviceToHost, s));
    RL_TRY_CUDA(cudaStreamSynchronize(s));
    fill_info(info, o);
    return RL_OK;
}

}  // extern "C"
