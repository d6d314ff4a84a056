// hhp_precond.cu -- Jacobi-preconditioned BiCGStab as right preconditioning.
//
// The reference carries an ILU preconditioner for gpu_BiCGStab only as commented-out cuSPARSE
// SpSV calls (src/entry/bicgstab_gpu.c:185-201, 238-254); this is the diagonal (Jacobi) form of
// that path. With M = diag(A), BiCGStab solves (A M^-1) y = b and returns x = M^-1 y. A M^-1 is A
// with column j scaled by 1/a_jj, stored once as a derived matrix (A->jac) with its own SpMV
// plan, so an iteration costs exactly what an unpreconditioned one costs. The residual
// b - (A M^-1) y equals b - A x, so the stop test and the reported relative residual are still
// those of the original system.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include "hhp_device.cuh"
#include "hhp_internal.h"

namespace hhp {

namespace {

// dinv[i] = 1 / (sum of row i's diagonal entries); bad[0] = first row (+1) whose diagonal is
// missing, zero or not finite.
__global__ void k_diag_inv(const int *__restrict__ rowptr, const int *__restrict__ col,
                           const double *__restrict__ val, int m, double *dinv, int *bad) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < m; i += gridDim.x * blockDim.x) {
        double d = 0.0;
        for (int k = rowptr[i]; k < rowptr[i + 1]; ++k)
            if (col[k] == i) d += val[k];
        const double r = 1.0 / d;
        if (d == 0.0 || !isfinite(r)) {
            atomicMin(bad, i + 1);
            dinv[i] = 1.0;
        } else {
            dinv[i] = r;
        }
    }
}

// out[k] = val[k] * dinv[row of k]: row i of A scaled by 1/a_ii
__global__ void k_scale_rows(const int *__restrict__ rowptr, const double *__restrict__ val,
                             const double *__restrict__ dinv, int m, double *out) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < m; i += gridDim.x * blockDim.x) {
        const double d = dinv[i];
        for (int k = rowptr[i]; k < rowptr[i + 1]; ++k) out[k] = val[k] * d;
    }
}

__global__ void k_scale_cols(const int *__restrict__ col, const double *__restrict__ val,
                             const double *__restrict__ dinv, int nnz, double *out) {
    for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < nnz; k += gridDim.x * blockDim.x)
        out[k] = val[k] * dinv[col[k]];
}

// x[i] *= s[i] (invert: x[i] /= s[i])
__global__ void k_scale_vec(double *x, const double *__restrict__ s, int n, int invert) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
        x[i] = invert ? x[i] / s[i] : x[i] * s[i];
}

__global__ void k_max_abs_diff(const double *__restrict__ a, const double *__restrict__ b, int n,
                               unsigned long long *out_bits) {
    double mx = 0.0;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
        mx = fmax(mx, fabs(a[i] - b[i]));
    // non-negative doubles order like their bit patterns
    atomicMax(out_bits, static_cast<unsigned long long>(__double_as_longlong(mx)));
}

int grid_for(const hhp_mat *A, long long n) {
    return static_cast<int>(std::max(1LL, std::min((n + 255) / 256, 8LL * A->ctx->num_sms)));
}

}  // namespace

hhp_status ensure_jacobi(hhp_mat *A) {
    if (A->jac) return HHP_OK;
    HHP_TRY(csr_needed(A, "Jacobi preconditioning"));
    if (A->m != A->n) {
        set_error("Jacobi preconditioning needs a square matrix");
        return HHP_ERR_ARG;
    }
    cudaStream_t st = A->ctx->stream;
    double *dinv = nullptr;
    int *bad = nullptr;
    HHP_CUDA(cudaMalloc(&dinv, sizeof(double) * (static_cast<size_t>(A->m) + 4)));
    if (cudaMalloc(&bad, sizeof(int)) != cudaSuccess) {
        cudaFree(dinv);
        set_error("out of device memory for the Jacobi preconditioner");
        return HHP_ERR_OOM;
    }
    const int none = 0x7fffffff;
    hhp_status rc = HHP_OK;
    int first_bad = none;
    if (cudaMemcpyAsync(bad, &none, sizeof(int), cudaMemcpyHostToDevice, st) != cudaSuccess) rc = HHP_ERR_CUDA;
    if (rc == HHP_OK && A->m > 0) {
        k_diag_inv<<<grid_for(A, A->m), 256, 0, st>>>(A->rowptr, A->col, A->val, A->m, dinv, bad);
        if (cudaGetLastError() != cudaSuccess) rc = HHP_ERR_CUDA;
    }
    if (rc == HHP_OK && (cudaMemcpyAsync(&first_bad, bad, sizeof(int), cudaMemcpyDeviceToHost, st) != cudaSuccess ||
                         cudaStreamSynchronize(st) != cudaSuccess))
        rc = HHP_ERR_CUDA;
    cudaFree(bad);
    if (rc == HHP_OK && first_bad != none) {
        set_error("Jacobi preconditioning needs a nonzero finite diagonal; row %d has none", first_bad - 1);
        rc = HHP_ERR_ARG;
    }
    hhp_mat *J = nullptr;
    if (rc == HHP_OK) rc = mat_create_dev(A->ctx, A->m, A->n, A->nnz, &J);
    if (rc == HHP_OK) {
        const size_t rp = static_cast<size_t>(A->m) + 1;
        if (cudaMemcpyAsync(J->rowptr, A->rowptr, sizeof(int) * rp, cudaMemcpyDeviceToDevice, st) != cudaSuccess ||
            (A->nnz > 0 && cudaMemcpyAsync(J->col, A->col, sizeof(int) * static_cast<size_t>(A->nnz),
                                           cudaMemcpyDeviceToDevice, st) != cudaSuccess))
            rc = HHP_ERR_CUDA;
        if (rc == HHP_OK && A->nnz > 0) {
            k_scale_cols<<<grid_for(A, A->nnz), 256, 0, st>>>(A->col, A->val, dinv, A->nnz, J->val);
            if (cudaGetLastError() != cudaSuccess) rc = HHP_ERR_CUDA;
        }
        J->rowptr_host = A->rowptr_host;
    }
    if (rc != HHP_OK) {
        if (rc == HHP_ERR_CUDA) set_error("building the Jacobi-scaled matrix failed: %s",
                                          cudaGetErrorString(cudaGetLastError()));
        if (J) hhp_mat_destroy(J);
        cudaFree(dinv);
        return rc;
    }
    A->jac = J;
    A->dinv = dinv;
    A->dinv_host.resize(static_cast<size_t>(A->m));
    HHP_CUDA(cudaMemcpyAsync(A->dinv_host.data(), dinv, sizeof(double) * static_cast<size_t>(A->m),
                             cudaMemcpyDeviceToHost, st));
    HHP_CUDA(cudaStreamSynchronize(st));
    return HHP_OK;
}

// A with row i scaled by 1/a_ii (A->jac_row), and room for the scaled right-hand side.
hhp_status ensure_jacobi_row(hhp_mat *A) {
    if (A->jac_row) return HHP_OK;
    HHP_TRY(csr_needed(A, "row Jacobi preconditioning"));
    HHP_TRY(ensure_jacobi(A));  // the diagonal (and its checks) come from the column-scaled form
    cudaStream_t st = A->ctx->stream;
    hhp_mat *J = nullptr;
    HHP_TRY(mat_create_dev(A->ctx, A->m, A->n, A->nnz, &J));
    hhp_status rc = HHP_OK;
    if (cudaMemcpyAsync(J->rowptr, A->rowptr, sizeof(int) * (static_cast<size_t>(A->m) + 1), cudaMemcpyDeviceToDevice,
                        st) != cudaSuccess ||
        (A->nnz > 0 && cudaMemcpyAsync(J->col, A->col, sizeof(int) * static_cast<size_t>(A->nnz),
                                       cudaMemcpyDeviceToDevice, st) != cudaSuccess))
        rc = HHP_ERR_CUDA;
    if (rc == HHP_OK && A->m > 0) {
        k_scale_rows<<<grid_for(A, A->m), 256, 0, st>>>(A->rowptr, A->val, A->dinv, A->m, J->val);
        if (cudaGetLastError() != cudaSuccess) rc = HHP_ERR_CUDA;
    }
    double *bs = nullptr;
    if (rc == HHP_OK && cudaMalloc(&bs, sizeof(double) * (static_cast<size_t>(A->n) + 4)) != cudaSuccess) rc = HHP_ERR_OOM;
    if (rc != HHP_OK) {
        set_error("building the row-scaled matrix failed: %s", cudaGetErrorString(cudaGetLastError()));
        hhp_mat_destroy(J);
        cudaFree(bs);
        return rc;
    }
    J->rowptr_host = A->rowptr_host;
    A->jac_row = J;
    A->jac_row_b = bs;
    HHP_CUDA(cudaStreamSynchronize(st));
    return HHP_OK;
}

void release_jacobi(hhp_mat *A) {
    if (A->jac_row) hhp_mat_destroy(A->jac_row);
    A->jac_row = nullptr;
    cudaFree(A->jac_row_b);
    A->jac_row_b = nullptr;
    if (A->jac) hhp_mat_destroy(A->jac);
    A->jac = nullptr;
    cudaFree(A->dinv);
    A->dinv = nullptr;
    A->dinv_host.clear();
}

// x0 -> y0 = M x0, solve (A M^-1) y = b, x = M^-1 y; the error against x_target is taken on x.
hhp_status solve_jacobi(hhp_mat *A, const double *b, double *x, const double *xt, const hhp_solve_opts *o,
                        hhp_solve_info *info, bool host) {
    HHP_TRY(ensure_jacobi(A));
    const int n = A->n;
    hhp_solve_info in{};
    hhp_status rc;
    double err = NAN;
    if (host) {
        std::vector<double> y(x, x + n);
        for (int i = 0; i < n; ++i) y[static_cast<size_t>(i)] /= A->dinv_host[static_cast<size_t>(i)];
        rc = solve_any(A->jac, b, y.data(), nullptr, o, &in, true);
        for (int i = 0; i < n; ++i) x[i] = y[static_cast<size_t>(i)] * A->dinv_host[static_cast<size_t>(i)];
        if (xt) {
            err = 0.0;
            for (int i = 0; i < n; ++i) err = std::max(err, std::fabs(x[i] - xt[i]));
        }
    } else {
        cudaStream_t st = A->ctx->stream;
        if (n > 0) {
            k_scale_vec<<<grid_for(A, n), 256, 0, st>>>(x, A->dinv, n, 1);
            HHP_CUDA(cudaGetLastError());
        }
        rc = solve_any(A->jac, b, x, nullptr, o, &in, false);
        if (n > 0) {
            k_scale_vec<<<grid_for(A, n), 256, 0, st>>>(x, A->dinv, n, 0);
            HHP_CUDA(cudaGetLastError());
        }
        if (xt && n > 0) {
            unsigned long long *d = nullptr, bits = 0;
            HHP_CUDA(cudaMalloc(&d, sizeof(bits)));
            cudaMemsetAsync(d, 0, sizeof(bits), st);
            k_max_abs_diff<<<grid_for(A, n), 256, 0, st>>>(x, xt, n, d);
            cudaMemcpyAsync(&bits, d, sizeof(bits), cudaMemcpyDeviceToHost, st);
            cudaStreamSynchronize(st);
            cudaFree(d);
            std::memcpy(&err, &bits, sizeof(err));
        }
        HHP_CUDA(cudaStreamSynchronize(st));
    }
    in.err_vs_target = err;
    if (info) *info = in;
    return rc;
}

// Row (left) Jacobi: BiCGStab on M^-1 A x = M^-1 b, M = diag(A), which equilibrates rows whose
// scales differ by orders of magnitude (a power-law matrix with diagonals from 1e-9 to 1e5 is
// not solved to 1e-10 unpreconditioned, nor with column scaling). The scaled solve's stop test is
// on M^-1 (b - A x); after each pass the residual of A x = b itself is formed (a zero-iteration
// solve of A from x: the FP64 residual SpMV), and while it is above rtol the scaled solve
// continues from x with its tolerance tightened by the shortfall. The status and the reported
// residual are those of A x = b.
hhp_status solve_jacobi_row(hhp_mat *A, const double *b, double *x, const double *xt, const hhp_solve_opts *o,
                            hhp_solve_info *info, bool host) {
    HHP_TRY(ensure_jacobi_row(A));
    const int n = A->n;
    cudaStream_t st = A->ctx->stream;
    std::vector<double> bs_host;
    const double *bs = nullptr;
    if (host) {
        bs_host.resize(static_cast<size_t>(n));
        for (int i = 0; i < n; ++i) bs_host[static_cast<size_t>(i)] = b[i] * A->dinv_host[static_cast<size_t>(i)];
        bs = bs_host.data();
    } else {
        HHP_CUDA(cudaMemcpyAsync(A->jac_row_b, b, sizeof(double) * static_cast<size_t>(n), cudaMemcpyDeviceToDevice, st));
        if (n > 0) {
            k_scale_vec<<<grid_for(A, n), 256, 0, st>>>(A->jac_row_b, A->dinv, n, 0);
            HHP_CUDA(cudaGetLastError());
        }
        bs = A->jac_row_b;
    }
    hhp_solve_opts os = *o;
    os.precond = HHP_PRECOND_NONE;
    hhp_solve_opts oc = *o;  // the residual check: no iterations, no callback
    oc.precond = HHP_PRECOND_NONE;
    oc.maxit = 0;
    oc.fixed_iters = 0;
    oc.print_every = 0;
    oc.cb = nullptr;
    hhp_solve_info is{}, ic{};
    hhp_status rc = HHP_ERR_MAXIT;
    int iters = 0, passes = 0;
    double t = 0.0, rtol_s = o->rtol;
    for (int pass = 0; pass < 8; ++pass) {
        os.rtol = rtol_s;
        os.maxit = o->maxit - iters;
        const hhp_status rs = solve_any(A->jac_row, bs, x, nullptr, &os, &is, host);
        if (rs != HHP_OK && rs != HHP_ERR_MAXIT && rs != HHP_ERR_BREAKDOWN) return rs;
        iters += is.iters;
        passes += std::max(is.outer_iters, 1);
        t += is.t_solve_s;
        const hhp_status rcheck = solve_any(A, b, x, xt, &oc, &ic, host);
        if (rcheck != HHP_OK && rcheck != HHP_ERR_MAXIT) return rcheck;
        t += ic.t_solve_s;
        if (ic.rel_res_true <= o->rtol) {
            rc = HHP_OK;
            break;
        }
        rc = rs == HHP_OK ? HHP_ERR_MAXIT : rs;  // reported if this is the last pass
        if (rs != HHP_OK || iters >= o->maxit) break;
        // the scaled residual met its tolerance but the original one did not: ask the scaled solve
        // for the missing factor (and a margin), never less than 1e-4 per pass
        rtol_s *= std::max(1e-4, 0.5 * o->rtol / ic.rel_res_true);
        if (rtol_s < 1e-17) break;
    }
    if (info) {
        *info = ic;
        info->iters = iters;
        info->outer_iters = passes;
        info->half_step = is.half_step;
        info->rel_res_recursive = is.rel_res_recursive;
        info->t_solve_s = t;
        info->status = rc;
        info->fp64_fallback = is.fp64_fallback;
    }
    return rc;
}

}  // namespace hhp
