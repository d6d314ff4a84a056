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

void release_jacobi(hhp_mat *A) {
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

}  // namespace hhp
