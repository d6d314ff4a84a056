// hhp_api.cu -- the C ABI (include/hhp_gpu.h): errors, contexts, matrices, host-buffer wrappers.
#include <algorithm>
#include <cmath>
#include <cstdarg>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "hhp_internal.h"

namespace hhp {

namespace {
thread_local std::string g_last_error;
}

void set_error(const char *fmt, ...) {
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    std::vsnprintf(buf, sizeof buf, fmt, ap);
    va_end(ap);
    g_last_error = buf;
}

hhp_status cuda_fail(cudaError_t e, const char *what, const char *file, int line) {
    set_error("%s failed: %s (%s:%d)", what, cudaGetErrorString(e), file, line);
    if (e == cudaErrorMemoryAllocation) return HHP_ERR_OOM;
    return HHP_ERR_CUDA;
}

int env_int(const char *name, int dflt) {
    const char *v = std::getenv(name);
    if (!v || !*v) return dflt;
    char *end = nullptr;
    const long x = std::strtol(v, &end, 10);
    if (!end || *end != '\0') return dflt;
    return static_cast<int>(std::min<long>(std::max<long>(x, -(1L << 30)), 1L << 30));
}

// The per-matrix choices below are the library's; the environment overrides exist for kernel
// sweeps and are read only when HHP_TUNING=1 (otherwise the environment is ignored).
const Tuning &tuning() {
    static const Tuning t = [] {
        Tuning d;
        if (env_int("HHP_TUNING", 0) != 1) return d;
        d.cap = env_int("HHP_SPMV_CHUNK", d.cap);
        d.long_thr = env_int("HHP_SPMV_LONG", d.long_thr);
        d.window = env_int("HHP_SPMV_WINDOW", d.window);
        d.wpc = env_int("HHP_SPMV_WPC", d.wpc);
        d.ctas_per_sm = env_int("HHP_SPMV_CPS", d.ctas_per_sm);
        d.vec_blocks_per_sm = env_int("HHP_VEC_BLOCKS_PER_SM", d.vec_blocks_per_sm);
        d.unroll_iters = env_int("HHP_UNROLL_ITERS", d.unroll_iters);
        d.spmv_unroll = env_int("HHP_SPMV_UNROLL", d.spmv_unroll);
        d.rpl64 = env_int("HHP_SPMV_RPL64", d.rpl64);
        d.rpl32 = env_int("HHP_SPMV_RPL32", d.rpl32);
        d.d16 = env_int("HHP_SPMV_D16", d.d16);
        d.uni = env_int("HHP_SPMV_UNI", d.uni);
        // out-of-range overrides fall back to the defaults' valid ranges (a zero window or chunk
        // cap would never advance the plan builder's loops)
        const Tuning def;
        auto clamp = [](int v, int lo, int hi) { return std::min(std::max(v, lo), hi); };
        d.cap = clamp(d.cap, 32, 1 << 24);
        d.long_thr = clamp(d.long_thr, 1, 1 << 24);
        d.window = clamp(d.window, 1, 1 << 30);
        d.wpc = clamp(d.wpc, 1, 8);
        d.ctas_per_sm = clamp(d.ctas_per_sm, 0, 32);
        d.vec_blocks_per_sm = clamp(d.vec_blocks_per_sm, 1, 32);
        d.unroll_iters = clamp(d.unroll_iters, 1, 16);
        if (d.spmv_unroll != 0 && d.spmv_unroll != 2 && d.spmv_unroll != 4) d.spmv_unroll = def.spmv_unroll;
        if (d.rpl64 != 0 && d.rpl64 != 1 && d.rpl64 != 2) d.rpl64 = def.rpl64;
        if (d.rpl32 != 2 && d.rpl32 != 4) d.rpl32 = def.rpl32;
        d.d16 = d.d16 != 0 ? 1 : 0;
        d.uni = d.uni != 0 ? 1 : 0;
        return d;
    }();
    return t;
}

namespace {

__global__ void k_to_f32(const double *__restrict__ v, float *o, int n) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) o[i] = static_cast<float>(v[i]);
}

__global__ void k_check_cols(const int *__restrict__ col, int nnz, int n, int *bad) {
    for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < nnz; k += gridDim.x * blockDim.x)
        if (col[k] < 0 || col[k] >= n) atomicAdd(bad, 1);
}

hhp_status check_host_csr(int m, int n, int nnz, const int *rowptr, const int *col) {
    if (m < 0 || n < 0 || nnz < 0 || !rowptr || (nnz > 0 && !col)) {
        set_error("CSR: invalid sizes or null arrays");
        return HHP_ERR_ARG;
    }
    if (rowptr[0] != 0 || rowptr[m] != nnz) {
        set_error("CSR: rowptr[0] must be 0 and rowptr[m] must equal nnz (%d)", nnz);
        return HHP_ERR_ARG;
    }
    for (int r = 0; r < m; ++r)
        if (rowptr[r + 1] < rowptr[r]) {
            set_error("CSR: rowptr decreases at row %d", r);
            return HHP_ERR_ARG;
        }
    for (int k = 0; k < nnz; ++k)
        if (col[k] < 0 || col[k] >= n) {
            set_error("CSR: column index %d at entry %d is outside [0, %d)", col[k], k, n);
            return HHP_ERR_ARG;
        }
    return HHP_OK;
}

}  // namespace

hhp_status mat_create_dev(hhp_ctx *ctx, int m, int n, int nnz, hhp_mat **out) {
    hhp_mat *A = new hhp_mat();
    A->ctx = ctx;
    A->m = m;
    A->n = n;
    A->nnz = nnz;
    const size_t rp = static_cast<size_t>(m) + 1 + 4, nz = static_cast<size_t>(nnz) + 4;
    if (cudaMalloc(&A->rowptr, rp * sizeof(int)) != cudaSuccess || cudaMalloc(&A->col, nz * sizeof(int)) != cudaSuccess ||
        cudaMalloc(&A->val, nz * sizeof(double)) != cudaSuccess) {
        hhp_mat_destroy(A);
        set_error("out of device memory for a %d x %d matrix with %d nonzeros", m, n, nnz);
        return HHP_ERR_OOM;
    }
    // on the context's stream: it is non-blocking, so work on the legacy default stream would not
    // be ordered before the kernels that later read these arrays
    HHP_CUDA(cudaMemsetAsync(A->rowptr, 0, rp * sizeof(int), ctx->stream));
    HHP_CUDA(cudaMemsetAsync(A->col, 0, nz * sizeof(int), ctx->stream));
    HHP_CUDA(cudaMemsetAsync(A->val, 0, nz * sizeof(double), ctx->stream));
    *out = A;
    return HHP_OK;
}

hhp_status csr_needed(const hhp_mat *A, const char *what) {
    if (!A->csr_dropped) return HHP_OK;
    set_error("%s needs the matrix's CSR arrays, which hhp_mat_drop_csr released", what);
    return HHP_ERR_STATE;
}

hhp_status mat_refresh_derived(hhp_mat *A) {
    HHP_TRY(csr_needed(A, "the FP32 value copy"));
    if (!A->val32) {
        HHP_CUDA(cudaMalloc(&A->val32, (static_cast<size_t>(A->nnz) + 4) * sizeof(float)));
        HHP_CUDA(cudaMemsetAsync(A->val32, 0, (static_cast<size_t>(A->nnz) + 4) * sizeof(float), A->ctx->stream));
    }
    if (A->nnz > 0) {
        const int grid = static_cast<int>(std::max(1LL, std::min((A->nnz + 255LL) / 256, 8LL * A->ctx->num_sms)));
        k_to_f32<<<grid, 256, 0, A->ctx->stream>>>(A->val, A->val32, A->nnz);
        HHP_CUDA(cudaGetLastError());
    }
    HHP_TRY(refresh_plan_values(A));
    if (A->t) HHP_TRY(refresh_transpose_values(A));
    return HHP_OK;
}

}  // namespace hhp

using namespace hhp;

extern "C" {

const char *hhp_status_str(hhp_status s) {
    switch (s) {
        case HHP_OK: return "HHP_OK";
        case HHP_ERR_ARG: return "HHP_ERR_ARG";
        case HHP_ERR_IO: return "HHP_ERR_IO";
        case HHP_ERR_CUDA: return "HHP_ERR_CUDA";
        case HHP_ERR_OOM: return "HHP_ERR_OOM";
        case HHP_ERR_BREAKDOWN: return "HHP_ERR_BREAKDOWN";
        case HHP_ERR_MAXIT: return "HHP_ERR_MAXIT";
        case HHP_ERR_TIMEOUT: return "HHP_ERR_TIMEOUT";
        case HHP_ERR_FORMAT: return "HHP_ERR_FORMAT";
        case HHP_ERR_STATE: return "HHP_ERR_STATE";
    }
    return "HHP_ERR_UNKNOWN";
}

const char *hhp_last_error(void) { return g_last_error.c_str(); }

hhp_status hhp_ctx_create(int device, hhp_ctx **out) {
    HHP_API_BEGIN
    if (!out) {
        set_error("hhp_ctx_create: out is NULL");
        return HHP_ERR_ARG;
    }
    *out = nullptr;
    int ndev = 0;
    HHP_CUDA(cudaGetDeviceCount(&ndev));
    if (device < 0 || device >= ndev) {
        set_error("hhp_ctx_create: device %d not present (%d devices)", device, ndev);
        return HHP_ERR_ARG;
    }
    HHP_CUDA(cudaSetDevice(device));
    cudaDeviceProp prop;
    HHP_CUDA(cudaGetDeviceProperties(&prop, device));
    if (prop.major < 10) {
        set_error("device %d (%s, sm_%d%d) is not a Blackwell GPU; this library is built for sm_103a", device,
                  prop.name, prop.major, prop.minor);
        return HHP_ERR_ARG;
    }
    hhp_ctx *c = new hhp_ctx();
    c->device = device;
    c->num_sms = prop.multiProcessorCount;
    c->smem_optin = prop.sharedMemPerBlockOptin;
    if (cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking) != cudaSuccess ||
        cudaEventCreate(&c->ev0) != cudaSuccess || cudaEventCreate(&c->ev1) != cudaSuccess ||
        cudaMalloc(&c->dev_err, sizeof(int)) != cudaSuccess ||
        cudaMemsetAsync(c->dev_err, 0, sizeof(int), c->stream) != cudaSuccess ||
        cudaStreamSynchronize(c->stream) != cudaSuccess) {
        hhp_ctx_destroy(c);
        set_error("hhp_ctx_create: CUDA setup failed: %s", cudaGetErrorString(cudaGetLastError()));
        return HHP_ERR_CUDA;
    }
    *out = c;
    return HHP_OK;
    HHP_API_END
}

void hhp_ctx_destroy(hhp_ctx *c) {
    if (!c) return;
    if (c->stream) cudaStreamSynchronize(c->stream);
    release_blas1(c);
    if (c->dev_err) cudaFree(c->dev_err);
    if (c->ev0) cudaEventDestroy(c->ev0);
    if (c->ev1) cudaEventDestroy(c->ev1);
    if (c->stream) cudaStreamDestroy(c->stream);
    delete c;
}

void *hhp_ctx_stream(hhp_ctx *c) { return c ? static_cast<void *>(c->stream) : nullptr; }

hhp_status hhp_ctx_sync(hhp_ctx *c) {
    if (!c) return HHP_ERR_ARG;
    HHP_CUDA(cudaStreamSynchronize(c->stream));
    return HHP_OK;
}

long long hhp_ctx_kernel_launches(const hhp_ctx *c) { return c ? c->kernel_launches : 0; }

hhp_status hhp_mat_from_csr(hhp_ctx *ctx, int m, int n, int nnz, const int *rowptr, const int *col, const double *val,
                            const int *perm, hhp_mat **out) {
    HHP_API_BEGIN
    if (!ctx || !out || (nnz > 0 && !val)) {
        set_error("hhp_mat_from_csr: null argument");
        return HHP_ERR_ARG;
    }
    HHP_TRY(check_host_csr(m, n, nnz, rowptr, col));
    std::vector<int> prp, pcol;
    std::vector<double> pval;
    if (perm) {
        // csr_permute (src/util/hhp_dp_helpers.c:18-37): row i <- row perm[i], col j -> perm_inv[j]
        if (m != n) {
            set_error("hhp_mat_from_csr: a permutation needs a square matrix");
            return HHP_ERR_ARG;
        }
        std::vector<int> inv(static_cast<size_t>(m), -1);
        for (int i = 0; i < m; ++i) {
            if (perm[i] < 0 || perm[i] >= m || inv[static_cast<size_t>(perm[i])] != -1) {
                set_error("hhp_mat_from_csr: perm is not a permutation of 0..%d", m - 1);
                return HHP_ERR_ARG;
            }
            inv[static_cast<size_t>(perm[i])] = i;
        }
        prp.assign(static_cast<size_t>(m) + 1, 0);
        pcol.resize(static_cast<size_t>(nnz));
        pval.resize(static_cast<size_t>(nnz));
        for (int i = 0; i < m; ++i) prp[static_cast<size_t>(i) + 1] = prp[static_cast<size_t>(i)] + rowptr[perm[i] + 1] - rowptr[perm[i]];
        for (int i = 0; i < m; ++i) {
            const int s = rowptr[perm[i]], cnt = rowptr[perm[i] + 1] - s, d = prp[static_cast<size_t>(i)];
            for (int k = 0; k < cnt; ++k) {
                pcol[static_cast<size_t>(d + k)] = inv[static_cast<size_t>(col[s + k])];
                pval[static_cast<size_t>(d + k)] = val[s + k];
            }
        }
        rowptr = prp.data();
        col = pcol.data();
        val = pval.data();
    }
    hhp_mat *A = nullptr;
    HHP_TRY(mat_create_dev(ctx, m, n, nnz, &A));
    A->rowptr_host.assign(rowptr, rowptr + m + 1);
    const cudaStream_t st = ctx->stream;
    // ordered after the zero fill on the same stream; the wait keeps the (possibly temporary) host
    // arrays alive until the copies have landed
    if (cudaMemcpyAsync(A->rowptr, rowptr, sizeof(int) * (static_cast<size_t>(m) + 1), cudaMemcpyHostToDevice, st) ||
        (nnz > 0 && cudaMemcpyAsync(A->col, col, sizeof(int) * static_cast<size_t>(nnz), cudaMemcpyHostToDevice, st)) ||
        (nnz > 0 && cudaMemcpyAsync(A->val, val, sizeof(double) * static_cast<size_t>(nnz), cudaMemcpyHostToDevice, st)) ||
        cudaStreamSynchronize(st) != cudaSuccess) {
        hhp_mat_destroy(A);
        set_error("hhp_mat_from_csr: upload failed");
        return HHP_ERR_CUDA;
    }
    *out = A;
    return HHP_OK;
    HHP_API_END
}

hhp_status hhp_mat_from_csr_dev(hhp_ctx *ctx, int m, int n, int nnz, const int *rowptr_dev, const int *col_dev,
                                const double *val_dev, hhp_mat **out) {
    HHP_API_BEGIN
    if (!ctx || !out || m < 0 || n < 0 || nnz < 0 || !rowptr_dev || (nnz > 0 && (!col_dev || !val_dev))) {
        set_error("hhp_mat_from_csr_dev: invalid arguments");
        return HHP_ERR_ARG;
    }
    std::vector<int> rp(static_cast<size_t>(m) + 1);
    // the caller's arrays may have been written by work on this context's stream
    HHP_CUDA(cudaStreamSynchronize(ctx->stream));
    HHP_CUDA(cudaMemcpy(rp.data(), rowptr_dev, sizeof(int) * rp.size(), cudaMemcpyDeviceToHost));
    if (rp[0] != 0 || rp[static_cast<size_t>(m)] != nnz) {
        set_error("hhp_mat_from_csr_dev: rowptr[0] must be 0 and rowptr[m] must equal nnz");
        return HHP_ERR_ARG;
    }
    for (int r = 0; r < m; ++r)
        if (rp[static_cast<size_t>(r) + 1] < rp[static_cast<size_t>(r)]) {
            set_error("hhp_mat_from_csr_dev: rowptr decreases at row %d", r);
            return HHP_ERR_ARG;
        }
    hhp_mat *A = nullptr;
    HHP_TRY(mat_create_dev(ctx, m, n, nnz, &A));
    A->rowptr_host = std::move(rp);
    int *bad = nullptr;
    int hbad = 0;
    const cudaStream_t st = ctx->stream;
    if (cudaMalloc(&bad, sizeof(int)) ||
        cudaMemcpyAsync(A->rowptr, rowptr_dev, sizeof(int) * (static_cast<size_t>(m) + 1), cudaMemcpyDeviceToDevice, st) ||
        (nnz > 0 && cudaMemcpyAsync(A->col, col_dev, sizeof(int) * static_cast<size_t>(nnz), cudaMemcpyDeviceToDevice, st)) ||
        (nnz > 0 && cudaMemcpyAsync(A->val, val_dev, sizeof(double) * static_cast<size_t>(nnz), cudaMemcpyDeviceToDevice, st)) ||
        cudaMemsetAsync(bad, 0, sizeof(int), st)) {
        cudaFree(bad);
        hhp_mat_destroy(A);
        set_error("hhp_mat_from_csr_dev: copy failed");
        return HHP_ERR_CUDA;
    }
    if (nnz > 0) {
        k_check_cols<<<static_cast<int>(std::max(1LL, std::min((nnz + 255LL) / 256, 8LL * ctx->num_sms))), 256, 0,
                       st>>>(A->col, nnz, n, bad);
        cudaMemcpyAsync(&hbad, bad, sizeof(int), cudaMemcpyDeviceToHost, st);
    }
    const cudaError_t e_sync = cudaStreamSynchronize(st);
    cudaFree(bad);
    if (e_sync != cudaSuccess) {
        hhp_mat_destroy(A);
        return cuda_fail(e_sync, "hhp_mat_from_csr_dev: copy", __FILE__, __LINE__);
    }
    if (hbad != 0) {
        hhp_mat_destroy(A);
        set_error("hhp_mat_from_csr_dev: %d column indices outside [0, %d)", hbad, n);
        return HHP_ERR_ARG;
    }
    *out = A;
    return HHP_OK;
    HHP_API_END
}

hhp_status hhp_mat_from_mtx(hhp_ctx *ctx, const char *path, hhp_mat **out) {
    HHP_API_BEGIN
    if (!ctx || !out) {
        set_error("hhp_mat_from_mtx: null argument");
        return HHP_ERR_ARG;
    }
    int m = 0, n = 0, nnz = 0;
    std::vector<int> rp, col;
    std::vector<double> val;
    HHP_TRY(read_mtx(path, m, n, nnz, rp, col, val));
    return hhp_mat_from_csr(ctx, m, n, nnz, rp.data(), col.data(), val.data(), nullptr, out);
    HHP_API_END
}

void hhp_mat_destroy(hhp_mat *A) {
    if (!A) return;
    if (A->ctx && A->ctx->stream) cudaStreamSynchronize(A->ctx->stream);
    if (A->t) hhp_mat_destroy(A->t);
    release_jacobi(A);
    release_ilu(A);
    solver_release(A->solver);
    A->plan64.release();
    A->plan32.release();
    cudaFree(A->rowptr);
    cudaFree(A->col);
    cudaFree(A->val);
    cudaFree(A->val32);
    cudaFree(A->t_map);
    cudaFree(A->rowidx);
    delete A;
}

hhp_status hhp_mat_drop_csr(hhp_mat *A, int keep_fp32) {
    HHP_API_BEGIN
    if (!A) {
        set_error("hhp_mat_drop_csr: null matrix");
        return HHP_ERR_ARG;
    }
    if (A->csr_dropped) return HHP_OK;
    HHP_TRY(ensure_plan(A, false));
    if (keep_fp32) {
        if (!A->val32) HHP_TRY(mat_refresh_derived(A));
        HHP_TRY(ensure_plan(A, true));
    }
    if (A->plan64.n_chunks > 0 || (A->plan32.built() && A->plan32.n_chunks > 0)) {
        set_error("hhp_mat_drop_csr: rows longer than the slice limit are summed from the CSR arrays");
        return HHP_ERR_ARG;
    }
    HHP_CUDA(cudaStreamSynchronize(A->ctx->stream));
    ilu_keep_col(A);  // ILU(0) factors built before the drop keep their column array
    cudaFree(A->col);
    cudaFree(A->val);
    cudaFree(A->val32);
    A->col = nullptr;
    A->val = nullptr;
    A->val32 = nullptr;
    A->csr_dropped = true;
    return HHP_OK;
    HHP_API_END
}

hhp_status hhp_mat_shape(const hhp_mat *A, int *m, int *n, int *nnz) {
    if (!A) return HHP_ERR_ARG;
    if (m) *m = A->m;
    if (n) *n = A->n;
    if (nnz) *nnz = A->nnz;
    return HHP_OK;
}

static hhp_status set_values(hhp_mat *A, const double *v, cudaMemcpyKind kind) {
    if (!A || (A->nnz > 0 && !v)) {
        set_error("hhp_mat_set_values: invalid arguments");
        return HHP_ERR_ARG;
    }
    HHP_TRY(csr_needed(A, "hhp_mat_set_values"));
    if (A->nnz > 0)
        HHP_CUDA(cudaMemcpyAsync(A->val, v, sizeof(double) * static_cast<size_t>(A->nnz), kind, A->ctx->stream));
    if (A->val32 || A->t || A->plan64.built() || A->plan32.built()) HHP_TRY(mat_refresh_derived(A));
    HHP_CUDA(cudaStreamSynchronize(A->ctx->stream));
    release_jacobi(A);  // rebuilt from the new values on the next preconditioned solve
    release_ilu(A);
    return HHP_OK;
}

hhp_status hhp_mat_set_values(hhp_mat *A, const double *val) { return set_values(A, val, cudaMemcpyHostToDevice); }
hhp_status hhp_mat_set_values_dev(hhp_mat *A, const double *val) { return set_values(A, val, cudaMemcpyDeviceToDevice); }

hhp_status hhp_mat_get_csr(const hhp_mat *A, int *rowptr, int *col, double *val) {
    HHP_API_BEGIN
    if (!A) return HHP_ERR_ARG;
    HHP_TRY(csr_needed(A, "hhp_mat_get_csr"));
    HHP_CUDA(cudaStreamSynchronize(A->ctx->stream));
    if (rowptr) HHP_CUDA(cudaMemcpy(rowptr, A->rowptr, sizeof(int) * (static_cast<size_t>(A->m) + 1), cudaMemcpyDeviceToHost));
    if (col && A->nnz) HHP_CUDA(cudaMemcpy(col, A->col, sizeof(int) * static_cast<size_t>(A->nnz), cudaMemcpyDeviceToHost));
    if (val && A->nnz) HHP_CUDA(cudaMemcpy(val, A->val, sizeof(double) * static_cast<size_t>(A->nnz), cudaMemcpyDeviceToHost));
    return HHP_OK;
    HHP_API_END
}

hhp_status hhp_mat_get_transpose(hhp_mat *A, int *t_rowptr, int *t_col, double *t_val) {
    HHP_API_BEGIN
    if (!A) return HHP_ERR_ARG;
    HHP_TRY(ensure_transpose(A));
    return hhp_mat_get_csr(A->t, t_rowptr, t_col, t_val);
    HHP_API_END
}

hhp_status hhp_spmv_dev(hhp_ctx *ctx, hhp_mat *A, double alpha, const double *x, double beta, double *y) {
    HHP_API_BEGIN
    if (!ctx || !A || A->ctx != ctx || (A->n > 0 && !x) || (A->m > 0 && !y)) {
        set_error("hhp_spmv_dev: invalid arguments");
        return HHP_ERR_ARG;
    }
    if (A->m == 0) return HHP_OK;
    return launch_spmv64(A, ctx->stream, EP_AXPBY, x, y, nullptr, alpha, beta);
    HHP_API_END
}

hhp_status hhp_spmv_f32_dev(hhp_ctx *ctx, hhp_mat *A, const float *x, float *y) {
    HHP_API_BEGIN
    if (!ctx || !A || A->ctx != ctx || (A->n > 0 && !x) || (A->m > 0 && !y)) {
        set_error("hhp_spmv_f32_dev: invalid arguments");
        return HHP_ERR_ARG;
    }
    if (!A->val32) HHP_TRY(mat_refresh_derived(A));
    if (A->m == 0) return HHP_OK;
    return launch_spmv32(A, ctx->stream, EP_AXPBY, x, y, nullptr);
    HHP_API_END
}

hhp_status hhp_spmv_t_dev(hhp_ctx *ctx, hhp_mat *A, const double *x, double *y) {
    HHP_API_BEGIN
    if (!ctx || !A || A->ctx != ctx || (A->m > 0 && !x) || (A->n > 0 && !y)) {
        set_error("hhp_spmv_t_dev: invalid arguments");
        return HHP_ERR_ARG;
    }
    HHP_TRY(ensure_transpose(A));
    if (A->n == 0) return HHP_OK;
    return launch_spmv64(A->t, ctx->stream, EP_AXPBY, x, y, nullptr, 1.0, 0.0);
    HHP_API_END
}

hhp_status hhp_spmv(hhp_ctx *ctx, hhp_mat *A, const double *x, double *y) {
    HHP_API_BEGIN
    if (!ctx || !A || A->ctx != ctx || (A->n > 0 && !x) || (A->m > 0 && !y)) {
        set_error("hhp_spmv: invalid arguments");
        return HHP_ERR_ARG;
    }
    double *dx = nullptr, *dy = nullptr;
    HHP_CUDA(cudaMalloc(&dx, sizeof(double) * (static_cast<size_t>(A->n) + 1)));
    if (cudaMalloc(&dy, sizeof(double) * (static_cast<size_t>(A->m) + 1)) != cudaSuccess) {
        cudaFree(dx);
        set_error("hhp_spmv: out of device memory");
        return HHP_ERR_OOM;
    }
    hhp_status rc = HHP_OK;
    if (cudaMemcpyAsync(dx, x, sizeof(double) * static_cast<size_t>(A->n), cudaMemcpyHostToDevice, ctx->stream) != cudaSuccess)
        rc = HHP_ERR_CUDA;
    if (rc == HHP_OK && A->m > 0) rc = launch_spmv64(A, ctx->stream, EP_AXPBY, dx, dy, nullptr, 1.0, 0.0);
    if (rc == HHP_OK &&
        cudaMemcpyAsync(y, dy, sizeof(double) * static_cast<size_t>(A->m), cudaMemcpyDeviceToHost, ctx->stream) != cudaSuccess)
        rc = HHP_ERR_CUDA;
    if (rc == HHP_OK && cudaStreamSynchronize(ctx->stream) != cudaSuccess) rc = HHP_ERR_CUDA;
    if (rc == HHP_ERR_CUDA) set_error("hhp_spmv: %s", cudaGetErrorString(cudaGetLastError()));
    cudaFree(dx);
    cudaFree(dy);
    return rc;
    HHP_API_END
}

static hhp_solve_opts default_opts() {
    hhp_solve_opts o;
    std::memset(&o, 0, sizeof o);
    o.rtol = 1e-10;
    o.maxit = 2000;
    o.precision = HHP_PREC_FP64;
    o.inner_rtol = 0.05;
    o.max_outer = 50;
    return o;
}

static hhp_status check_solve(hhp_ctx *ctx, hhp_mat *A, const void *b, const void *x, const hhp_solve_opts *o) {
    if (!ctx || !A || A->ctx != ctx || !b || !x) {
        set_error("bicgstab: null argument or matrix from another context");
        return HHP_ERR_ARG;
    }
    if (A->m != A->n || A->m == 0) {
        set_error("bicgstab: the matrix must be square and non-empty (got %d x %d)", A->m, A->n);
        return HHP_ERR_ARG;
    }
    if (o && (o->maxit < 0 || !(o->rtol >= 0.0) || (o->precision != HHP_PREC_FP64 && o->precision != HHP_PREC_MIXED) ||
              (o->precond != HHP_PRECOND_NONE && o->precond != HHP_PRECOND_JACOBI &&
               o->precond != HHP_PRECOND_JACOBI_ROW && o->precond != HHP_PRECOND_ILU0) ||
              (o->loop != HHP_LOOP_AUTO && o->loop != HHP_LOOP_MERGED && o->loop != HHP_LOOP_CLASSIC))) {
        set_error("bicgstab: invalid options (maxit %d, rtol %g, precision %d, precond %d, loop %d)", o->maxit,
                  o->rtol, o->precision, o->precond, o->loop);
        return HHP_ERR_ARG;
    }
    return HHP_OK;
}

hhp_status hhp_bicgstab(hhp_ctx *ctx, hhp_mat *A, const double *b, double *x, const double *xt,
                        const hhp_solve_opts *opts, hhp_solve_info *info) {
    HHP_API_BEGIN
    HHP_TRY(check_solve(ctx, A, b, x, opts));
    const hhp_solve_opts o = opts ? *opts : default_opts();
    if (o.precond == HHP_PRECOND_JACOBI) return solve_jacobi(A, b, x, xt, &o, info, true);
    if (o.precond == HHP_PRECOND_JACOBI_ROW) return solve_jacobi_row(A, b, x, xt, &o, info, true);
    return solve_any(A, b, x, xt, &o, info, true);
    HHP_API_END
}

hhp_status hhp_bicgstab_dev(hhp_ctx *ctx, hhp_mat *A, const double *b, double *x, const double *xt,
                            const hhp_solve_opts *opts, hhp_solve_info *info) {
    HHP_API_BEGIN
    HHP_TRY(check_solve(ctx, A, b, x, opts));
    const hhp_solve_opts o = opts ? *opts : default_opts();
    if (o.precond == HHP_PRECOND_JACOBI) return solve_jacobi(A, b, x, xt, &o, info, false);
    if (o.precond == HHP_PRECOND_JACOBI_ROW) return solve_jacobi_row(A, b, x, xt, &o, info, false);
    return solve_any(A, b, x, xt, &o, info, false);
    HHP_API_END
}

hhp_status hhp_ilu0_factor(hhp_ctx *ctx, hhp_mat *A, double *lu, int *levels) {
    HHP_API_BEGIN
    if (!ctx || !A || A->ctx != ctx) {
        set_error("ilu0_factor: null argument or matrix from another context");
        return HHP_ERR_ARG;
    }
    HHP_TRY(ensure_ilu(A, levels));
    if (lu) HHP_TRY(ilu_factors(A, lu));
    return HHP_OK;
    HHP_API_END
}

hhp_status hhp_ilu0_apply_dev(hhp_ctx *ctx, hhp_mat *A, const double *r_dev, double *z_dev) {
    HHP_API_BEGIN
    if (!ctx || !A || A->ctx != ctx || !r_dev || !z_dev) {
        set_error("ilu0_apply: null argument or matrix from another context");
        return HHP_ERR_ARG;
    }
    HHP_TRY(ensure_ilu(A));
    HHP_CUDA(cudaMemsetAsync(ctx->dev_err, 0, sizeof(int), ctx->stream));
    return launch_ilu_apply(A, ctx->stream, r_dev, z_dev, nullptr);
    HHP_API_END
}

hhp_status hhp_bicgstab_backward_dev(hhp_ctx *ctx, hhp_mat *A, const double *x, const double *dldx, double *dldb,
                                     double *dlda, const hhp_solve_opts *opts, hhp_solve_info *info) {
    HHP_API_BEGIN
    HHP_TRY(check_solve(ctx, A, dldx, x, opts));
    if (!dldb) {
        set_error("bicgstab_backward: dldb is NULL");
        return HHP_ERR_ARG;
    }
    hhp_solve_opts o = opts ? *opts : default_opts();
    if (!opts) o.inner_rtol = 0.0;  // the adjoint's own default factor
    o.fixed_iters = 0;
    return backward_dev(A, x, dldx, dldb, dlda, &o, info);
    HHP_API_END
}

hhp_status hhp_bicgstab_backward(hhp_ctx *ctx, hhp_mat *A, const double *x, const double *dldx, double *dldb,
                                 double *dlda, const hhp_solve_opts *opts, hhp_solve_info *info) {
    HHP_API_BEGIN
    HHP_TRY(check_solve(ctx, A, dldx, x, opts));
    if (!dldb) {
        set_error("bicgstab_backward: dldb is NULL");
        return HHP_ERR_ARG;
    }
    const size_t n = static_cast<size_t>(A->n), nz = static_cast<size_t>(A->nnz);
    double *d = nullptr;
    HHP_CUDA(cudaMalloc(&d, sizeof(double) * (3 * n + nz + 1)));
    double *dx = d, *dg = d + n, *db = d + 2 * n, *da = d + 3 * n;
    hhp_status rc = HHP_OK;
    if (cudaMemcpyAsync(dx, x, sizeof(double) * n, cudaMemcpyHostToDevice, ctx->stream) != cudaSuccess ||
        cudaMemcpyAsync(dg, dldx, sizeof(double) * n, cudaMemcpyHostToDevice, ctx->stream) != cudaSuccess) {
        set_error("bicgstab_backward: upload failed");
        rc = HHP_ERR_CUDA;
    }
    if (rc == HHP_OK) {
        hhp_solve_opts o = opts ? *opts : default_opts();
        if (!opts) o.inner_rtol = 0.0;  // the adjoint's own default factor
        o.fixed_iters = 0;
        rc = backward_dev(A, dx, dg, db, dlda ? da : nullptr, &o, info);
    }
    if (rc == HHP_OK || rc == HHP_ERR_MAXIT) {
        if (cudaMemcpyAsync(dldb, db, sizeof(double) * n, cudaMemcpyDeviceToHost, ctx->stream) != cudaSuccess ||
            (dlda && nz &&
             cudaMemcpyAsync(dlda, da, sizeof(double) * nz, cudaMemcpyDeviceToHost, ctx->stream) != cudaSuccess) ||
            cudaStreamSynchronize(ctx->stream) != cudaSuccess) {
            set_error("bicgstab_backward: download failed");
            rc = HHP_ERR_CUDA;
        }
    }
    cudaFree(d);
    return rc;
    HHP_API_END
}

}  // extern "C"
