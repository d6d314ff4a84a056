// hhp_blas1.cu -- BLAS-1 on device vectors: the reference's device_vector_dot / device_vector_scale /
// device_vector_axpy / device_vector_GPUtoGPU (src/util/hhp_cuda.c:163-202: cuBLAS Ddot, Dscal,
// Daxpy and a device-to-device copy), and the device-pointer-mode Ddot of the dp loop
// (src/entry/bicgstab_gpu_dp.c:163-190), on the context's stream.
//
// The dot product is deterministic (cuBLAS's is not guaranteed to be): each thread sums a fixed
// strided subset with fused multiply-adds, each block folds its threads in a fixed tree, and the
// block that finishes last (an atomic count; no block waits for another) adds the block partials
// in block order and stores the result. One launch; the partials live in context-owned scratch,
// so calls on one context are serialised on its stream.
#include <algorithm>

#include "hhp_device.cuh"
#include "hhp_internal.h"

namespace hhp {

namespace {

constexpr int kDotThreads = 256;
constexpr int kDotMaxBlocks = 1024;

__global__ void __launch_bounds__(kDotThreads) k_dot(const double *__restrict__ x, const double *__restrict__ y,
                                                     long long n, double *part, unsigned *count, double *out) {
    __shared__ double red[kDotThreads / 32];
    __shared__ int last;
    const long long stride = static_cast<long long>(gridDim.x) * blockDim.x;
    double acc = 0.0;
    for (long long i = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; i < n; i += stride)
        acc = fma(__ldg(x + i), __ldg(y + i), acc);
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    acc = warp_sum(acc);
    if (lane == 0) red[warp] = acc;
    __syncthreads();
    if (warp == 0) {
        double s = lane < kDotThreads / 32 ? red[lane] : 0.0;
        s = warp_sum(s);
        if (lane == 0) {
            part[blockIdx.x] = s;
            __threadfence();
            last = atomicAdd(count, 1u) == gridDim.x - 1;
        }
    }
    __syncthreads();
    if (!last || warp != 0) return;
    __threadfence();
    double s = 0.0;
    for (int b = lane; b < static_cast<int>(gridDim.x); b += 32) s += __ldcg(part + b);
    s = warp_sum(s);
    if (lane == 0) {
        *out = s;
        *count = 0u;  // ready for the next launch
    }
}

__global__ void k_axpy(long long n, double alpha, const double *__restrict__ x, double *y) {
    for (long long i = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; i < n;
         i += static_cast<long long>(gridDim.x) * blockDim.x)
        y[i] = fma(alpha, x[i], y[i]);
}

__global__ void k_scal(long long n, double alpha, double *x) {
    for (long long i = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; i < n;
         i += static_cast<long long>(gridDim.x) * blockDim.x)
        x[i] = alpha * x[i];
}

int stream_grid(const hhp_ctx *ctx, long long n) {
    return static_cast<int>(std::max(1LL, std::min((n + 255) / 256, 4LL * ctx->num_sms)));
}

hhp_status ensure_dot_scratch(hhp_ctx *ctx) {
    if (ctx->dot_part) return HHP_OK;
    if (cudaMalloc(&ctx->dot_part, sizeof(double) * kDotMaxBlocks) != cudaSuccess ||
        cudaMalloc(&ctx->dot_count, sizeof(unsigned)) != cudaSuccess ||
        cudaMemsetAsync(ctx->dot_count, 0, sizeof(unsigned), ctx->stream) != cudaSuccess) {
        set_error("dot: out of device memory for the partials");
        return HHP_ERR_OOM;
    }
    return HHP_OK;
}

hhp_status dot_launch(hhp_ctx *ctx, int n, const double *x, const double *y, double *out_dev) {
    if (!ctx || n < 0 || (n > 0 && (!x || !y)) || !out_dev) {
        set_error("dot: null argument or negative length");
        return HHP_ERR_ARG;
    }
    if (n == 0) {
        HHP_CUDA(cudaMemsetAsync(out_dev, 0, sizeof(double), ctx->stream));
        return HHP_OK;
    }
    HHP_TRY(ensure_dot_scratch(ctx));
    const int grid = static_cast<int>(std::min<long long>((n + 4LL * kDotThreads - 1) / (4LL * kDotThreads),
                                                          std::min(kDotMaxBlocks, 2 * ctx->num_sms)));
    k_dot<<<grid, kDotThreads, 0, ctx->stream>>>(x, y, n, ctx->dot_part, ctx->dot_count, out_dev);
    HHP_CUDA(cudaGetLastError());
    ctx->kernel_launches += 1;
    return HHP_OK;
}

}  // namespace

void release_blas1(hhp_ctx *ctx) {
    cudaFree(ctx->dot_part);
    cudaFree(ctx->dot_count);
    ctx->dot_part = nullptr;
    ctx->dot_count = nullptr;
}

}  // namespace hhp

using namespace hhp;

hhp_status hhp_dot_dev(hhp_ctx *ctx, int n, const double *x_dev, const double *y_dev, double *result_dev) {
    return dot_launch(ctx, n, x_dev, y_dev, result_dev);
}

hhp_status hhp_dot(hhp_ctx *ctx, int n, const double *x_dev, const double *y_dev, double *result) {
    if (!result) {
        set_error("dot: result is NULL");
        return HHP_ERR_ARG;
    }
    if (!ctx) {
        set_error("dot: null context");
        return HHP_ERR_ARG;
    }
    HHP_TRY(ensure_dot_scratch(ctx));
    double *slot = ctx->dot_part + (kDotMaxBlocks - 1);  // never a block partial: grids stay below
    HHP_TRY(dot_launch(ctx, n, x_dev, y_dev, slot));
    HHP_CUDA(cudaMemcpyAsync(result, slot, sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
    HHP_CUDA(cudaStreamSynchronize(ctx->stream));
    return HHP_OK;
}

hhp_status hhp_axpy_dev(hhp_ctx *ctx, int n, double alpha, const double *x_dev, double *y_dev) {
    if (!ctx || n < 0 || (n > 0 && (!x_dev || !y_dev))) {
        set_error("axpy: null argument or negative length");
        return HHP_ERR_ARG;
    }
    if (n == 0) return HHP_OK;
    k_axpy<<<stream_grid(ctx, n), 256, 0, ctx->stream>>>(n, alpha, x_dev, y_dev);
    HHP_CUDA(cudaGetLastError());
    ctx->kernel_launches += 1;
    return HHP_OK;
}

hhp_status hhp_scal_dev(hhp_ctx *ctx, int n, double alpha, double *x_dev) {
    if (!ctx || n < 0 || (n > 0 && !x_dev)) {
        set_error("scal: null argument or negative length");
        return HHP_ERR_ARG;
    }
    if (n == 0) return HHP_OK;
    k_scal<<<stream_grid(ctx, n), 256, 0, ctx->stream>>>(n, alpha, x_dev);
    HHP_CUDA(cudaGetLastError());
    ctx->kernel_launches += 1;
    return HHP_OK;
}

hhp_status hhp_copy_dev(hhp_ctx *ctx, int n, const double *src_dev, double *dst_dev) {
    if (!ctx || n < 0 || (n > 0 && (!src_dev || !dst_dev))) {
        set_error("copy: null argument or negative length");
        return HHP_ERR_ARG;
    }
    if (n == 0) return HHP_OK;
    HHP_CUDA(cudaMemcpyAsync(dst_dev, src_dev, sizeof(double) * static_cast<size_t>(n), cudaMemcpyDeviceToDevice,
                             ctx->stream));
    return HHP_OK;
}
