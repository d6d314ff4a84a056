// hhp_probe.cu -- measured FP64 multiply-add throughput of the context's device.
//
// GB300's FP64 rate is low (measured about 20 SM-cycles per warp-wide FP64 FMA, i.e. ~1.6 FMA
// lanes per clock per SM), low enough that the FP64 SpMV and the BiCGStab vector kernels are as
// much bound by the FP64 pipe as by HBM. bench.py reports that second floor beside the HBM roofline;
// this probe measures its denominator on the device the library runs on, instead of a nominal figure.
#include "hhp_internal.h"

namespace hhp {
namespace {

constexpr int kProbeChains = 4;  // independent FMA chains per thread (one chain per SMSP already saturates)
constexpr int kProbeIters = 2048;
constexpr int kProbeThreads = 512;

__device__ double g_probe_sink;  // the probe's result lands here only if a sum is negative (never)

__global__ void __launch_bounds__(kProbeThreads) k_fp64_probe(int iters, double seed) {
    double a[kProbeChains];
#pragma unroll
    for (int k = 0; k < kProbeChains; ++k) a[k] = seed + 1e-7 * threadIdx.x + k;
    for (int i = 0; i < iters; ++i) {
#pragma unroll
        for (int k = 0; k < kProbeChains; ++k) a[k] = fma(a[k], 0.999999999, 1e-9);
    }
    double s = 0.0;
#pragma unroll
    for (int k = 0; k < kProbeChains; ++k) s += a[k];
    if (s < 0.0) g_probe_sink = s;  // never true (every chain stays near 1): keeps the chains live
}

}  // namespace
}  // namespace hhp

extern "C" hhp_status hhp_ctx_fp64_fma_rate(hhp_ctx *ctx, double *fma_per_s) {
    using namespace hhp;
    if (!ctx || !fma_per_s) {
        set_error("hhp_ctx_fp64_fma_rate: null argument");
        return HHP_ERR_ARG;
    }
    const dim3 grid(ctx->num_sms), block(kProbeThreads);
    k_fp64_probe<<<grid, block, 0, ctx->stream>>>(64, 1.0);  // warm-up (clocks, instruction cache)
    HHP_CUDA(cudaGetLastError());
    HHP_CUDA(cudaEventRecord(ctx->ev0, ctx->stream));
    k_fp64_probe<<<grid, block, 0, ctx->stream>>>(kProbeIters, 1.0);
    HHP_CUDA(cudaGetLastError());
    HHP_CUDA(cudaEventRecord(ctx->ev1, ctx->stream));
    HHP_CUDA(cudaEventSynchronize(ctx->ev1));
    float ms = 0.f;
    HHP_CUDA(cudaEventElapsedTime(&ms, ctx->ev0, ctx->ev1));
    ctx->kernel_launches += 2;
    const double fmas = static_cast<double>(ctx->num_sms) * kProbeThreads * kProbeChains * kProbeIters;
    *fma_per_s = ms > 0.f ? fmas / (ms * 1e-3) : 0.0;
    return HHP_OK;
}
