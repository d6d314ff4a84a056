// hhp_device.cuh -- device-side building blocks for the sm_103a kernels: 1-D TMA bulk copies
// (cp.async.bulk) completing on shared-memory mbarriers, bounded mbarrier waits, and warp/block
// reductions with a fixed summation order (so every reduction is bit-reproducible run to run).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

namespace hhp {

// Device error codes written to the context's error word (first writer wins).
enum : int {
    DEV_OK = 0,
    DEV_ERR_TIMEOUT = 1,   // an mbarrier wait exceeded its time limit
};

// Solver status values kept in device memory.
enum : int {
    ST_RUNNING = 0,
    ST_CONVERGED = 1,      // ||r|| <= threshold after a full iteration
    ST_HALF = 2,           // ||s|| <= threshold: x += alpha*p is the last update (set mid-iteration)
    ST_CONVERGED_HALF = 3, // terminal form of ST_HALF
    ST_BREAKDOWN = 4,      // rho, (r0,v) or (t,t) is zero or not finite
    ST_MAXIT = 5,          // iteration cap reached
    ST_DEVICE_ERROR = 6,   // a kernel recorded a device error (e.g. a wait timeout)
};

__device__ __forceinline__ uint32_t smem_u32(const void *p) {
    return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ uint64_t global_timer_ns() {
    uint64_t t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

__device__ __forceinline__ void mbar_init(uint64_t *bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}

// Makes mbarrier initialisation visible to the async (TMA) proxy.
__device__ __forceinline__ void fence_mbar_init() {
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

// Orders this thread's earlier generic-proxy shared-memory accesses before later async-proxy
// writes (a TMA copy into a buffer the warp has just read).
__device__ __forceinline__ void fence_proxy_async_smem() {
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t *bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes)
                 : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint64_t *bar, uint32_t parity) {
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(smem_u32(bar)), "r"(parity)
        : "memory");
    return ok != 0;
}

// Waits for the mbarrier phase with the given parity to complete, for at most `limit_ns`.
// Returns false on timeout (the caller records the error and stops issuing work).
__device__ __forceinline__ bool mbar_wait_bounded(uint64_t *bar, uint32_t parity, uint64_t limit_ns) {
    if (mbar_try_wait(bar, parity)) return true;
    const uint64_t t0 = global_timer_ns();
    while (true) {
        if (mbar_try_wait(bar, parity)) return true;
        if (global_timer_ns() - t0 > limit_ns) return false;
    }
}

// 1-D bulk copy global -> shared (TMA engine), completion counted on `bar` in bytes.
// Both addresses 16-byte aligned, bytes a multiple of 16.
__device__ __forceinline__ void bulk_g2s(void *dst_smem, const void *src_gmem, uint32_t bytes, uint64_t *bar) {
    asm volatile(
        "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
            smem_u32(dst_smem)),
        "l"(src_gmem), "r"(bytes), "r"(smem_u32(bar))
        : "memory");
}

__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}
__device__ __forceinline__ float warp_sum(float v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

// Block-wide sum of NC values per thread; result valid in thread 0 of the block. Warp sums are
// combined in warp order by thread 0, so the result does not depend on scheduling.
template <int NC>
__device__ __forceinline__ void block_sum(double (&v)[NC], double *scratch /* >= 32*NC doubles */) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = (blockDim.x + 31) >> 5;
#pragma unroll
    for (int c = 0; c < NC; ++c) v[c] = warp_sum(v[c]);
    if (lane == 0) {
#pragma unroll
        for (int c = 0; c < NC; ++c) scratch[warp * NC + c] = v[c];
    }
    __syncthreads();
    if (threadIdx.x == 0) {
#pragma unroll
        for (int c = 0; c < NC; ++c) {
            double s = 0.0;
            for (int w = 0; w < nw; ++w) s += scratch[w * NC + c];
            v[c] = s;
        }
    }
    __syncthreads();
}

// Sum of per-block partials part[i*NC + c] for i in [0, n), plus extra[j*NC + c] for j in
// [0, n_extra), computed identically by every calling block: every thread first loads its
// share (thread t takes entries t, t + blockDim.x, ...; all loads are issued before any add,
// so the whole reduction costs one memory round trip), then a warp butterfly and a sum of the
// warp results in warp order. The order is fixed, so every block gets the same bits. Must be
// called by all threads; the result is returned to every thread. Loads use ld.global.cg so values
// written by earlier kernels are read from L2.
template <int NC>
__device__ __forceinline__ void reduce_partials(const double *__restrict__ part, int n,
                                                const double *__restrict__ extra, int n_extra,
                                                double (&out)[NC], double *scratch /* >= 32*NC doubles */) {
    double s[NC];
#pragma unroll
    for (int c = 0; c < NC; ++c) s[c] = 0.0;
    const int T = blockDim.x, t = threadIdx.x;
    double a[2][NC], b[2][NC];
#pragma unroll
    for (int q = 0; q < 2; ++q) {
        const int i = t + q * T;
#pragma unroll
        for (int c = 0; c < NC; ++c) {
            a[q][c] = i < n ? __ldcg(part + (size_t)i * NC + c) : 0.0;
            b[q][c] = i < n_extra ? __ldcg(extra + (size_t)i * NC + c) : 0.0;
        }
    }
#pragma unroll
    for (int c = 0; c < NC; ++c) s[c] = (a[0][c] + a[1][c]) + (b[0][c] + b[1][c]);
    for (int i = t + 2 * T; i < n; i += T) {  // only for more than 2*blockDim partials
#pragma unroll
        for (int c = 0; c < NC; ++c) s[c] += __ldcg(part + (size_t)i * NC + c);
    }
    for (int i = t + 2 * T; i < n_extra; i += T) {
#pragma unroll
        for (int c = 0; c < NC; ++c) s[c] += __ldcg(extra + (size_t)i * NC + c);
    }
    const int lane = t & 31, warp = t >> 5, nw = (T + 31) >> 5;
#pragma unroll
    for (int c = 0; c < NC; ++c) s[c] = warp_sum(s[c]);
    if (lane == 0) {
#pragma unroll
        for (int c = 0; c < NC; ++c) scratch[warp * NC + c] = s[c];
    }
    __syncthreads();
#pragma unroll
    for (int c = 0; c < NC; ++c) {
        double v = 0.0;
        for (int w = 0; w < nw; ++w) v += scratch[w * NC + c];
        out[c] = v;
    }
    __syncthreads();
}

__device__ __forceinline__ bool finite_nonzero(double v) { return isfinite(v) && v != 0.0; }

}  // namespace hhp
