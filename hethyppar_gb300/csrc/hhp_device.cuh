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

// Block-wide sum of NC values per thread; result valid in thread 0 of the block. Every thread
// parks its values in shared memory and warp 0 alone adds them (lane l: threads l, l+32, ... in
// order, then a butterfly), so the FP64 work is ~blockDim adds rather than a butterfly in every
// warp. Fixed order: the result does not depend on scheduling. scratch: blockDim.x * NC doubles.
template <int NC>
__device__ __forceinline__ void block_sum(double (&v)[NC], double *scratch) {
    const int t = threadIdx.x, T = blockDim.x;
#pragma unroll
    for (int c = 0; c < NC; ++c) scratch[c * T + t] = v[c];
    __syncthreads();
    if (t < 32) {
        double s[NC];
#pragma unroll
        for (int c = 0; c < NC; ++c) {
            s[c] = 0.0;
            for (int i = t; i < T; i += 32) s[c] += scratch[c * T + i];
            s[c] = warp_sum(s[c]);
        }
        if (t == 0) {
#pragma unroll
            for (int c = 0; c < NC; ++c) v[c] = s[c];
        }
    }
    __syncthreads();
}

// Shared-memory doubles a kernel provides to reduce_partials (records are staged in chunks).
constexpr int kRedScratch = 2048;

// Sum of per-block partials part[i*NC + c] for i in [0, n), plus extra[j*NC + c] for j in
// [0, n_extra), computed identically by every calling block. Records are staged through shared
// memory in chunks of kRedScratch/NC: all threads load a chunk at once (one memory round trip per
// chunk), then warp 0 alone adds it (lane l: records l, l+32, ... in order, continuing its running
// sums), and a final butterfly combines the lanes. Only warp 0 does FP64 adds, keeping the FP64
// work per block near the record count (the FP64 pipe is GB300's scarcest unit). The order is
// fixed, so every block gets the same bits. Must be called by all threads; the result is
// returned to every thread. Loads use ld.global.cg (values written by earlier kernels).
template <int NC>
__device__ __forceinline__ void reduce_partials(const double *__restrict__ part, int n,
                                                const double *__restrict__ extra, int n_extra,
                                                double (&out)[NC], double *scratch /* kRedScratch */) {
    const int T = blockDim.x, t = threadIdx.x;
    constexpr int kRec = kRedScratch / NC;
    const int tot = n + n_extra;
    double s[NC];
#pragma unroll
    for (int c = 0; c < NC; ++c) s[c] = 0.0;
    for (int r0 = 0; r0 < tot; r0 += kRec) {
        const int cnt = min(kRec, tot - r0);
        for (int i = t; i < cnt * NC; i += T) {
            const int g = r0 * NC + i;
            scratch[i] = g < n * NC ? __ldcg(part + g) : __ldcg(extra + (g - n * NC));
        }
        __syncthreads();
        if (t < 32) {
            for (int i = t; i < cnt; i += 32) {
#pragma unroll
                for (int c = 0; c < NC; ++c) s[c] += scratch[i * NC + c];
            }
        }
        __syncthreads();
    }
    if (t < 32) {
#pragma unroll
        for (int c = 0; c < NC; ++c) s[c] = warp_sum(s[c]);
        if (t == 0) {
#pragma unroll
            for (int c = 0; c < NC; ++c) scratch[c] = s[c];
        }
    }
    __syncthreads();
#pragma unroll
    for (int c = 0; c < NC; ++c) out[c] = scratch[c];
    __syncthreads();
}

// Two independent reductions (A = part_a + extra_a, B = part_b) staged together, so they cost
// one memory round trip and one pass of warp 0 instead of two. Same order guarantees as
// reduce_partials.
template <int NC>
__device__ __forceinline__ void reduce_pair(const double *__restrict__ part_a, int na, const double *__restrict__ extra_a,
                                            int nea, const double *__restrict__ part_b, int nb, double (&out_a)[NC],
                                            double (&out_b)[NC], double *scratch /* kRedScratch */) {
    const int T = blockDim.x, t = threadIdx.x;
    constexpr int kRec = kRedScratch / NC;
    const int ta = na + nea, tot = ta + nb;
    double sa[NC], sb[NC];
#pragma unroll
    for (int c = 0; c < NC; ++c) sa[c] = sb[c] = 0.0;
    for (int r0 = 0; r0 < tot; r0 += kRec) {
        const int cnt = min(kRec, tot - r0);
        for (int i = t; i < cnt * NC; i += T) {
            const int g = r0 * NC + i;
            double v;
            if (g < na * NC) v = __ldcg(part_a + g);
            else if (g < ta * NC) v = __ldcg(extra_a + (g - na * NC));
            else v = __ldcg(part_b + (g - ta * NC));
            scratch[i] = v;
        }
        __syncthreads();
        if (t < 32) {
            for (int i = t; i < cnt; i += 32) {
                const bool in_a = r0 + i < ta;
#pragma unroll
                for (int c = 0; c < NC; ++c) {
                    if (in_a) sa[c] += scratch[i * NC + c];
                    else sb[c] += scratch[i * NC + c];
                }
            }
        }
        __syncthreads();
    }
    if (t < 32) {
#pragma unroll
        for (int c = 0; c < NC; ++c) {
            sa[c] = warp_sum(sa[c]);
            sb[c] = warp_sum(sb[c]);
        }
        if (t == 0) {
#pragma unroll
            for (int c = 0; c < NC; ++c) {
                scratch[c] = sa[c];
                scratch[NC + c] = sb[c];
            }
        }
    }
    __syncthreads();
#pragma unroll
    for (int c = 0; c < NC; ++c) {
        out_a[c] = scratch[c];
        out_b[c] = scratch[NC + c];
    }
    __syncthreads();
}

__device__ __forceinline__ bool finite_nonzero(double v) { return isfinite(v) && v != 0.0; }

}  // namespace hhp
