// hhp_device.cuh -- device-side building blocks for the sm_103a kernels: status codes, warp and
// block reductions with a fixed summation order (so every reduction is bit-reproducible run to
// run), and the host-side kernel launcher.
#pragma once

#include <cuda_runtime.h>

#include <utility>
#include <stdint.h>

namespace hhp {

// Device error codes for the context's error word. The only waits in this library are the grid
// barriers between dependency levels inside the ILU(0) kernels (cooperative launches, so every
// block is resident); each is bounded, and one that runs out sets DEV_ERR_TIMEOUT. SpMV launches,
// the ILU kernels and the solve loop check the word, so every later launch stops and the solve
// returns HHP_ERR_TIMEOUT. (The SpMV's long-row combine is a last-arriver atomic count, not a
// wait; every other ordering is a kernel boundary.)
enum : int {
    DEV_OK = 0,
    DEV_ERR_TIMEOUT = 1,
};

// Solver status values kept in device memory.
enum : int {
    ST_RUNNING = 0,
    ST_CONVERGED = 1,      // ||r|| <= threshold after a full iteration
    ST_CONVERGED_HALF = 3, // ||s|| <= threshold: x += alpha*p was the last update
    ST_BREAKDOWN = 4,      // rho, (r0,v) or (t,t) is zero or not finite
    ST_MAXIT = 5,          // iteration cap reached
    ST_DEVICE_ERROR = 6,   // a kernel recorded a device error (e.g. a wait timeout)
    ST_UPDATE_PENDING = 7, // mixed form, not terminal: an FP64 update is decided and the loop's
                           // kernels skip until the update's K_P has run and reset the status
};

// float -> double, exactly, on the integer pipe for normal numbers: the IEEE 754 binary32 fields
// re-biased into binary64 (exponent + 1023 - 127, fraction shifted up by 29 bits). Zero,
// subnormal, infinite and NaN inputs take the hardware conversion. Same value as
// static_cast<double>(f) in every case; it keeps conversions off GB300's narrow FP64 pipe.
__device__ __forceinline__ double widen(float f) {
    const unsigned u = __float_as_uint(f);
    const unsigned ex = (u >> 23) & 0xffu;
    if (ex - 1u >= 254u) return static_cast<double>(f);
    const unsigned hi = (u & 0x80000000u) | ((ex + (1023u - 127u)) << 20) | ((u & 0x7fffffu) >> 3);
    const unsigned lo = u << 29;
    return __hiloint2double(static_cast<int>(hi), static_cast<int>(lo));
}
__device__ __forceinline__ double widen(double f) { return f; }

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

// Two warp sums for the price of one butterfly: after the exchange at distance 16 lanes 0-15
// carry partial sums of `a` and lanes 16-31 partial sums of `b`, and four more levels finish
// both (5 FP64 adds instead of 10). On return lanes 0-15 hold sum(a) in both outputs and lanes
// 16-31 hold sum(b): read a at lane 0 and b at lane 16. Fixed order: reproducible.
__device__ __forceinline__ void warp_sum2(double &a, double &b, int lane) {
    const bool hi = (lane & 16) != 0;
    double keep = hi ? b : a;
    const double give = hi ? a : b;
    keep += __shfl_xor_sync(0xffffffffu, give, 16);
#pragma unroll
    for (int o = 8; o >= 1; o >>= 1) keep += __shfl_xor_sync(0xffffffffu, keep, o);
    a = keep;
    b = keep;
}

// NQ warp sums at once with a transposed butterfly: at each of the first levels a lane hands
// half of the quantities it still carries to its partner and keeps the other half, so the FP64
// adds per warp are 5 (NQ = 1), 5 (NQ = 2), 6 (NQ = 4) or 9 (NQ = 8) instead of 5 * NQ. On
// return `r` holds, in lanes [q * 32/NQ, (q+1) * 32/NQ), the warp's sum of quantity q. Fixed
// order: reproducible.
template <int NQ>
__device__ __forceinline__ double warp_reduce(const double (&v)[NQ], int lane);
template <>
__device__ __forceinline__ double warp_reduce<1>(const double (&v)[1], int) {
    return warp_sum(v[0]);
}
template <>
__device__ __forceinline__ double warp_reduce<2>(const double (&v)[2], int lane) {
    double a = v[0], b = v[1];
    warp_sum2(a, b, lane);
    return a;
}
template <>
__device__ __forceinline__ double warp_reduce<4>(const double (&v)[4], int lane) {
    const bool h16 = (lane & 16) != 0, h8 = (lane & 8) != 0;
    double k0 = h16 ? v[2] : v[0], k1 = h16 ? v[3] : v[1];
    const double g0 = h16 ? v[0] : v[2], g1 = h16 ? v[1] : v[3];
    k0 += __shfl_xor_sync(0xffffffffu, g0, 16);
    k1 += __shfl_xor_sync(0xffffffffu, g1, 16);
    double k = h8 ? k1 : k0;
    const double g = h8 ? k0 : k1;
    k += __shfl_xor_sync(0xffffffffu, g, 8);
#pragma unroll
    for (int o = 4; o >= 1; o >>= 1) k += __shfl_xor_sync(0xffffffffu, k, o);
    return k;
}
template <>
__device__ __forceinline__ double warp_reduce<8>(const double (&v)[8], int lane) {
    // three halving levels (4 + 2 + 1 adds) leave quantity q in lanes [4q, 4q + 4); two more
    // levels finish it: 9 FP64 adds per warp instead of 40
    double k4[4];
    const bool h16 = (lane & 16) != 0;
#pragma unroll
    for (int i = 0; i < 4; ++i) {
        const double keep = h16 ? v[i + 4] : v[i], give = h16 ? v[i] : v[i + 4];
        k4[i] = keep + __shfl_xor_sync(0xffffffffu, give, 16);
    }
    double k2[2];
    const bool h8 = (lane & 8) != 0;
#pragma unroll
    for (int i = 0; i < 2; ++i) {
        const double keep = h8 ? k4[i + 2] : k4[i], give = h8 ? k4[i] : k4[i + 2];
        k2[i] = keep + __shfl_xor_sync(0xffffffffu, give, 8);
    }
    const bool h4 = (lane & 4) != 0;
    double k = h4 ? k2[1] : k2[0];
    const double g = h4 ? k2[0] : k2[1];
    k += __shfl_xor_sync(0xffffffffu, g, 4);
    k += __shfl_xor_sync(0xffffffffu, k, 2);
    k += __shfl_xor_sync(0xffffffffu, k, 1);
    return k;
}

// Shared-memory doubles a kernel provides to the block reductions below (block_sum stages
// blockDim.x * NC values, up to 512 x 2).
constexpr int kRedScratch = 1024 + 80;

// Sums of NQ values per thread over the first `nwa` warps of the block (nwa <= 16), returned to
// every thread. Each of those warps reduces with warp_reduce, warp 0 adds the per-warp results
// (3-5 more FP64 adds). Fixed order: every block running the same code on the same data gets the
// same bits. Must be called by all threads. scratch: >= 16 * NQ + NQ doubles.
template <int NQ>
__device__ __forceinline__ void group_allreduce(double (&v)[NQ], int nwa, double *scratch) {
    constexpr int G = 32 / NQ;  // lanes per quantity after warp_reduce
    const int t = threadIdx.x, lane = t & 31, w = t >> 5;
    if (w < nwa) {
        const double r = warp_reduce<NQ>(v, lane);
        if ((lane & (G - 1)) == 0) scratch[(lane / G) * 16 + w] = r;
    }
    __syncthreads();
    if (w == 0) {
        const int q = lane / G, i = lane & (G - 1);
        double s = i < nwa ? scratch[q * 16 + i] : 0.0;
        if (G < 16 && nwa > G) s += i + G < nwa ? scratch[q * 16 + i + G] : 0.0;
        // combine the per-warp values held by the G lanes of each quantity (only as many
        // levels as there are warps)
#pragma unroll
        for (int o = 16; o >= 1; o >>= 1)
            if (o < G && o < nwa) s += __shfl_xor_sync(0xffffffffu, s, o);
        if (i == 0) scratch[16 * NQ + q] = s;
    }
    __syncthreads();
#pragma unroll
    for (int q = 0; q < NQ; ++q) v[q] = scratch[16 * NQ + q];
    __syncthreads();
}

// Block-wide sum of NC values per thread (blockDim.x a power of two, 32..512), returned to every
// thread. A dense tree in shared memory -- at each level the lower half of the live threads adds
// the upper half's values, so every FP64 instruction has all its lanes busy -- down to one warp,
// then one warp_reduce. About 15*NC + 5 FP64 warp instructions for 512 threads, against 16*5 for
// a butterfly in every warp. Fixed order.
template <int NC>
__device__ __forceinline__ void block_sum(double (&v)[NC], double *scratch) {
    const int t = threadIdx.x, T = blockDim.x;
#pragma unroll
    for (int c = 0; c < NC; ++c) scratch[c * T + t] = v[c];
    __syncthreads();
    for (int h = T >> 1; h >= 32; h >>= 1) {
        if (t < h) {
#pragma unroll
            for (int c = 0; c < NC; ++c) scratch[c * T + t] += scratch[c * T + t + h];
        }
        __syncthreads();
    }
    double r[NC];
#pragma unroll
    for (int c = 0; c < NC; ++c) r[c] = t < 32 ? scratch[c * T + t] : 0.0;
    __syncthreads();
    group_allreduce<NC>(r, 1, scratch);
#pragma unroll
    for (int c = 0; c < NC; ++c) v[c] = r[c];
}

// One thread's running sums over records i = k, k + K, ... of part[i*S + c] (i < n, c < NC)
// followed by extra[(i-n)*S + c]: the first NC components of records S doubles wide. The first
// record is assigned, not added. ld.global.cg: the records were written by an earlier kernel.
template <int NC, int S = NC>
__device__ __forceinline__ void thread_records(const double *__restrict__ part, int n, const double *__restrict__ extra,
                                               int n_extra, double *s, int k, int K) {
    const int tot = n + n_extra;
    int i = k;
#pragma unroll
    for (int c = 0; c < NC; ++c) s[c] = 0.0;
    if (i < tot) {
        const double *src = i < n ? part + i * S : extra + (i - n) * S;
#pragma unroll
        for (int c = 0; c < NC; ++c) s[c] = __ldcg(src + c);
    }
    for (i += K; i < tot; i += K) {
        const double *src = i < n ? part + i * S : extra + (i - n) * S;
#pragma unroll
        for (int c = 0; c < NC; ++c) s[c] += __ldcg(src + c);
    }
}

// Warps that reduce the partial records: one per scheduler, so the four FP64 pipes share the
// adds and no warp's adds are spent on empty lanes of a mostly idle block.
__device__ __forceinline__ int reducing_warps() { return min(static_cast<int>((blockDim.x + 31) >> 5), 4); }

// Sum of the first NC components of per-block records part[i*S + c] for i in [0, n), plus
// extra[j*S + c] for j in [0, n_extra), computed identically by every calling block and returned
// to every thread. The first four warps take records t, t + 128, ... in order and group_allreduce
// combines them (GB300's FP64 pipe, ~64 cycles per warp instruction per scheduler, is the scarcest
// unit, so only the components a consumer uses are added).
template <int NC, int S = NC>
__device__ __forceinline__ void reduce_partials(const double *__restrict__ part, int n,
                                                const double *__restrict__ extra, int n_extra,
                                                double (&out)[NC], double *scratch /* kRedScratch */) {
    const int nwa = reducing_warps(), K = nwa * 32, t = threadIdx.x;
    if (t < K) thread_records<NC, S>(part, n, extra, n_extra, out, t, K);
    group_allreduce<NC>(out, nwa, scratch);
}

// Two independent reductions in one pass: out[0 .. NA) = the first NA components of records
// part_a (+ extra_a), S_A wide; out[NA .. NA+NB) = the first NB components of records part_b, S_B
// wide; the rest of out[NQ] is zero (NQ a power of two >= NA + NB). One memory round trip and one
// group_allreduce. Same order guarantees as reduce_partials.
template <int NA, int SA, int NB, int SB, int NQ>
__device__ __forceinline__ void reduce_two(const double *__restrict__ part_a, int na, const double *__restrict__ extra_a,
                                           int nea, const double *__restrict__ part_b, int nb, double (&out)[NQ],
                                           double *scratch /* kRedScratch */) {
    static_assert(NA + NB <= NQ, "NQ too small");
    const int nwa = reducing_warps(), K = nwa * 32, t = threadIdx.x;
#pragma unroll
    for (int c = 0; c < NQ; ++c) out[c] = 0.0;
    if (t < K) {
        thread_records<NA, SA>(part_a, na, extra_a, nea, out, t, K);
        thread_records<NB, SB>(part_b, nb, nullptr, 0, out + NA, t, K);
    }
    group_allreduce<NQ>(out, nwa, scratch);
}

__device__ __forceinline__ bool finite_nonzero(double v) { return isfinite(v) && v != 0.0; }

// kern<<<grid, block, smem, stream>>>(args...), returning the launch error.
template <typename... KArgs, typename... Args>
cudaError_t launch_k(void (*kern)(KArgs...), dim3 grid, dim3 block, size_t smem, cudaStream_t stream,
                     Args &&...args) {
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = grid;
    cfg.blockDim = block;
    cfg.dynamicSmemBytes = smem;
    cfg.stream = stream;
    return cudaLaunchKernelEx(&cfg, kern, std::forward<Args>(args)...);
}

}  // namespace hhp
