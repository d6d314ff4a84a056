// hhp_spmv.cu -- CSR SpMV for sm_103a with fused epilogues (FP64 and FP32 values).
//
// Replaces the reference's cuSPARSE call device_csr_spmv (src/util/hhp_cuda.c:226-236) and
// computes what CSR_spmxv_seq computes (src/util/hhp_cpu.c:445-455).
//
// Design (GB300):
//  * Layout: the CSR handed to the library is re-laid out once on the device into slices of
//    H = 32*RPL rows (RPL rows per lane, chosen per matrix: 1-2 for FP64, 2-4 for FP32; column
//    indices as 16-bit offsets from the row where they fit, else int32). Within a slice the j-th
//    nonzero of every row sits next to the j-th nonzero of its slice-mates, so at each step a
//    lane loads the values / column indices of its RPL rows with one vector load (up to 128
//    bits) and the warp's load is one contiguous request: the value and index streams are read
//    from HBM exactly once, fully coalesced, with no shared-memory staging.
//  * Registers instead of staging: every lane keeps UNROLL steps of loads (values, indices, then
//    x gathers through the read-only L1/L2 path) in flight, and the register budget that takes
//    sets the occupancy (3-6 CTAs of 8 warps per SM by instantiation). HBM latency is hidden by
//    warps, not by buffers (shared-memory rings filled by cp.async or TMA measured slower).
//  * Arithmetic: each lane sums each of its rows sequentially in CSR order with fused
//    multiply-adds -- one FP64 FMA per nonzero, the minimum on GB300 whose FP64 rate (~2
//    FMA/clk/SM) is as much a limit as HBM here -- and the RPL independent chains per lane give
//    the FP64 pipe instruction-level parallelism. The result of every such row is bit-identical
//    to the same order computed with fma() on a CPU.
//  * Long rows (> long_thr nonzeros) are cut into chunks that one warp sums (lane-strided, then a
//    fixed butterfly); chunk sums are combined in chunk order by the warp finishing a row's last
//    chunk. Work units (slices and chunks) are dealt to warps at plan time, longest first to the
//    least-loaded warp, so power-law matrices stay balanced; every warp walks a fixed list, so
//    every reduction has a fixed order and results are reproducible run to run. Each list entry
//    carries its slice's start and length, so a slice's streams are requested one dependent load
//    after the warp reads the entry.
//  * Epilogues fuse the BiCGStab dot products (r0.v, t.s, t.t, and r0.t for the merged loop) and
//    the residual r = b - A x into the store of y; one partial per CTA, summed in a fixed order by
//    the consumer.
#include <algorithm>
#include <cstring>
#include <mutex>
#include <type_traits>

#include "hhp_device.cuh"
#include "hhp_internal.h"

namespace hhp {

namespace {

constexpr int kChunkUnroll = 4;

// A lane's words of one slice step: the values (V) and column indices (I: int32 columns; I16:
// 16-bit offsets col - row) of its R rows, each read with one load (32 lanes make one contiguous
// request).
template <typename VT, int R>
struct Vec;
template <>
struct Vec<double, 1> {
    using V = double;
    using I = int;
    using I16 = short;
};
template <>
struct Vec<double, 2> {
    using V = double2;
    using I = int2;
    using I16 = short2;
};
template <>
struct Vec<float, 2> {
    using V = float2;
    using I = int2;
    using I16 = short2;
};
template <>
struct Vec<float, 4> {
    using V = float4;
    using I = int4;
    using I16 = short4;
};

// Loads of the matrix streams (slice values and indices, chunk CSR ranges). FP64 matrices are not
// allocated in L1 (ld.global.nc.L1::no_allocate: L1 stays with the x gathers; measured faster in
// the FP64 solves); FP32 ones take the default read-only path (their solves measured slower
// without L1 allocation).
template <typename VT, typename T>
__device__ __forceinline__ T ld_stream(const T *p) {
    static_assert(sizeof(T) == 2 || sizeof(T) == 4 || sizeof(T) == 8 || sizeof(T) == 16, "2 to 16 bytes");
    if (!std::is_same<VT, double>::value) return __ldg(p);
    T out;
    if (sizeof(T) == 2) {
        unsigned short r;
        asm volatile("ld.global.nc.L1::no_allocate.b16 %0, [%1];" : "=h"(r) : "l"(p));
        memcpy(&out, &r, 2);
    } else if (sizeof(T) == 4) {
        uint32_t r;
        asm volatile("ld.global.nc.L1::no_allocate.b32 %0, [%1];" : "=r"(r) : "l"(p));
        memcpy(&out, &r, 4);
    } else if (sizeof(T) == 8) {
        uint32_t r[2];
        asm volatile("ld.global.nc.L1::no_allocate.v2.b32 {%0, %1}, [%2];" : "=r"(r[0]), "=r"(r[1]) : "l"(p));
        memcpy(&out, r, 8);
    } else {
        uint32_t r[4];
        asm volatile("ld.global.nc.L1::no_allocate.v4.b32 {%0, %1, %2, %3}, [%4];"
                     : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3])
                     : "l"(p));
        memcpy(&out, r, 16);
    }
    return out;
}

template <typename VT>
struct SellArgs {
    const long long *slice_ptr;
    const int *pos_row;
    const int *pos_len;
    const int *warp_ptr;
    const int *warp_units;
    const int4 *unit_rec;
    const VT *sval;
    const int *scol;       // int32 columns, or
    const short *scol16;   // 16-bit offsets col - row (plans whose every |col - row| < 2^15)
    const VT *csr_val;  // CSR values (FP64, or the FP32 copy) for long-row chunks
    const int *csr_col;
    const int4 *chunks;
    const int *long_first;
    const int *chunk_long;
    double *chunk_part;
    unsigned *long_cnt;
    double *long_dot;
    unsigned *group_cnt;  // per group of kLongGroup long rows: rows finished this launch
    double *group_dot;    // per group: the fixed-order sum of its rows' long_dot records
    double *cta_part;
    const VT *x;
    VT *y;
    const VT *w1;
    const VT *w2;      // EP_DOT3's second dot operand
    double alpha, beta;
    int scale, accum;  // alpha != 1, beta != 0 (decided on the host)
    const int *gate;   // nullable: skip the whole launch when *gate == 0
    const int *stop;   // nullable: skip the whole launch when *stop != 0
    int *err;
    int m, n_slices, n_chunks, n_long;
    bool has_perm;
    int doff[kMaxDiag];  // uniform-diagonal plans: the diagonals' offsets (pos_len then holds row masks)
};

__device__ __forceinline__ double vfma(double a, double b, double c) { return fma(a, b, c); }
__device__ __forceinline__ float vfma(float a, float b, float c) { return fmaf(a, b, c); }

template <typename V, typename T>
__device__ __forceinline__ T comp(const V &v, int t) {
    return reinterpret_cast<const T *>(&v)[t];
}

// Row epilogue: stores y[r]; accumulates dot partials into (d0, d1, d2), in the value type (the
// caller folds them into FP64 once per slice for FP32 data).
template <typename VT, int EP, typename DT>
__device__ __forceinline__ void row_epilogue(const SellArgs<VT> &a, int r, VT acc, DT &d0, DT &d1, DT &d2,
                                             VT w1r, VT w2r) {
    if (EP == EP_Y) {
        a.y[r] = acc;
    } else if (EP == EP_AXPBY) {
        VT out = acc;
        if (a.scale) out = static_cast<VT>(a.alpha) * out;  // integer flags: no FP64 compares per row
        if (a.accum) out = vfma(static_cast<VT>(a.beta), a.y[r], out);
        a.y[r] = out;
    } else if (EP == EP_DOT1) {
        a.y[r] = acc;
        d0 = vfma(static_cast<DT>(acc), static_cast<DT>(w1r), d0);
    } else if (EP == EP_DOT2) {
        a.y[r] = acc;
        d0 = vfma(static_cast<DT>(acc), static_cast<DT>(w1r), d0);
        d1 = vfma(static_cast<DT>(acc), static_cast<DT>(acc), d1);
    } else if (EP == EP_DOT3) {
        a.y[r] = acc;
        d0 = vfma(static_cast<DT>(acc), static_cast<DT>(w1r), d0);
        d1 = vfma(static_cast<DT>(acc), static_cast<DT>(acc), d1);
        d2 = vfma(static_cast<DT>(acc), static_cast<DT>(w2r), d2);
    } else {  // EP_RESID
        const VT b = w1r;
        const VT res = b - acc;
        a.y[r] = res;
        d0 = vfma(static_cast<DT>(res), static_cast<DT>(res), d0);
        d1 = vfma(static_cast<DT>(b), static_cast<DT>(b), d1);
    }
}

template <typename VT, int R, int U, int EP, bool D16, bool UNI>
__device__ __forceinline__ void do_slice(const SellArgs<VT> &a, int s, long long base, int wmax, int lane,
                                         double &d0, double &d1, double &d2) {
    using VV = typename Vec<VT, R>::V;
    using IV = typename Vec<VT, R>::I;
    using CW = typename std::conditional<D16, typename Vec<VT, R>::I16, IV>::type;  // index word
    using CT = typename std::conditional<D16, short, int>::type;
    constexpr int H = 32 * R;
    // base: the slice's first stored word; wmax: its longest row, every lane walks this many
    // steps (uniform across the warp)
    const int q0 = s * H + lane * R;
    const IV lv = *reinterpret_cast<const IV *>(a.pos_len + q0);
    int len[R], row[R];
#pragma unroll
    for (int t = 0; t < R; ++t) len[t] = comp<IV, int>(lv, t);
    if (a.has_perm) {
        const IV rv = *reinterpret_cast<const IV *>(a.pos_row + q0);
#pragma unroll
        for (int t = 0; t < R; ++t) row[t] = comp<IV, int>(rv, t);
    } else {
#pragma unroll
        for (int t = 0; t < R; ++t) row[t] = q0 + t;
    }
    // column of row t's entry in an index word: stored, or the row plus a 16-bit offset
    auto colof = [&](const CW &w, int t) -> int {
        return D16 ? row[t] + static_cast<int>(comp<CW, CT>(w, t)) : static_cast<int>(comp<CW, CT>(w, t));
    };
    // the epilogue's vector operands, requested before the slice's main loop so that their
    // latency is hidden behind it
    // (only where the registers allow: the wide-unroll instantiations)
    constexpr bool W1 = EP == EP_DOT1 || EP == EP_DOT2 || EP == EP_DOT3 || EP == EP_RESID;
    constexpr bool EARLY = R * U >= 8;
    VT w1v[R], w2v[R];
    auto load_w = [&]() {
#pragma unroll
        for (int t = 0; t < R; ++t) {
            const bool ok = row[t] >= 0 && row[t] < a.m;
            w1v[t] = (W1 && ok) ? __ldg(a.w1 + row[t]) : VT(0);
            w2v[t] = (EP == EP_DOT3 && ok) ? __ldg(a.w2 + row[t]) : VT(0);
        }
    };
    if constexpr (EARLY) load_w();
    const VV *vp = reinterpret_cast<const VV *>(a.sval + base) + lane;
    VT acc[R];
#pragma unroll
    for (int t = 0; t < R; ++t) acc[t] = VT(0);
    if constexpr (UNI) {
        // Uniform diagonals: step k of every row is its entry on diagonal doff[k] (the column is
        // the row plus that offset; no index stream), absent where bit k of the row's mask is
        // clear -- no gather and no multiply-add there, so every row still sums exactly its
        // stored entries in CSR order. pos_len holds the masks.
        int mk[R];
#pragma unroll
        for (int t = 0; t < R; ++t) mk[t] = len[t];
        VV v[U];
#pragma unroll
        for (int u = 0; u < U; ++u) v[u] = u < wmax ? ld_stream<VT>(vp + static_cast<size_t>(u) * 32) : VV();
        int j = 0;
        for (; j + U <= wmax; j += U) {
            VV vn[U];
#pragma unroll
            for (int u = 0; u < U; ++u) {
                const int jn = j + U + u;
                vn[u] = jn < wmax ? ld_stream<VT>(vp + static_cast<size_t>(jn) * 32) : VV();
            }
            VT xv[U][R];
#pragma unroll
            for (int u = 0; u < U; ++u) {
                const int off = a.doff[j + u];
#pragma unroll
                for (int t = 0; t < R; ++t) xv[u][t] = ((mk[t] >> (j + u)) & 1) ? __ldg(a.x + row[t] + off) : VT(0);
            }
#pragma unroll
            for (int u = 0; u < U; ++u)
#pragma unroll
                for (int t = 0; t < R; ++t)
                    if ((mk[t] >> (j + u)) & 1) acc[t] = vfma(comp<VV, VT>(v[u], t), xv[u][t], acc[t]);
#pragma unroll
            for (int u = 0; u < U; ++u) v[u] = vn[u];
        }
#pragma unroll 1
        for (; j < wmax; ++j) {
            const VV vt = ld_stream<VT>(vp + static_cast<size_t>(j) * 32);
            const int off = a.doff[j];
            VT xt[R];
#pragma unroll
            for (int t = 0; t < R; ++t) xt[t] = ((mk[t] >> j) & 1) ? __ldg(a.x + row[t] + off) : VT(0);
#pragma unroll
            for (int t = 0; t < R; ++t)
                if ((mk[t] >> j) & 1) acc[t] = vfma(comp<VV, VT>(vt, t), xt[t], acc[t]);
        }
    } else {
    const CW *cp = D16 ? reinterpret_cast<const CW *>(a.scol16 + base) + lane
                       : reinterpret_cast<const CW *>(a.scol + base) + lane;
    // Software pipeline over full groups of U steps: the values and indices of group g+1
    // are requested before the gathers and multiply-adds of group g, so the HBM latency of the
    // streams overlaps the L1/L2 latency of the gathers (warps issue in order: a load placed
    // after a stalled FMA would wait for it). The last wmax % U steps run one at a time
    // after the loop: a multiply-add predicated off still occupies GB300's FP64 pipe for a full
    // warp slot, so no group is ever padded with dead steps.
    VV v[U];
    CW c[U];
#pragma unroll
    for (int u = 0; u < U; ++u) {
        v[u] = u < wmax ? ld_stream<VT>(vp + static_cast<size_t>(u) * 32) : VV();
        c[u] = u < wmax ? ld_stream<VT>(cp + static_cast<size_t>(u) * 32) : CW();
    }
    int j = 0;
    for (; j + U <= wmax; j += U) {
        VV vn[U];
        CW cn[U];
#pragma unroll
        for (int u = 0; u < U; ++u) {
            const int jn = j + U + u;
            vn[u] = jn < wmax ? ld_stream<VT>(vp + static_cast<size_t>(jn) * 32) : VV();
            cn[u] = jn < wmax ? ld_stream<VT>(cp + static_cast<size_t>(jn) * 32) : CW();
        }
        VT xv[U][R];
#pragma unroll
        for (int u = 0; u < U; ++u)
#pragma unroll
            for (int t = 0; t < R; ++t) xv[u][t] = (j + u < len[t]) ? __ldg(a.x + colof(c[u], t)) : VT(0);
#pragma unroll
        for (int u = 0; u < U; ++u)
#pragma unroll
            for (int t = 0; t < R; ++t)
                if (j + u < len[t]) acc[t] = vfma(comp<VV, VT>(v[u], t), xv[u][t], acc[t]);
#pragma unroll
        for (int u = 0; u < U; ++u) {
            v[u] = vn[u];
            c[u] = cn[u];
        }
    }
    // tail steps, one at a time (their words were requested by the last prefetch)
#pragma unroll 1
    for (; j < wmax; ++j) {
        const VV vt = ld_stream<VT>(vp + static_cast<size_t>(j) * 32);
        const CW ct = ld_stream<VT>(cp + static_cast<size_t>(j) * 32);
        VT xt[R];
#pragma unroll
        for (int t = 0; t < R; ++t) xt[t] = (j < len[t]) ? __ldg(a.x + colof(ct, t)) : VT(0);
#pragma unroll
        for (int t = 0; t < R; ++t)
            if (j < len[t]) acc[t] = vfma(comp<VV, VT>(vt, t), xt[t], acc[t]);
    }
    }
    if constexpr (!EARLY) load_w();
    VT e0 = VT(0), e1 = VT(0), e2 = VT(0);
#pragma unroll
    for (int t = 0; t < R; ++t) {
        const int r = row[t];
        if (r >= 0 && r < a.m) row_epilogue<VT, EP>(a, r, acc[t], e0, e1, e2, w1v[t], w2v[t]);
    }
    if (EP != EP_AXPBY && EP != EP_Y) {
        d0 += widen(e0);
        d1 += widen(e1);
    }
    if (EP == EP_DOT3) d2 += widen(e2);
}

// Long rows' epilogue records are folded by groups of kLongGroup consecutive long rows: the warp
// that completes the last row of a group sums the group's records, one per lane, with a fixed
// butterfly, so consumers reduce n_long / kLongGroup records instead of n_long (a 3.5M-row power
// law has ~4600 long rows: their records made every consumer block's reduction several times
// longer than the vector work it precedes).
template <typename VT, int EP>
__device__ __forceinline__ void fold_long_group(const SellArgs<VT> &a, int l, int lane) {
    constexpr int S = EP == EP_DOT3 ? 4 : 2;
    const int g = l / kLongGroup, first = g * kLongGroup, size = min(kLongGroup, a.n_long - first);
    unsigned last = 0;
    if (lane == 0) {
        __threadfence();  // this row's long_dot record before the group count
        last = atomicAdd(&a.group_cnt[g], 1u) == static_cast<unsigned>(size - 1);
    }
    last = __shfl_sync(0xffffffffu, last, 0);
    if (!last) return;
    __threadfence();
    const double *rec = a.long_dot + static_cast<size_t>(first + lane) * S;
    if (EP == EP_DOT3) {
        const double v[4] = {lane < size ? __ldcg(rec) : 0.0, lane < size ? __ldcg(rec + 1) : 0.0,
                             lane < size ? __ldcg(rec + 2) : 0.0, 0.0};
        const double r = warp_reduce<4>(v, lane);  // quantity q in lanes [8q, 8q + 8)
        if ((lane & 7) == 0) a.group_dot[static_cast<size_t>(g) * 4 + (lane >> 3)] = r;
    } else {
        double d0 = lane < size ? __ldcg(rec) : 0.0, d1 = lane < size ? __ldcg(rec + 1) : 0.0;
        warp_sum2(d0, d1, lane);
        if (lane == 0) a.group_dot[static_cast<size_t>(g) * 2] = d0;
        if (lane == 16) a.group_dot[static_cast<size_t>(g) * 2 + 1] = d1;
    }
    if (lane == 0) a.group_cnt[g] = 0u;  // ready for the next launch
}

template <typename VT, int EP>
__device__ __forceinline__ void do_chunk(const SellArgs<VT> &a, int c, int lane) {
    const int4 d = __ldg(&a.chunks[c]);
    VT acc = VT(0);
    for (int k = d.z + lane; k < d.w; k += 32 * kChunkUnroll) {
        VT v[kChunkUnroll], xv[kChunkUnroll];
        int cc[kChunkUnroll];
#pragma unroll
        for (int u = 0; u < kChunkUnroll; ++u) {
            const int kk = k + 32 * u;
            v[u] = kk < d.w ? ld_stream<VT>(a.csr_val + kk) : VT(0);
            cc[u] = kk < d.w ? ld_stream<VT>(a.csr_col + kk) : 0;
        }
#pragma unroll
        for (int u = 0; u < kChunkUnroll; ++u) xv[u] = (k + 32 * u < d.w) ? __ldg(a.x + cc[u]) : VT(0);
#pragma unroll
        for (int u = 0; u < kChunkUnroll; ++u)
            if (k + 32 * u < d.w) acc = vfma(v[u], xv[u], acc);
    }
    acc = warp_sum(acc);
    int done = -1;  // the long row this warp completed (its epilogue record written), else -1
    if (lane == 0) {
        const int cid = d.y;
        a.chunk_part[cid] = static_cast<double>(acc);
        __threadfence();
        const int l = a.chunk_long[cid];
        const int c_first = a.long_first[l], nch = a.long_first[l + 1] - c_first;
        const unsigned prev = atomicAdd(&a.long_cnt[l], 1u);
        if (prev == static_cast<unsigned>(nch - 1)) {
            __threadfence();
            double tot = 0.0;
            for (int q = 0; q < nch; ++q) tot += __ldcg(a.chunk_part + c_first + q);
            a.long_cnt[l] = 0u;  // ready for the next launch
            double e0 = 0.0, e1 = 0.0, e2 = 0.0;
            constexpr bool W1 = EP == EP_DOT1 || EP == EP_DOT2 || EP == EP_DOT3 || EP == EP_RESID;
            const VT w1r = W1 ? __ldg(a.w1 + d.x) : VT(0), w2r = EP == EP_DOT3 ? __ldg(a.w2 + d.x) : VT(0);
            row_epilogue<VT, EP, double>(a, d.x, static_cast<VT>(tot), e0, e1, e2, w1r, w2r);
            if (EP == EP_DOT3) {
                a.long_dot[4 * l] = e0;
                a.long_dot[4 * l + 1] = e1;
                a.long_dot[4 * l + 2] = e2;
                a.long_dot[4 * l + 3] = 0.0;
            } else if (EP != EP_AXPBY && EP != EP_Y) {
                a.long_dot[2 * l] = e0;
                a.long_dot[2 * l + 1] = e1;
            }
            done = l;
        }
    }
    if (EP != EP_AXPBY && EP != EP_Y) {
        done = __shfl_sync(0xffffffffu, done, 0);
        if (done >= 0) fold_long_group<VT, EP>(a, done, lane);
    }
}

// Resident CTAs of 256 threads that the register need of R*U words in flight per lane allows.
template <int R, int U>
struct MinCtas {
    static constexpr int value = R * U >= 8 ? 3 : (R * U >= 4 ? 5 : 6);
};

// Uniform-diagonal slices carry no index words: the wide FP32 layouts (R * U >= 8) then fit 4 CTAs
// of 256 threads per SM in 64 registers without spills, and the plan launches 4 (the mixed solve
// of the 160^3 7-point stencil: 127.9 -> 121.1 us per inner iteration). FP64 keeps its counts (the stencil layout, R * U = 4,
// runs 5; the wide FP64 one would spill at 64 registers).
template <typename VT, int R, int U, bool UNI>
struct MinCtasFor {
    static constexpr int value = UNI && sizeof(VT) == 4 && R * U >= 8 ? 4 : MinCtas<R, U>::value;
};

template <typename VT, int R, int U, int EP, bool D16, bool UNI = false>
__global__ void __launch_bounds__(256, MinCtasFor<VT, R, U, UNI>::value) k_spmv(const SellArgs<VT> a) {
    // After a recorded device error, with the gate closed, or once the solver's status is
    // terminal, the launch returns at once (uniform across the grid). The three words were
    // written by earlier launches: read together (one memory latency, not three), through L2.
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
    const int gw = blockIdx.x * nw + warp;
    // this warp's units, balanced at plan time (fixed order: reductions are reproducible); read
    // with the skip words, on which they do not depend
    const int ub = __ldg(a.warp_ptr + gw), ue = __ldg(a.warp_ptr + gw + 1);
    const int err = __ldcg(a.err), gate = a.gate ? __ldcg(a.gate) : 1, stop = a.stop ? __ldcg(a.stop) : 0;
    if (err != DEV_OK || gate == 0 || stop != 0) return;
    __shared__ double red[32];
    double d0 = 0.0, d1 = 0.0, d2 = 0.0;
    for (int i = ub; i < ue; ++i) {
        const int4 rec = __ldg(a.unit_rec + i);
        // the next record is pulled into L1 while this unit runs (no registers held for it)
        if (i + 1 < ue) asm volatile("prefetch.global.L1 [%0];" ::"l"(a.unit_rec + i + 1));
        const int u = rec.x;
        if (u < a.n_slices) {
            const long long base = static_cast<long long>(static_cast<unsigned>(rec.z)) |
                                   (static_cast<long long>(rec.w) << 32);
            do_slice<VT, R, U, EP, D16, UNI>(a, u, base, rec.y, lane, d0, d1, d2);
        } else {
            do_chunk<VT, EP>(a, u - a.n_slices, lane);
        }
    }
    if (EP == EP_DOT3) {
        // records of 4: (d0, d1, d2, 0); each warp's transposed butterfly leaves quantity q in
        // lanes [8q, 8q + 8), warp 0 adds the warps' results within each group of 8 lanes
        const double dv[4] = {d0, d1, d2, 0.0};
        const double r = warp_reduce<4>(dv, lane);
        if ((lane & 7) == 0) red[lane + warp] = r;  // red[8q + warp], nw <= 8
        __syncthreads();
        if (warp == 0) {
            double s = (lane < 24 && (lane & 7) < nw) ? red[lane] : 0.0;
#pragma unroll
            for (int o = 4; o >= 1; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
            if ((lane & 7) == 0) a.cta_part[4 * blockIdx.x + (lane >> 3)] = s;
        }
    } else if (EP != EP_AXPBY && EP != EP_Y) {
        // per-CTA partial: each warp folds its lanes' (d0, d1) with a transposed butterfly
        // (5 FP64 adds for both sums), warp 0 adds the warps' results; fixed order throughout
        warp_sum2(d0, d1, lane);
        if (lane == 0) red[warp] = d0;
        if (lane == 16) red[8 + warp] = d1;
        __syncthreads();
        if (warp == 0) {
            // lanes 0-7 take the warps' d0 sums, lanes 8-15 their d1 sums (nw <= 8 warps)
            double s = (lane < 16 && (lane & 7) < nw) ? red[lane] : 0.0;
#pragma unroll
            for (int o = 4; o >= 1; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
            if (lane == 0) a.cta_part[2 * blockIdx.x] = s;
            if (lane == 8) a.cta_part[2 * blockIdx.x + 1] = s;
        }
    }
}

template <typename VT, int R, int U, bool D16, bool UNI = false>
cudaError_t launch_rud(EpKind ep, const PlanDev &p, const SellArgs<VT> &a, cudaStream_t s) {
    const dim3 grid(p.ctas), block(p.warps_per_cta * 32);
    switch (ep) {
        case EP_DOT1: return launch_k(k_spmv<VT, R, U, EP_DOT1, D16, UNI>, grid, block, 0, s, a);
        case EP_DOT2: return launch_k(k_spmv<VT, R, U, EP_DOT2, D16, UNI>, grid, block, 0, s, a);
        case EP_DOT3: return launch_k(k_spmv<VT, R, U, EP_DOT3, D16, UNI>, grid, block, 0, s, a);
        case EP_RESID: return launch_k(k_spmv<VT, R, U, EP_RESID, D16, UNI>, grid, block, 0, s, a);
        default:
            // y = A x needs no epilogue arithmetic: a separate instantiation keeps the FP64 pipe
            // free of predicated-off scale and accumulate instructions
            if (!a.scale && !a.accum) return launch_k(k_spmv<VT, R, U, EP_Y, D16, UNI>, grid, block, 0, s, a);
            return launch_k(k_spmv<VT, R, U, EP_AXPBY, D16, UNI>, grid, block, 0, s, a);
    }
}

// Index mode from the plan: uniform diagonals (no index stream; plans with R >= 2 only, the
// layouts of short regular rows), 16-bit offsets, or int32 columns.
template <typename VT, int R, int U>
cudaError_t launch_ru(EpKind ep, const PlanDev &p, const SellArgs<VT> &a, cudaStream_t s) {
    if constexpr (R >= 2) {
        if (p.uni) return launch_rud<VT, R, U, false, true>(ep, p, a, s);
    }
    return p.d16 ? launch_rud<VT, R, U, true>(ep, p, a, s) : launch_rud<VT, R, U, false>(ep, p, a, s);
}

// Rows per lane come from the plan, the unroll from the tuning (2 or 4 steps in flight per lane).
template <typename VT>
cudaError_t launch_ep(EpKind ep, const PlanDev &p, const SellArgs<VT> &a, cudaStream_t s) {
    const bool u2 = p.unroll == 2;
    if constexpr (std::is_same<VT, double>::value) {
        if (p.rpl == 1) return u2 ? launch_ru<VT, 1, 2>(ep, p, a, s) : launch_ru<VT, 1, 4>(ep, p, a, s);
        return u2 ? launch_ru<VT, 2, 2>(ep, p, a, s) : launch_ru<VT, 2, 4>(ep, p, a, s);
    } else {
        if (p.rpl == 2) return u2 ? launch_ru<VT, 2, 2>(ep, p, a, s) : launch_ru<VT, 2, 4>(ep, p, a, s);
        return u2 ? launch_ru<VT, 4, 2>(ep, p, a, s) : launch_ru<VT, 4, 4>(ep, p, a, s);
    }
}

// Device re-layout: position p of the slices <- row pos_row[p] of the CSR (values cast to VT).
template <typename VT>
__global__ void k_sell_fill(const int *__restrict__ rowptr, const int *__restrict__ col, const double *__restrict__ val,
                            const int *__restrict__ pos_row, const int *__restrict__ pos_len,
                            const long long *__restrict__ slice_ptr, int H, long long npos, VT *sval, int *scol,
                            short *scol16) {
    for (long long p = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; p < npos;
         p += static_cast<long long>(gridDim.x) * blockDim.x) {
        const int r = pos_row[p], len = pos_len[p];
        if (r < 0 || len == 0) continue;
        const long long s = p / H, q = p % H;
        const long long dst = slice_ptr[s] + q;
        const int src = rowptr[r];
        for (int j = 0; j < len; ++j) {
            const long long d = dst + static_cast<long long>(j) * H;
            sval[d] = static_cast<VT>(val[src + j]);
            if (scol) scol[d] = col[src + j];
            if (scol16) scol16[d] = static_cast<short>(col[src + j] - r);
        }
    }
}

// Uniform-diagonal re-layout: row r's entry on diagonal doff[k] goes to step k of its slice (rows
// in natural order, slices K steps wide; absent entries stay zero and masked off).
struct DiagSet {
    int K;
    int d[kMaxDiag];
};
template <typename VT>
__global__ void k_sell_fill_uni(const int *__restrict__ rowptr, const int *__restrict__ col,
                                const double *__restrict__ val, int m, int H, DiagSet ds, VT *sval) {
    for (int r = blockIdx.x * blockDim.x + threadIdx.x; r < m; r += gridDim.x * blockDim.x) {
        const long long dst = static_cast<long long>(r / H) * ds.K * H + r % H;
        for (int p = rowptr[r]; p < rowptr[r + 1]; ++p) {
            const int o = col[p] - r;
            int k = 0;
            while (k + 1 < ds.K && ds.d[k] != o) ++k;
            sval[dst + static_cast<long long>(k) * H] = static_cast<VT>(val[p]);
        }
    }
}

// bad[0] = 1 if some entry of a row with at most long_thr entries has |col - row| >= 2^15.
__global__ void k_offsets_fit(const int *__restrict__ rowptr, const int *__restrict__ col, int m, int long_thr,
                              int *bad) {
    for (int r = blockIdx.x * blockDim.x + threadIdx.x; r < m; r += gridDim.x * blockDim.x) {
        const int b = rowptr[r], e = rowptr[r + 1];
        if (e - b > long_thr) continue;  // long rows are read from the CSR
        for (int k = b; k < e; ++k) {
            const int d = col[k] - r;
            if (d > 32767 || d < -32767) {
                *bad = 1;
                break;
            }
        }
    }
}

// Device copy of a host vector (zero-padded to min_elems), ordered on `st`: the library's streams
// are non-blocking, so zero fills or copies on the legacy default stream would not be ordered
// before the kernels that read these arrays.
template <typename T>
hhp_status upload(T **dst, const std::vector<T> &src, cudaStream_t st, size_t min_elems = 1) {
    const size_t n = std::max(src.size(), min_elems);
    HHP_CUDA(cudaMalloc(reinterpret_cast<void **>(dst), n * sizeof(T)));
    HHP_CUDA(cudaMemsetAsync(*dst, 0, n * sizeof(T), st));
    if (!src.empty()) HHP_CUDA(cudaMemcpyAsync(*dst, src.data(), src.size() * sizeof(T), cudaMemcpyHostToDevice, st));
    return HHP_OK;
}

template <typename VT>
hhp_status fill_values(hhp_mat *A, PlanDev &p, bool with_cols) {
    const long long npos = static_cast<long long>(p.n_slices) * p.H;
    if (npos == 0) return HHP_OK;
    if (p.uni) {
        DiagSet ds;
        ds.K = p.K;
        for (int k = 0; k < kMaxDiag; ++k) ds.d[k] = p.doff[k];
        const int grid = static_cast<int>(std::min<long long>((A->m + 255) / 256, 8LL * A->ctx->num_sms));
        k_sell_fill_uni<VT><<<grid, 256, 0, A->ctx->stream>>>(A->rowptr, A->col, A->val, A->m, p.H, ds,
                                                              static_cast<VT *>(p.sval));
        HHP_CUDA(cudaGetLastError());
        return HHP_OK;
    }
    const int grid = static_cast<int>(std::min<long long>((npos + 255) / 256, 8LL * A->ctx->num_sms));
    k_sell_fill<VT><<<grid, 256, 0, A->ctx->stream>>>(A->rowptr, A->col, A->val, p.pos_row, p.pos_len, p.slice_ptr,
                                                      p.H, npos, static_cast<VT *>(p.sval),
                                                      with_cols ? p.scol : nullptr, with_cols ? p.scol16 : nullptr);
    HHP_CUDA(cudaGetLastError());
    return HHP_OK;
}

template <typename VT>
hhp_status build_plan_dev(hhp_mat *A, PlanDev &p) {
    const Tuning &t = tuning();
    hhp_ctx *ctx = A->ctx;
    // Layout and launch shape, measured on GB300 over the banded, power-law and stencil workloads
    // (environment knobs override each choice). FP32: 4 rows per lane (16-byte words), 4 steps in
    // flight, 3 CTAs per SM. FP64: short regular rows (stencils: no long rows, no length sorting
    // needed, under 10 nonzeros per row) take 2 rows per lane, 2 steps, 5 CTAs; length-sorted
    // matrices (power-law rows) 1 row per lane, 4 steps, 5 CTAs, so more warps share the
    // scattered gathers; others (banded) 2 rows per lane, 4 steps, 3 CTAs.
    SellHost h;
    int R, U, cps;
    if (std::is_same<VT, double>::value) {
        build_plan(A->m, A->rowptr_host.data(), 2, std::max(t.long_thr, 1), std::max(t.cap, 32),
                   std::max(t.window, 1), h);
        const bool regular = h.long_rows.empty() && !h.sorted && A->nnz < 10LL * std::max(A->m, 1);
        R = t.rpl64 == 1 || t.rpl64 == 2 ? t.rpl64 : (h.sorted && !regular ? 1 : 2);
        U = t.spmv_unroll == 2 || t.spmv_unroll == 4 ? t.spmv_unroll : (regular ? 2 : 4);
        cps = t.ctas_per_sm > 0 ? t.ctas_per_sm : (regular || R == 1 ? 5 : 3);
        if (R != 2)
            build_plan(A->m, A->rowptr_host.data(), R, std::max(t.long_thr, 1), std::max(t.cap, 32),
                       std::max(t.window, 1), h);
    } else {
        R = t.rpl32 == 2 ? 2 : 4;
        U = t.spmv_unroll == 2 || t.spmv_unroll == 4 ? t.spmv_unroll : 4;
        cps = t.ctas_per_sm > 0 ? t.ctas_per_sm : 3;
        build_plan(A->m, A->rowptr_host.data(), R, std::max(t.long_thr, 1), std::max(t.cap, 32),
                   std::max(t.window, 1), h);
    }
    // Uniform diagonals (stencils): every entry on one of at most kMaxDiag diagonals, rows in
    // natural order, no long rows. The slices then store values only, K steps each (step k =
    // diagonal doff[k]), and pos_len holds each row's bit mask of present diagonals. The column
    // check reads a prefix first, so a matrix with scattered columns costs one small copy.
    bool uni = false;
    int K = 0, doff[kMaxDiag] = {};
    if (t.uni && R >= 2 && h.long_rows.empty() && !h.has_perm && !h.sorted && A->m > 0 && A->nnz > 0) {
        std::vector<int> hc;
        std::vector<int> mask;
        const std::vector<int> &rp = A->rowptr_host;
        int m_pre = static_cast<int>(std::upper_bound(rp.begin(), rp.end(), 65536) - rp.begin()) - 1;
        m_pre = std::max(1, std::min(m_pre, A->m));
        const size_t n_pre = static_cast<size_t>(rp[static_cast<size_t>(m_pre)]);
        hc.resize(static_cast<size_t>(A->nnz));
        HHP_CUDA(cudaStreamSynchronize(ctx->stream));
        HHP_CUDA(cudaMemcpy(hc.data(), A->col, sizeof(int) * n_pre, cudaMemcpyDeviceToHost));
        if (uniform_diagonals(m_pre, rp.data(), hc.data(), kMaxDiag, 0.10, doff, K, mask)) {
            HHP_CUDA(cudaMemcpy(hc.data() + n_pre, A->col + n_pre, sizeof(int) * (hc.size() - n_pre),
                                cudaMemcpyDeviceToHost));
            uni = uniform_diagonals(A->m, rp.data(), hc.data(), kMaxDiag, 0.10, doff, K, mask);
        }
        if (uni) {
            for (int s2 = 0; s2 <= h.n_slices; ++s2)
                h.slice_ptr[static_cast<size_t>(s2)] = static_cast<long long>(s2) * K * h.H;
            h.total = static_cast<long long>(h.n_slices) * K * h.H;
            for (size_t q = 0; q < h.pos_len.size(); ++q)
                h.pos_len[q] = q < static_cast<size_t>(A->m) ? mask[q] : 0;
            h.padding = static_cast<double>(h.total) / static_cast<double>(A->nnz);
        }
    }
    if (uni && !std::is_same<VT, double>::value && R * U >= 8 && t.ctas_per_sm <= 0) cps = 4;
    p.release();
    p.uni = uni;
    p.K = K;
    for (int k = 0; k < kMaxDiag; ++k) p.doff[k] = doff[k];
    p.rpl = R;
    p.unroll = U;
    p.H = h.H;
    p.n_slices = h.n_slices;
    p.n_long = static_cast<int>(h.long_rows.size());
    p.n_chunks = static_cast<int>(h.chunks.size());
    p.has_perm = h.has_perm;
    p.sorted = h.sorted;
    p.total = h.total;
    p.padding = h.padding;
    p.warps_per_cta = std::min(std::max(t.wpc, 1), 8);
    // A small matrix gets no more CTAs than it has work units for its warps: every CTA writes a
    // partial record that every consumer of the epilogue's dot products reduces, and a 65k-row
    // stencil (1024 slices) on 5 CTAs per SM left 5 of every 6 warps idle while its consumers
    // reduced 760 records (that solve: 27.7 -> 24.4 us per iteration on one CTA per SM)
    if (t.ctas_per_sm <= 0) {
        const long long units = static_cast<long long>(h.n_slices) + static_cast<long long>(h.chunks.size());
        const long long per_cps = static_cast<long long>(ctx->num_sms) * p.warps_per_cta;
        cps = static_cast<int>(std::max(1LL, std::min<long long>(cps, (units + per_cps - 1) / per_cps)));
        // One unit per warp, one CTA per SM: the launch is as long as one warp's chain of
        // dependent loads, so every step of a stencil row goes out at once rather than in pairs
        // (65k-row 5-point stencil: 24.4 -> 23.5 us per solve iteration). Registers are no
        // constraint at this occupancy.
        if (units <= per_cps && t.spmv_unroll != 2) p.unroll = 4;
    }
    p.ctas = ctx->num_sms * std::min(std::max(cps, 1), 8);
    std::vector<int> wptr, wunits;
    assign_units(h, p.ctas * p.warps_per_cta, wptr, wunits, &p.imbalance);
    HHP_TRY(upload(&p.warp_ptr, wptr, ctx->stream));
    HHP_TRY(upload(&p.warp_units, wunits, ctx->stream));
    {
        std::vector<int4> rec(wunits.size());
        for (size_t i = 0; i < wunits.size(); ++i) {
            const int u = wunits[i];
            if (u < h.n_slices) {
                const long long b = h.slice_ptr[static_cast<size_t>(u)];
                const int steps = static_cast<int>((h.slice_ptr[static_cast<size_t>(u) + 1] - b) / h.H);
                rec[i] = make_int4(u, steps, static_cast<int>(static_cast<unsigned>(b & 0xffffffffLL)),
                                   static_cast<int>(b >> 32));
            } else {
                rec[i] = make_int4(u, 0, 0, 0);
            }
        }
        HHP_TRY(upload(&p.unit_rec, rec, ctx->stream));
    }
    HHP_TRY(upload(&p.slice_ptr, h.slice_ptr, ctx->stream));
    HHP_TRY(upload(&p.pos_row, h.pos_row, ctx->stream, 4));
    HHP_TRY(upload(&p.pos_len, h.pos_len, ctx->stream, 4));
    HHP_TRY(upload(&p.chunks, h.chunks, ctx->stream));
    HHP_TRY(upload(&p.long_first, h.long_first, ctx->stream));
    HHP_TRY(upload(&p.chunk_long, h.chunk_long, ctx->stream));
    const size_t tot = static_cast<size_t>(std::max<long long>(h.total, 1));
    HHP_CUDA(cudaMalloc(&p.sval, tot * sizeof(VT)));
    HHP_CUDA(cudaMemsetAsync(p.sval, 0, tot * sizeof(VT), ctx->stream));
    // Index words: 16-bit offsets col - row when every slice row's entries lie within 2^15 of
    // the diagonal (stencils: 2 bytes per nonzero instead of 4), else int32 columns.
    p.d16 = false;
    if (t.d16 && !p.uni && A->m > 0 && A->nnz > 0) {
        int *bad = nullptr, hbad = 0;
        HHP_CUDA(cudaMalloc(&bad, sizeof(int)));
        cudaMemsetAsync(bad, 0, sizeof(int), ctx->stream);
        const int g = static_cast<int>(std::min<long long>((A->m + 255) / 256, 8LL * ctx->num_sms));
        k_offsets_fit<<<g, 256, 0, ctx->stream>>>(A->rowptr, A->col, A->m, std::max(t.long_thr, 1), bad);
        const cudaError_t e1 = cudaMemcpyAsync(&hbad, bad, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream);
        const cudaError_t e2 = cudaStreamSynchronize(ctx->stream);
        cudaFree(bad);
        HHP_CUDA(e1);
        HHP_CUDA(e2);
        p.d16 = hbad == 0;
    }
    if (p.uni) {
        // no index stream
    } else if (p.d16) {
        HHP_CUDA(cudaMalloc(&p.scol16, tot * sizeof(short)));
        HHP_CUDA(cudaMemsetAsync(p.scol16, 0, tot * sizeof(short), ctx->stream));
    } else {
        HHP_CUDA(cudaMalloc(&p.scol, tot * sizeof(int)));
        HHP_CUDA(cudaMemsetAsync(p.scol, 0, tot * sizeof(int), ctx->stream));
    }
    HHP_CUDA(cudaMalloc(&p.chunk_part, sizeof(double) * std::max(1, p.n_chunks)));
    HHP_CUDA(cudaMalloc(&p.long_cnt, sizeof(unsigned) * std::max(1, p.n_long)));
    HHP_CUDA(cudaMemsetAsync(p.long_cnt, 0, sizeof(unsigned) * std::max(1, p.n_long), ctx->stream));
    HHP_CUDA(cudaMalloc(&p.long_dot, sizeof(double) * 4 * std::max(1, p.n_long)));
    HHP_CUDA(cudaMemsetAsync(p.long_dot, 0, sizeof(double) * 4 * std::max(1, p.n_long), ctx->stream));
    p.n_groups = (p.n_long + kLongGroup - 1) / kLongGroup;
    HHP_CUDA(cudaMalloc(&p.group_cnt, sizeof(unsigned) * std::max(1, p.n_groups)));
    HHP_CUDA(cudaMemsetAsync(p.group_cnt, 0, sizeof(unsigned) * std::max(1, p.n_groups), ctx->stream));
    HHP_CUDA(cudaMalloc(&p.group_dot, sizeof(double) * 4 * std::max(1, p.n_groups)));
    HHP_CUDA(cudaMemsetAsync(p.group_dot, 0, sizeof(double) * 4 * std::max(1, p.n_groups), ctx->stream));
    HHP_CUDA(cudaMalloc(&p.cta_part, sizeof(double) * 4 * p.ctas));
    HHP_CUDA(cudaMemsetAsync(p.cta_part, 0, sizeof(double) * 4 * p.ctas, ctx->stream));
    HHP_TRY(fill_values<VT>(A, p, true));
    HHP_CUDA(cudaStreamSynchronize(ctx->stream));
    return HHP_OK;
}

template <typename VT>
SellArgs<VT> make_args(hhp_mat *A, const PlanDev &p, const VT *csr_val, const VT *x, VT *y, const VT *w1,
                       double alpha, double beta) {
    SellArgs<VT> a;
    a.slice_ptr = p.slice_ptr;
    a.pos_row = p.pos_row;
    a.pos_len = p.pos_len;
    a.warp_ptr = p.warp_ptr;
    a.warp_units = p.warp_units;
    a.unit_rec = p.unit_rec;
    a.sval = static_cast<const VT *>(p.sval);
    a.scol = p.scol;
    a.scol16 = p.scol16;
    a.csr_val = csr_val;
    a.csr_col = A->col;
    a.chunks = p.chunks;
    a.long_first = p.long_first;
    a.chunk_long = p.chunk_long;
    a.chunk_part = p.chunk_part;
    a.long_cnt = p.long_cnt;
    a.long_dot = p.long_dot;
    a.group_cnt = p.group_cnt;
    a.group_dot = p.group_dot;
    a.cta_part = p.cta_part;
    a.x = x;
    a.y = y;
    a.w1 = w1;
    a.w2 = nullptr;
    a.alpha = alpha;
    a.beta = beta;
    a.scale = alpha != 1.0 ? 1 : 0;
    a.accum = beta != 0.0 ? 1 : 0;
    a.gate = nullptr;
    a.stop = nullptr;
    a.err = A->ctx->dev_err;
    a.m = A->m;
    a.n_slices = p.n_slices;
    a.n_chunks = p.n_chunks;
    a.n_long = p.n_long;
    a.has_perm = p.has_perm;
    for (int k = 0; k < kMaxDiag; ++k) a.doff[k] = p.doff[k];
    return a;
}

}  // namespace

void PlanDev::release() {
    cudaFree(slice_ptr);
    cudaFree(pos_row);
    cudaFree(pos_len);
    cudaFree(warp_ptr);
    cudaFree(warp_units);
    cudaFree(unit_rec);
    cudaFree(sval);
    cudaFree(scol);
    cudaFree(scol16);
    cudaFree(chunks);
    cudaFree(long_first);
    cudaFree(chunk_long);
    cudaFree(chunk_part);
    cudaFree(long_cnt);
    cudaFree(long_dot);
    cudaFree(group_cnt);
    cudaFree(group_dot);
    cudaFree(cta_part);
    *this = PlanDev();
}

hhp_status ensure_plan(hhp_mat *A, bool fp32) {
    PlanDev &p = fp32 ? A->plan32 : A->plan64;
    if (p.built()) return HHP_OK;
    HHP_TRY(csr_needed(A, fp32 ? "an FP32 SpMV layout" : "an FP64 SpMV layout"));
    if (fp32) return build_plan_dev<float>(A, p);
    return build_plan_dev<double>(A, p);
}

hhp_status refresh_plan_values(hhp_mat *A) {
    if (A->plan64.built()) HHP_TRY(fill_values<double>(A, A->plan64, false));
    if (A->plan32.built()) HHP_TRY(fill_values<float>(A, A->plan32, false));
    return HHP_OK;
}

hhp_status launch_spmv64(hhp_mat *A, cudaStream_t stream, EpKind ep, const double *x, double *y, const double *w1,
                         double alpha, double beta, const int *gate, const double *w2, const int *stop) {
    HHP_TRY(ensure_plan(A, false));
    const PlanDev &p = A->plan64;
    SellArgs<double> a = make_args<double>(A, p, A->val, x, y, w1, alpha, beta);
    a.gate = gate;
    a.w2 = w2;
    a.stop = stop;
    HHP_CUDA(launch_ep<double>(ep, p, a, stream));
    A->ctx->kernel_launches += 1;
    return HHP_OK;
}

hhp_status launch_spmv32(hhp_mat *A, cudaStream_t stream, EpKind ep, const float *x, float *y, const float *w1,
                         const int *stop, const float *w2) {
    if (!A->val32) {
        set_error("FP32 SpMV requested before the FP32 copy of the values was built");
        return HHP_ERR_STATE;
    }
    HHP_TRY(ensure_plan(A, true));
    const PlanDev &p = A->plan32;
    SellArgs<float> a = make_args<float>(A, p, A->val32, x, y, w1, 1.0, 0.0);
    a.stop = stop;
    a.w2 = w2;
    HHP_CUDA(launch_ep<float>(ep, p, a, stream));
    A->ctx->kernel_launches += 1;
    return HHP_OK;
}

}  // namespace hhp
