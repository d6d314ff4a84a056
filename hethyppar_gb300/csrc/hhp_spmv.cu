// hhp_spmv.cu -- CSR SpMV for sm_103a with fused epilogues (FP64 and FP32 values).
//
// Replaces the reference's cuSPARSE call device_csr_spmv (src/util/hhp_cuda.c:226-236) and
// computes what CSR_spmxv_seq computes (src/util/hhp_cpu.c:445-455).
//
// Design (GB300):
//  * Persistent grid: one CTA per SM, `wpc` warps per CTA. Each warp owns a contiguous range of
//    work items (see hhp_plan.cpp) and streams them through its own NS-stage shared-memory ring.
//  * Loads: the warp's lane 0 issues 1-D TMA bulk copies (cp.async.bulk) of the item's values,
//    column indices and row pointers into the next free stage, completing on that stage's
//    mbarrier. Each copy is rounded outwards to 16-byte boundaries (the arrays carry zeroed
//    padding). With NS stages the warp keeps NS-1 items in flight while it computes one: the
//    bytes in flight per SM no longer depend on registers or occupancy.
//  * Compute: ROWS items (up to 32 short rows) give one row to each lane; the lane sums its row in
//    CSR order with fused multiply-adds, reading values/indices from shared memory and gathering x
//    through the read-only L1/L2 path. This is one FP64 FMA per nonzero, the minimum on GB300
//    whose FP64 rate (~2 FMA/clk/SM) is as much a limit as HBM for this kernel. VEC items (one
//    medium row) and CHUNK items (slices of a long row) are summed by the whole warp; slices are
//    combined in slice order by whichever warp finishes a row's last slice.
//  * Epilogues fuse the BiCGStab dot products (r0.v, t.s, t.t) and the residual r = b - A x into
//    the store of y. Per-CTA partials are summed in a fixed order, so results are reproducible.
#include <algorithm>
#include <mutex>

#include "hhp_device.cuh"
#include "hhp_internal.h"

namespace hhp {

namespace {

constexpr uint64_t kWaitLimitNs = 500000000ull;  // 0.5 s per mbarrier wait (a normal wait is microseconds)
constexpr int kBarBytes = 64;                     // room for up to 8 stage mbarriers per warp
constexpr int kRowPtrElems = 40;                  // 32 rows + 1, rounded out to 16 bytes

__host__ __device__ constexpr int align16(int b) { return (b + 15) & ~15; }

template <typename VT>
struct Geom {
    static constexpr int VPA = 16 / static_cast<int>(sizeof(VT));  // values per 16 bytes
    int cap;
    __host__ __device__ int val_bytes() const { return align16((cap + 2 * VPA) * static_cast<int>(sizeof(VT))); }
    __host__ __device__ int col_bytes() const { return align16((cap + 8) * 4); }
    __host__ __device__ int rp_bytes() const { return align16(kRowPtrElems * 4); }
    __host__ __device__ int stage_bytes() const { return val_bytes() + col_bytes() + rp_bytes(); }
    // gathered x values of the item being computed (one buffer per warp)
    __host__ __device__ int xs_bytes() const { return align16(cap * static_cast<int>(sizeof(VT))); }
    __host__ __device__ int warp_bytes(int ns, bool gather) const {
        return kBarBytes + ns * stage_bytes() + (gather ? xs_bytes() : 0);
    }
};

template <typename VT>
struct SpmvArgs {
    const int4 *items;
    const int *warp_begin;
    const int *rowptr;
    const int *col;
    const VT *val;
    const VT *x;
    VT *y;
    const VT *w1;
    double alpha, beta;
    const int *long_rows;
    const int *long_first;
    const int *chunk_long;
    double *chunk_part;
    unsigned *long_cnt;
    double *long_dot;
    double *cta_part;
    int *err;
    int cap;
    int warp_smem;
};

__device__ __forceinline__ double vfma(double a, double b, double c) { return fma(a, b, c); }
__device__ __forceinline__ float vfma(float a, float b, float c) { return fmaf(a, b, c); }

// Row epilogue. Returns the value stored in y[r]; accumulates dot partials into (d0, d1).
template <typename VT, int EP>
__device__ __forceinline__ void row_epilogue(const SpmvArgs<VT> &a, int r, VT acc, double &d0, double &d1) {
    if (EP == EP_AXPBY) {
        VT out = acc;
        if (a.alpha != 1.0) out = static_cast<VT>(a.alpha) * out;
        if (a.beta != 0.0) out = vfma(static_cast<VT>(a.beta), a.y[r], out);
        a.y[r] = out;
    } else if (EP == EP_DOT1) {
        a.y[r] = acc;
        d0 += static_cast<double>(acc * __ldg(a.w1 + r));
    } else if (EP == EP_DOT2) {
        a.y[r] = acc;
        d0 += static_cast<double>(acc * __ldg(a.w1 + r));
        d1 += static_cast<double>(acc * acc);
    } else {  // EP_RESID
        const VT b = __ldg(a.w1 + r);
        const VT res = b - acc;
        a.y[r] = res;
        d0 += static_cast<double>(res * res);
        d1 += static_cast<double>(b * b);
    }
}

template <typename VT>
__device__ __forceinline__ VT warp_sum_t(VT v) {
    return warp_sum(v);
}

template <typename VT, int NS, int EP, bool GATHER>
__global__ void __launch_bounds__(512) k_spmv(const SpmvArgs<VT> a) {
    extern __shared__ __align__(128) unsigned char smem[];
    // After a recorded device error every later launch returns at once (uniform across the CTA).
    if (*reinterpret_cast<volatile const int *>(a.err) != DEV_OK) return;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
    const int gw = blockIdx.x * nw + warp;
    const Geom<VT> geo{a.cap};
    constexpr int VPA = Geom<VT>::VPA;
    unsigned char *wb = smem + static_cast<size_t>(warp) * a.warp_smem;
    uint64_t *bar = reinterpret_cast<uint64_t *>(wb);
    unsigned char *stage_base = wb + kBarBytes;
    const int sbytes = geo.stage_bytes();
    VT *xs = GATHER ? reinterpret_cast<VT *>(stage_base + NS * sbytes) : nullptr;
    double *red = reinterpret_cast<double *>(smem + static_cast<size_t>(nw) * a.warp_smem);

    if (lane == 0) {
        for (int s = 0; s < NS; ++s) mbar_init(&bar[s], 1);
        fence_mbar_init();
    }
    __syncwarp();

    const int ib = a.warp_begin[gw], ie = a.warp_begin[gw + 1];

    // Lane 0: stage the item's arrays. Sizes are rounded out to 16-byte boundaries.
    auto issue = [&](int item, int s) {
        const int4 d = __ldg(&a.items[item]);
        const int kind = static_cast<unsigned>(d.y) >> KIND_SHIFT;
        unsigned char *st = stage_base + s * sbytes;
        const int k0a = d.z & ~(VPA - 1), k1a = (d.w + VPA - 1) & ~(VPA - 1);
        const int k0c = d.z & ~3, k1c = (d.w + 3) & ~3;
        const uint32_t vb = static_cast<uint32_t>(k1a - k0a) * sizeof(VT);
        const uint32_t cb = static_cast<uint32_t>(k1c - k0c) * 4u;
        uint32_t rb = 0;
        int r0a = 0;
        if (kind == KIND_ROWS) {
            const int nrows = d.y & PAYLOAD_MASK;
            r0a = d.x & ~3;
            const int r1a = (d.x + nrows + 1 + 3) & ~3;
            rb = static_cast<uint32_t>(r1a - r0a) * 4u;
        }
        mbar_arrive_expect_tx(&bar[s], vb + cb + rb);
        if (vb) bulk_g2s(st, a.val + k0a, vb, &bar[s]);
        if (cb) bulk_g2s(st + geo.val_bytes(), a.col + k0c, cb, &bar[s]);
        if (rb) bulk_g2s(st + geo.val_bytes() + geo.col_bytes(), a.rowptr + r0a, rb, &bar[s]);
    };

    if (lane == 0) {
        for (int s = 0; s < NS && ib + s < ie; ++s) issue(ib + s, s);
    }

    double d0 = 0.0, d1 = 0.0;
    uint32_t phase = 0;
    int issued_until = min(ib + NS, ie);  // items [ib, issued_until) have been issued
    int i = ib;
    bool ok = true;
    for (; i < ie; ++i) {
        const int s = (i - ib) % NS;
        const bool got = mbar_wait_bounded(&bar[s], (phase >> s) & 1u, kWaitLimitNs);
        if (!__all_sync(0xffffffffu, got)) {
            ok = false;
            break;
        }
        phase ^= (1u << s);
        const int4 d = __ldg(&a.items[i]);
        const int kind = static_cast<unsigned>(d.y) >> KIND_SHIFT;
        const unsigned char *st = stage_base + s * sbytes;
        const int k0a = d.z & ~(VPA - 1), k0c = d.z & ~3;
        const VT *sv = reinterpret_cast<const VT *>(st);
        const int *sc = reinterpret_cast<const int *>(st + geo.val_bytes());
        // Gather pass: the whole warp fetches x for every nonzero of the item, lane-strided and
        // in batches of 8 independent loads per lane, so one item costs about one L2 round trip
        // instead of one per nonzero of the longest row. Values land in xs (item-relative).
        if (GATHER) {
            const int nk = d.w - d.z;
            for (int base = 0; base < nk; base += 32 * 8) {
                VT v[8];
#pragma unroll
                for (int j = 0; j < 8; ++j) {
                    const int kk = base + lane + 32 * j;
                    v[j] = kk < nk ? __ldg(a.x + sc[d.z + kk - k0c]) : VT(0);
                }
#pragma unroll
                for (int j = 0; j < 8; ++j) {
                    const int kk = base + lane + 32 * j;
                    if (kk < nk) xs[kk] = v[j];
                }
            }
            __syncwarp();
        }
        if (kind == KIND_ROWS) {
            const int nrows = d.y & PAYLOAD_MASK;
            const int r0a = d.x & ~3;
            const int *sr = reinterpret_cast<const int *>(st + geo.val_bytes() + geo.col_bytes());
            if (lane < nrows) {
                const int r = d.x + lane;
                const int kb = sr[r - r0a], ke = sr[r + 1 - r0a];
                VT acc = VT(0);
                if (GATHER) {
                    for (int k = kb; k < ke; ++k) acc = vfma(sv[k - k0a], xs[k - d.z], acc);
                } else {
                    // gathers issued 8 at a time ahead of their multiply-adds
                    int k = kb;
                    for (; k + 8 <= ke; k += 8) {
                        VT xv[8];
#pragma unroll
                        for (int j = 0; j < 8; ++j) xv[j] = __ldg(a.x + sc[k + j - k0c]);
#pragma unroll
                        for (int j = 0; j < 8; ++j) acc = vfma(sv[k + j - k0a], xv[j], acc);
                    }
                    for (; k < ke; ++k) acc = vfma(sv[k - k0a], __ldg(a.x + sc[k - k0c]), acc);
                }
                row_epilogue<VT, EP>(a, r, acc, d0, d1);
            }
        } else {
            // One row (VEC) or one slice of a long row (CHUNK), summed by the warp: lane l takes
            // entries l, l+32, ... in order; the 32 lane sums meet in a fixed butterfly.
            VT acc = VT(0);
            for (int k = d.z + lane; k < d.w; k += 32)
                acc = vfma(sv[k - k0a], GATHER ? xs[k - d.z] : __ldg(a.x + sc[k - k0c]), acc);
            acc = warp_sum_t<VT>(acc);
            if (kind == KIND_VEC) {
                if (lane == 0) row_epilogue<VT, EP>(a, d.x, acc, d0, d1);
            } else if (lane == 0) {
                const int cid = d.y & PAYLOAD_MASK;
                a.chunk_part[cid] = static_cast<double>(acc);
                __threadfence();
                const int l = a.chunk_long[cid];
                const int c_first = a.long_first[l], nch = a.long_first[l + 1] - c_first;
                const unsigned prev = atomicAdd(&a.long_cnt[l], 1u);
                if (prev == static_cast<unsigned>(nch - 1)) {
                    __threadfence();
                    double tot = 0.0;
                    for (int c = 0; c < nch; ++c) tot += __ldcg(a.chunk_part + c_first + c);
                    a.long_cnt[l] = 0u;  // ready for the next launch
                    double e0 = 0.0, e1 = 0.0;
                    row_epilogue<VT, EP>(a, d.x, static_cast<VT>(tot), e0, e1);
                    if (EP != EP_AXPBY) {
                        a.long_dot[2 * l] = e0;
                        a.long_dot[2 * l + 1] = e1;
                    }
                }
            }
        }
        // The stage is free: order this warp's shared-memory reads before the next TMA write.
        fence_proxy_async_smem();
        __syncwarp();
        if (lane == 0 && issued_until < ie) {
            issue(issued_until, (issued_until - ib) % NS);
            ++issued_until;
        }
    }
    if (!ok) {
        if (lane == 0) atomicCAS(a.err, DEV_OK, DEV_ERR_TIMEOUT);
        // Let every copy still in flight land before the CTA's shared memory is released.
        for (int j = i; j < issued_until; ++j) {
            const int s = (j - ib) % NS;
            mbar_wait_bounded(&bar[s], (phase >> s) & 1u, kWaitLimitNs);
            phase ^= (1u << s);
        }
    }
    if (EP != EP_AXPBY) {
        d0 = warp_sum(d0);
        d1 = warp_sum(d1);
        if (lane == 0) {
            red[2 * warp] = d0;
            red[2 * warp + 1] = d1;
        }
        __syncthreads();
        if (threadIdx.x == 0) {
            double s0 = 0.0, s1 = 0.0;
            for (int w = 0; w < nw; ++w) {
                s0 += red[2 * w];
                s1 += red[2 * w + 1];
            }
            a.cta_part[2 * blockIdx.x] = s0;
            a.cta_part[2 * blockIdx.x + 1] = s1;
        }
    }
}

template <typename VT, int NS, int EP, bool G>
cudaError_t launch_one(const PlanDev &p, const SpmvArgs<VT> &a, cudaStream_t s) {
    auto fn = k_spmv<VT, NS, EP, G>;
    static std::once_flag once;
    static cudaError_t attr_err = cudaSuccess;
    std::call_once(once, [&] {
        attr_err = cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, 227 * 1024);
    });
    if (attr_err != cudaSuccess) return attr_err;
    fn<<<p.ctas, p.warps_per_cta * 32, p.smem_bytes, s>>>(a);
    return cudaGetLastError();
}

template <typename VT, int EP, bool G>
cudaError_t launch_ns(const PlanDev &p, const SpmvArgs<VT> &a, cudaStream_t s) {
    switch (p.ns) {
        case 1: return launch_one<VT, 1, EP, G>(p, a, s);
        case 3: return launch_one<VT, 3, EP, G>(p, a, s);
        default: return launch_one<VT, 2, EP, G>(p, a, s);
    }
}

template <typename VT, int EP>
cudaError_t launch_g(const PlanDev &p, const SpmvArgs<VT> &a, cudaStream_t s) {
    return p.gather ? launch_ns<VT, EP, true>(p, a, s) : launch_ns<VT, EP, false>(p, a, s);
}

template <typename VT>
cudaError_t launch_ep(EpKind ep, const PlanDev &p, const SpmvArgs<VT> &a, cudaStream_t s) {
    switch (ep) {
        case EP_DOT1: return launch_g<VT, EP_DOT1>(p, a, s);
        case EP_DOT2: return launch_g<VT, EP_DOT2>(p, a, s);
        case EP_RESID: return launch_g<VT, EP_RESID>(p, a, s);
        default: return launch_g<VT, EP_AXPBY>(p, a, s);
    }
}

template <typename VT>
SpmvArgs<VT> make_args(hhp_mat *A, const PlanDev &p, const VT *val, const VT *x, VT *y, const VT *w1, double alpha,
                       double beta) {
    SpmvArgs<VT> a;
    a.items = p.items;
    a.warp_begin = p.warp_begin;
    a.rowptr = A->rowptr;
    a.col = A->col;
    a.val = val;
    a.x = x;
    a.y = y;
    a.w1 = w1;
    a.alpha = alpha;
    a.beta = beta;
    a.long_rows = p.long_rows;
    a.long_first = p.long_first;
    a.chunk_long = p.chunk_long;
    a.chunk_part = p.chunk_part;
    a.long_cnt = p.long_cnt;
    a.long_dot = p.long_dot;
    a.cta_part = p.cta_part;
    a.err = A->ctx->dev_err;
    a.cap = p.cap;
    a.warp_smem = Geom<VT>{p.cap}.warp_bytes(p.ns, p.gather);
    return a;
}

template <typename T>
hhp_status upload(T **dst, const std::vector<T> &src, size_t min_elems = 1) {
    const size_t n = std::max(src.size(), min_elems);
    HHP_CUDA(cudaMalloc(reinterpret_cast<void **>(dst), n * sizeof(T)));
    if (!src.empty()) HHP_CUDA(cudaMemcpy(*dst, src.data(), src.size() * sizeof(T), cudaMemcpyHostToDevice));
    return HHP_OK;
}

template <typename VT>
hhp_status build_plan_dev(hhp_mat *A, PlanDev &p, int cap_req) {
    const Tuning &t = tuning();
    hhp_ctx *ctx = A->ctx;
    const int ns = std::min(std::max(t.ns, 1), 3);
    const bool gather = t.gather != 0;
    const int cap = std::max(64, std::min(cap_req, 4096)) & ~31;
    const int cps = std::min(std::max(t.ctas_per_sm, 1), 8);
    int wpc = std::min(std::max(t.wpc, 1), 16);
    const Geom<VT> geo{cap};
    // shared memory of one SM is split between its CTAs
    const size_t sm_budget = 228 * 1024 - 1024 * static_cast<size_t>(cps);
    const size_t cta_budget = std::min<size_t>(std::min<size_t>(ctx->smem_optin, 227 * 1024), sm_budget / cps);
    auto need = [&](int w) { return static_cast<size_t>(w) * geo.warp_bytes(ns, gather) + 64 * 8; };
    while (wpc > 1 && need(wpc) > cta_budget) --wpc;
    if (need(wpc) > cta_budget) {
        set_error("SpMV plan: stage buffers of cap=%d do not fit in shared memory", cap);
        return HHP_ERR_ARG;
    }
    PlanHost h;
    const int ctas = ctx->num_sms * cps;
    build_plan(A->m, A->rowptr_host.data(), ctas * wpc, cap, std::min(t.med, cap), h);
    p.release();
    p.n_warps = ctas * wpc;
    p.cap = cap;
    p.ns = ns;
    p.gather = gather;
    p.ctas = ctas;
    p.warps_per_cta = wpc;
    p.smem_bytes = need(wpc);
    p.n_items = static_cast<int>(h.items.size());
    p.n_long = static_cast<int>(h.long_rows.size());
    p.n_chunks = static_cast<int>(h.chunk_long.size());
    HHP_TRY(upload(&p.items, h.items));
    HHP_TRY(upload(&p.warp_begin, h.warp_begin));
    HHP_TRY(upload(&p.long_rows, h.long_rows));
    HHP_TRY(upload(&p.long_first, h.long_first));
    HHP_TRY(upload(&p.chunk_long, h.chunk_long));
    HHP_CUDA(cudaMalloc(&p.chunk_part, sizeof(double) * std::max(1, p.n_chunks)));
    HHP_CUDA(cudaMalloc(&p.long_cnt, sizeof(unsigned) * std::max(1, p.n_long)));
    HHP_CUDA(cudaMemset(p.long_cnt, 0, sizeof(unsigned) * std::max(1, p.n_long)));
    HHP_CUDA(cudaMalloc(&p.long_dot, sizeof(double) * 2 * std::max(1, p.n_long)));
    HHP_CUDA(cudaMemset(p.long_dot, 0, sizeof(double) * 2 * std::max(1, p.n_long)));
    HHP_CUDA(cudaMalloc(&p.cta_part, sizeof(double) * 2 * ctas));
    HHP_CUDA(cudaMemset(p.cta_part, 0, sizeof(double) * 2 * ctas));
    return HHP_OK;
}

}  // namespace

void PlanDev::release() {
    cudaFree(items);
    cudaFree(warp_begin);
    cudaFree(long_rows);
    cudaFree(long_first);
    cudaFree(chunk_long);
    cudaFree(chunk_part);
    cudaFree(long_cnt);
    cudaFree(long_dot);
    cudaFree(cta_part);
    *this = PlanDev();
}

hhp_status ensure_plan(hhp_mat *A, bool fp32) {
    PlanDev &p = fp32 ? A->plan32 : A->plan64;
    if (p.items != nullptr || (p.n_warps > 0)) return HHP_OK;
    const Tuning &t = tuning();
    if (fp32) return build_plan_dev<float>(A, p, t.cap32);
    return build_plan_dev<double>(A, p, t.cap64);
}

hhp_status launch_spmv64(hhp_mat *A, cudaStream_t stream, EpKind ep, const double *x, double *y, const double *w1,
                         double alpha, double beta) {
    HHP_TRY(ensure_plan(A, false));
    const PlanDev &p = A->plan64;
    SpmvArgs<double> a = make_args<double>(A, p, A->val, x, y, w1, alpha, beta);
    HHP_CUDA(launch_ep<double>(ep, p, a, stream));
    A->ctx->kernel_launches += 1;
    return HHP_OK;
}

hhp_status launch_spmv32(hhp_mat *A, cudaStream_t stream, EpKind ep, const float *x, float *y, const float *w1) {
    if (!A->val32) {
        set_error("FP32 SpMV requested before the FP32 copy of the values was built");
        return HHP_ERR_STATE;
    }
    HHP_TRY(ensure_plan(A, true));
    const PlanDev &p = A->plan32;
    SpmvArgs<float> a = make_args<float>(A, p, A->val32, x, y, w1, 1.0, 0.0);
    HHP_CUDA(launch_ep<float>(ep, p, a, stream));
    A->ctx->kernel_launches += 1;
    return HHP_OK;
}

}  // namespace hhp
