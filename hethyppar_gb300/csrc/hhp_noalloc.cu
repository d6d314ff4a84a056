// hhp_noalloc.cu -- y = alpha*A*x + beta*y on caller-owned device CSR arrays, without allocating.
//
// For callers that cannot call cudaMalloc: code that must not trigger the implicit device-wide
// synchronisation of cudaMalloc/cudaFree in the middle of its stream work, or that runs under a
// memory budget owned by someone else (a host application or framework that pre-sizes and owns
// all device memory). The caller passes every input and output; the only scratch this path
// needs -- one carry (row, partial sum) per CTA for rows split between CTAs -- lives in a
// file-scope __device__ array of kMaxCarry entries that every GPU loading the library holds
// until the process exits.
//
// Work split (merge path): the rows' end offsets and the nonzeros form one merged list of
// m + nnz items; CTA c takes items [c*D, (c+1)*D), in tiles of 2048 items. Per tile the CTA stages
// the row ends, the values and the gathered x of its nonzeros in shared memory (coalesced loads);
// each thread walks 8 items, summing in CSR order with one FMA per nonzero, and writes the rows
// that start and end inside its walk as alpha*sum + beta*y; rows that cross threads are combined
// by a fixed-order segmented scan, and a row still open at the end of a tile carries into the
// next. The row open at the end of the CTA's range goes to the CTA's carry slot, and a second
// kernel adds the carries of each row, in CTA order, to the row's y. Rows inside one thread's
// walk are summed exactly as hhp_spmv_dev sums them; rows split between threads or CTAs differ
// from it only in rounding. (Measured against the library's sliced plan on GB300, L2 flushed:
// 3.5M-row power law 420 vs 109 us, banded 450k 118 vs 32 us: the per-tile barriers and the
// 8-item dependent walks cost more than the plan's balanced slices.)
//
// Set-up: the first call on a device resolves the array's device address with
// cudaGetSymbolAddress, with that device current, and remembers it; make that first call before
// any stream capture. All calls share the one array and it keeps the last call's contents. Nothing
// in it needs to start at zero: a call writes every slot of its CTAs (an unused slot is marked
// row -1) before its second kernel reads any. Calls that overlap on the GPU (on different streams,
// or from different host threads on one device) race on the array and give wrong results.
#include <cuda_runtime.h>

#include <mutex>

#include "hhp_device.cuh"
#include "hhp_internal.h"

namespace {

constexpr int kMaxCarry = 4096;                          // CTAs of one call (= carry slots)
constexpr long long kItemsPerCtaMin = 2048;              // merge items a CTA takes at least
constexpr long long kItemsPerCtaMax = 1LL << 16;         // ... and at most
constexpr long long kMaxItems = kMaxCarry * kItemsPerCtaMax;  // largest m + nnz accepted (2^28)
constexpr int kThreads = 256;
constexpr int kMaxDevices = 64;

static __device__ __align__(256) double g_carry_val[kMaxCarry];
static __device__ __align__(256) int g_carry_row[kMaxCarry];

struct Scratch {
    double *val = nullptr;
    int *row = nullptr;
};
std::mutex g_mu;
Scratch g_scratch[kMaxDevices];
bool g_ready[kMaxDevices] = {};

// Merge-path coordinate on diagonal d of (row end offsets rowptr[1..m]) x (nonzeros 0..nnz-1):
// x rows completed, d - x nonzeros consumed.
__device__ __forceinline__ void merge_path(const int *__restrict__ rowptr, int m, long long nnz, long long d, int &row,
                                           long long &k) {
    long long lo = d - nnz > 0 ? d - nnz : 0, hi = d < m ? d : m;
    while (lo < hi) {
        const long long mid = (lo + hi) >> 1;
        if (rowptr[mid + 1] <= d - mid - 1) lo = mid + 1;
        else hi = mid;
    }
    row = static_cast<int>(lo);
    k = d - lo;
}

constexpr int kIpt = 8;                   // merge items per thread per tile
constexpr int kTile = kThreads * kIpt;    // merge items per tile (2048)
constexpr int kMaxTiles = static_cast<int>(kItemsPerCtaMax / kTile);

// Inclusive segmented scan over the block, in thread order, of (row, v) pairs whose rows do not
// decrease with the thread index: the sum of v over the run of threads up to and including this
// one that carry the same row, earlier values first. Fixed order: reproducible.
__device__ __forceinline__ double seg_scan(int row, double v, int *srow, double *sv) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const int r2 = __shfl_up_sync(0xffffffffu, row, o);
        const double v2 = __shfl_up_sync(0xffffffffu, v, o);
        if (lane >= o && r2 == row) v = v2 + v;
    }
    if (lane == 31) {
        srow[warp] = row;
        sv[warp] = v;
    }
    __syncthreads();
    if (threadIdx.x == 0) {  // the warps' totals, in order (8 of them)
        for (int w = 1; w < nw; ++w)
            if (srow[w] == srow[w - 1]) sv[w] = sv[w - 1] + sv[w];
    }
    __syncthreads();
    if (warp > 0 && srow[warp - 1] == row) v = sv[warp - 1] + v;
    return v;
}

// Merge-path SpMV, thread-sequential: CTA c takes merge items [c*D, (c+1)*D) of the list of row
// ends and nonzeros, in tiles of kTile items. Per tile the CTA stages, with coalesced loads, the
// row ends, the values and the gathered x[col] of its nonzeros in shared memory; thread t walks
// kIpt items of it, summing its rows in CSR order with one FMA per nonzero and writing every row
// that starts and ends inside its walk. The partial sums of rows that cross threads are combined
// by a segmented scan (fixed order), and a row still open at the end of a tile carries into the
// next tile; the row open at the end of the CTA's range goes to the CTA's carry slot.
__global__ void __launch_bounds__(kThreads) k_mp_spmv(int m, long long nnz, const int *__restrict__ rowptr,
                                                      const int *__restrict__ col, const double *__restrict__ val,
                                                      double alpha, const double *__restrict__ x, double beta,
                                                      double *y, long long D, double *carry_val, int *carry_row) {
    __shared__ int s_rend[kTile + 1];
    __shared__ double s_val[kTile], s_x[kTile];
    __shared__ long long s_bound_k[kMaxTiles + 1];
    __shared__ int s_bound_r[kMaxTiles + 1];
    __shared__ int s_srow[32];
    __shared__ double s_sv[32];
    const int c = blockIdx.x, t = threadIdx.x;
    const long long total = static_cast<long long>(m) + nnz;
    const long long c0 = static_cast<long long>(c) * D < total ? static_cast<long long>(c) * D : total;
    const long long c1 = c0 + D < total ? c0 + D : total;
    const int ntiles = static_cast<int>((c1 - c0 + kTile - 1) / kTile);
    // every tile boundary of the CTA's range at once (one search latency, not one per tile)
    if (t <= ntiles) {
        const long long d = c0 + static_cast<long long>(t) * kTile < c1 ? c0 + static_cast<long long>(t) * kTile : c1;
        int r;
        long long k;
        merge_path(rowptr, m, nnz, d, r, k);
        s_bound_r[t] = r;
        s_bound_k[t] = k;
    }
    __syncthreads();
    double tile_carry = 0.0;  // the open row's sum from earlier tiles of this CTA (row s_bound_r[tile])
    for (int tile = 0; tile < ntiles; ++tile) {
        const int ra = s_bound_r[tile], rb = s_bound_r[tile + 1];
        const long long ka = s_bound_k[tile], kb = s_bound_k[tile + 1];
        const int nr = rb - ra, nk = static_cast<int>(kb - ka);
        for (int i = t; i < nr; i += kThreads) s_rend[i] = rowptr[ra + i + 1];
        for (int i = t; i < nk; i += kThreads) {
            const long long k = ka + i;
            s_val[i] = __ldg(val + k);
            s_x[i] = __ldg(x + __ldg(col + k));
        }
        __syncthreads();
        // this thread's start on the tile's merge path
        const long long da = ka + ra;
        const long long dt = da + static_cast<long long>(t) * kIpt < kb + rb ? da + static_cast<long long>(t) * kIpt : kb + rb;
        const long long de = dt + kIpt < kb + rb ? dt + kIpt : kb + rb;
        long long lo = dt - kb > ra ? dt - kb : ra, hi = dt - ka < rb ? dt - ka : rb;
        while (lo < hi) {
            const long long mid = (lo + hi) >> 1;
            if (s_rend[mid - ra] <= dt - mid - 1) lo = mid + 1;
            else hi = mid;
        }
        int r = static_cast<int>(lo);
        long long k = dt - lo;
        double acc = 0.0, first_acc = 0.0;
        int first_row = -1;
        for (long long d = dt; d < de; ++d) {
            if (r < rb && s_rend[r - ra] <= k) {  // row r ends here
                if (first_row < 0) {
                    first_row = r;
                    first_acc = acc;
                } else {
                    y[r] = beta != 0.0 ? fma(beta, y[r], alpha * acc) : alpha * acc;
                }
                acc = 0.0;
                ++r;
            } else {
                acc = fma(s_val[k - ka], s_x[k - ka], acc);
                ++k;
            }
        }
        // thread 0's run continues the tile's carried row; the scan combines the runs across threads
        const double own = (t == 0 && first_row < 0) ? tile_carry + acc : acc;
        const double run = seg_scan(r, own, s_srow, s_sv);
        // thread t - 1's run and row (every lane takes part in the shuffles)
        const double prev = __shfl_up_sync(0xffffffffu, run, 1);
        const int prow = __shfl_up_sync(0xffffffffu, r, 1);
        if (first_row >= 0) {
            // the runs of the earlier threads on this row, or the tile's carry for thread 0
            double cin = t == 0 ? tile_carry : 0.0;
            if ((t & 31) != 0) {
                if (prow == first_row) cin = prev;
            } else if (t > 0 && s_srow[(t >> 5) - 1] == first_row) {
                cin = s_sv[(t >> 5) - 1];
            }
            const double tot = cin + first_acc;
            y[first_row] = beta != 0.0 ? fma(beta, y[first_row], alpha * tot) : alpha * tot;
        }
        // the row open at the tile's end carries into the next tile (the last thread's run)
        if (t == kThreads - 1) s_sv[31] = run;
        __syncthreads();
        tile_carry = s_sv[31];
        __syncthreads();
    }
    if (t == 0) {
        // the row left open at the end of the CTA's range, if this CTA consumed any of its nonzeros
        const int ro = s_bound_r[ntiles];
        const long long ko = s_bound_k[ntiles], k0 = s_bound_k[0];
        const bool open = ntiles > 0 && ro < m && ko > (rowptr[ro] > k0 ? rowptr[ro] : k0);
        carry_val[c] = open ? tile_carry : 0.0;
        carry_row[c] = open ? ro : -1;
    }
}

// Adds each row's carries, in CTA order, once: the first CTA carrying a row sums the run.
__global__ void k_mp_fixup(int n_cta, double alpha, double *y, const double *carry_val, const int *carry_row) {
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= n_cta) return;
    const int row = carry_row[c];
    if (row < 0 || (c > 0 && carry_row[c - 1] == row)) return;
    double s = 0.0;
    for (int q = c; q < n_cta && carry_row[q] == row; ++q) s += carry_val[q];
    y[row] = fma(alpha, s, y[row]);
}

hhp_status scratch_for_current_device(Scratch &out) {
    int dev = 0;
    HHP_CUDA(cudaGetDevice(&dev));
    if (dev < 0 || dev >= kMaxDevices) {
        hhp::set_error("hhp_spmv_csr_noalloc: device %d outside the supported range 0..%d", dev, kMaxDevices - 1);
        return HHP_ERR_ARG;
    }
    std::lock_guard<std::mutex> lock(g_mu);
    if (!g_ready[dev]) {
        Scratch s;
        HHP_CUDA(cudaGetSymbolAddress(reinterpret_cast<void **>(&s.val), g_carry_val));
        HHP_CUDA(cudaGetSymbolAddress(reinterpret_cast<void **>(&s.row), g_carry_row));
        g_scratch[dev] = s;
        g_ready[dev] = true;
    }
    out = g_scratch[dev];
    return HHP_OK;
}

}  // namespace

extern "C" hhp_status hhp_spmv_csr_noalloc(int m, int n, int nnz, const int *rowptr_dev, const int *col_dev,
                                           const double *val_dev, double alpha, const double *x_dev, double beta,
                                           double *y_dev, void *stream) {
    HHP_API_BEGIN
    if (m < 0 || n < 0 || nnz < 0 || !rowptr_dev || (nnz > 0 && (!col_dev || !val_dev)) || (m > 0 && !y_dev) ||
        (nnz > 0 && !x_dev)) {
        hhp::set_error("hhp_spmv_csr_noalloc: invalid sizes or null pointers");
        return HHP_ERR_ARG;
    }
    const long long total = static_cast<long long>(m) + nnz;
    if (total > kMaxItems) {
        hhp::set_error("hhp_spmv_csr_noalloc: m + nnz = %lld exceeds the maximum %lld (%d CTAs x %lld items)", total,
                       kMaxItems, kMaxCarry, kItemsPerCtaMax);
        return HHP_ERR_ARG;
    }
    if (m == 0) return HHP_OK;
    Scratch sc;
    HHP_TRY(scratch_for_current_device(sc));
    long long n_cta = (total + kItemsPerCtaMin - 1) / kItemsPerCtaMin;
    if (n_cta > kMaxCarry) n_cta = kMaxCarry;
    const long long D = (total + n_cta - 1) / n_cta;
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    k_mp_spmv<<<static_cast<int>(n_cta), kThreads, 0, st>>>(m, nnz, rowptr_dev, col_dev, val_dev, alpha, x_dev,
                                                             beta, y_dev, D, sc.val, sc.row);
    k_mp_fixup<<<static_cast<int>((n_cta + 255) / 256), 256, 0, st>>>(static_cast<int>(n_cta), alpha, y_dev, sc.val,
                                                                      sc.row);
    HHP_CUDA(cudaGetLastError());
    return HHP_OK;
    HHP_API_END
}
