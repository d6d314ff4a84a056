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
// m + nnz items; CTA c takes items [c*D, (c+1)*D). Rows that end inside a CTA's range are summed
// by its warps (lane-strided, then a butterfly) and written as alpha*sum + beta*y; the part of
// the row still open at the end of the range goes to the CTA's carry slot. A second kernel adds
// the carries of each row, in CTA order, to the row's y. The same per-row arithmetic as
// hhp_spmv_dev's warp-summed rows; rows split between CTAs differ from it only in rounding.
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

__device__ __forceinline__ double warp_range_sum(const int *__restrict__ col, const double *__restrict__ val,
                                                 const double *__restrict__ x, long long a, long long b, int lane) {
    double s = 0.0;
    for (long long k = a + lane; k < b; k += 32) s = fma(__ldg(val + k), __ldg(x + __ldg(col + k)), s);
    return hhp::warp_sum(s);
}

__global__ void __launch_bounds__(kThreads) k_mp_spmv(int m, long long nnz, const int *__restrict__ rowptr,
                                                      const int *__restrict__ col, const double *__restrict__ val,
                                                      double alpha, const double *__restrict__ x, double beta,
                                                      double *y, long long D, double *carry_val, int *carry_row) {
    const int c = blockIdx.x;
    const long long total = static_cast<long long>(m) + nnz;
    // the last CTAs can start past the end when the split is rounded up: they get an empty range
    const long long d0 = static_cast<long long>(c) * D < total ? static_cast<long long>(c) * D : total;
    const long long d1 = d0 + D < total ? d0 + D : total;
    int r0, r1;
    long long k0, k1;
    merge_path(rowptr, m, nnz, d0, r0, k0);
    merge_path(rowptr, m, nnz, d1, r1, k1);
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
    // rows ending inside this CTA's range
    for (int r = r0 + warp; r < r1; r += nw) {
        const long long a = rowptr[r] > k0 ? rowptr[r] : k0;
        const double s = warp_range_sum(col, val, x, a, rowptr[r + 1], lane);
        if (lane == 0) y[r] = beta != 0.0 ? fma(beta, y[r], alpha * s) : alpha * s;
    }
    // the row left open at the end of the range
    if (warp == 0) {
        double s = 0.0;
        int cr = -1;
        if (r1 < m) {
            const long long a = rowptr[r1] > k0 ? rowptr[r1] : k0;
            if (k1 > a) {
                s = warp_range_sum(col, val, x, a, k1, lane);
                cr = r1;
            }
        }
        if (lane == 0) {
            carry_val[c] = s;
            carry_row[c] = cr;
        }
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
