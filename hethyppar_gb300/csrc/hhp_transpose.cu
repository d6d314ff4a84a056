// hhp_transpose.cu -- CSR transpose built on the device, and the fused dL/dA kernel.
//
// The reference transposes on the host by count -> prefix sum -> scatter in row order
// (CSR_to_CSC, src/util/hhp_matrix.c:1476-1535), which leaves the entries of each column in
// increasing row order. Here the same order comes from a stable LSD radix sort of the nonzero
// indices k = 0..nnz-1 keyed by column (8-bit digits): since k increases with the row, a stable
// sort by column yields exactly CSR_to_CSC's order, deterministically.
//   radix pass: per-tile digit histograms -> exclusive scan (digit-major) -> stable scatter
//   (each tile is scattered by one warp, 32 entries at a time, ranks from __match_any_sync)
// t_map[p] = k records where A^T's entry p came from, so new values of A are gathered in one pass.
#include <algorithm>
#include <vector>

#include "hhp_device.cuh"
#include "hhp_internal.h"

namespace hhp {

namespace {

constexpr int kTile = 2048;  // entries per radix tile
constexpr int kScanBlock = 1024;

__global__ void k_iota_keys(const int *__restrict__ col, int *keys, int *vals, int nnz) {
    for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < nnz; k += gridDim.x * blockDim.x) {
        keys[k] = col[k];
        vals[k] = k;
    }
}

__global__ void k_digit_hist(const int *__restrict__ keys, int nnz, int shift, int n_tiles, int *hist) {
    __shared__ int h[256];
    for (int d = threadIdx.x; d < 256; d += blockDim.x) h[d] = 0;
    __syncthreads();
    const int t = blockIdx.x;
    const int k0 = t * kTile, k1 = min(k0 + kTile, nnz);
    for (int k = k0 + threadIdx.x; k < k1; k += blockDim.x) atomicAdd(&h[(keys[k] >> shift) & 255], 1);
    __syncthreads();
    for (int d = threadIdx.x; d < 256; d += blockDim.x) hist[d * n_tiles + t] = h[d];
}

// One warp per tile: entries are placed in tile order, so the pass is stable.
__global__ void k_digit_scatter(const int *__restrict__ keys_in, const int *__restrict__ vals_in, int nnz, int shift,
                                int n_tiles, const int *__restrict__ offs, int *keys_out, int *vals_out) {
    __shared__ int base[256];
    const int t = blockIdx.x;
    const int lane = threadIdx.x;
    for (int d = lane; d < 256; d += 32) base[d] = offs[d * n_tiles + t];
    __syncwarp();
    const int k0 = t * kTile, k1 = min(k0 + kTile, nnz);
    for (int k = k0; k < k1; k += 32) {
        const int kk = k + lane;
        const bool valid = kk < k1;
        const int key = valid ? keys_in[kk] : 0;
        const int d = valid ? ((key >> shift) & 255) : 256 + lane;  // invalid lanes match nobody
        const unsigned peers = __match_any_sync(0xffffffffu, d);
        const int rank = __popc(peers & ((1u << lane) - 1u));
        int pos = 0;
        if (valid) pos = base[d] + rank;
        __syncwarp();
        if (valid && rank == __popc(peers) - 1) base[d] += __popc(peers);  // last peer bumps the base
        __syncwarp();
        if (valid) {
            keys_out[pos] = key;
            vals_out[pos] = vals_in[kk];
        }
    }
}

// Exclusive scan, phase 1: per-block scan, block totals.
__global__ void k_scan_block(const int *__restrict__ in, int *out, int n, int *block_sums) {
    __shared__ int s[kScanBlock];
    const int i = blockIdx.x * kScanBlock + threadIdx.x;
    const int v = i < n ? in[i] : 0;
    s[threadIdx.x] = v;
    __syncthreads();
    for (int o = 1; o < kScanBlock; o <<= 1) {
        const int a = threadIdx.x >= o ? s[threadIdx.x - o] : 0;
        __syncthreads();
        s[threadIdx.x] += a;
        __syncthreads();
    }
    if (i < n) out[i] = s[threadIdx.x] - v;
    if (threadIdx.x == kScanBlock - 1) block_sums[blockIdx.x] = s[threadIdx.x];
}

// Phase 2: one block scans the block totals sequentially in chunks (exclusive).
__global__ void k_scan_sums(int *block_sums, int nb) {
    __shared__ int s[kScanBlock];
    __shared__ int carry;
    if (threadIdx.x == 0) carry = 0;
    __syncthreads();
    for (int c0 = 0; c0 < nb; c0 += kScanBlock) {
        const int i = c0 + threadIdx.x;
        const int v = i < nb ? block_sums[i] : 0;
        s[threadIdx.x] = v;
        __syncthreads();
        for (int o = 1; o < kScanBlock; o <<= 1) {
            const int a = threadIdx.x >= o ? s[threadIdx.x - o] : 0;
            __syncthreads();
            s[threadIdx.x] += a;
            __syncthreads();
        }
        if (i < nb) block_sums[i] = carry + s[threadIdx.x] - v;
        __syncthreads();
        if (threadIdx.x == kScanBlock - 1) carry += s[threadIdx.x];
        __syncthreads();
    }
}

__global__ void k_scan_add(int *out, int n, const int *__restrict__ block_sums) {
    const int i = blockIdx.x * kScanBlock + threadIdx.x;
    if (i < n) out[i] += block_sums[blockIdx.x];
}

hhp_status exclusive_scan(const int *in, int *out, int n, cudaStream_t st, int **scratch, int *scratch_n) {
    if (n <= 0) return HHP_OK;
    const int nb = (n + kScanBlock - 1) / kScanBlock;
    if (*scratch_n < nb) {
        cudaFree(*scratch);
        *scratch = nullptr;
        HHP_CUDA(cudaMalloc(scratch, sizeof(int) * static_cast<size_t>(nb)));
        *scratch_n = nb;
    }
    k_scan_block<<<nb, kScanBlock, 0, st>>>(in, out, n, *scratch);
    k_scan_sums<<<1, kScanBlock, 0, st>>>(*scratch, nb);
    k_scan_add<<<nb, kScanBlock, 0, st>>>(out, n, *scratch);
    HHP_CUDA(cudaGetLastError());
    return HHP_OK;
}

__global__ void k_rowidx(const int *__restrict__ rowptr, int m, int *rowidx) {
    const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
    const int nw = (gridDim.x * blockDim.x) >> 5;
    for (int r = warp; r < m; r += nw)
        for (int k = rowptr[r] + lane; k < rowptr[r + 1]; k += 32) rowidx[k] = r;
}

__global__ void k_col_count(const int *__restrict__ col, int nnz, int *cnt) {
    for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < nnz; k += gridDim.x * blockDim.x) atomicAdd(&cnt[col[k]], 1);
}

__global__ void k_t_fill(const int *__restrict__ tmap, const int *__restrict__ rowidx, const double *__restrict__ val,
                         int nnz, int *tcol, double *tval) {
    for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < nnz; p += gridDim.x * blockDim.x) {
        const int k = tmap[p];
        tcol[p] = rowidx[k];
        tval[p] = val[k];
    }
}

__global__ void k_t_vals(const int *__restrict__ tmap, const double *__restrict__ val, int nnz, double *tval) {
    for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < nnz; p += gridDim.x * blockDim.x) tval[p] = val[tmap[p]];
}

// dL/dA_k = -lambda[row(k)] * x[col(k)] over A's stored entries (fused with nothing else to read).
__global__ void k_dlda(const int *__restrict__ rowidx, const int *__restrict__ col, const double *__restrict__ lambda,
                       const double *__restrict__ x, int nnz, double *dlda) {
    for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < nnz; k += gridDim.x * blockDim.x)
        dlda[k] = -(__ldg(lambda + rowidx[k]) * __ldg(x + col[k]));
}

int grid_for(const hhp_ctx *ctx, long long n, int threads) {
    const long long want = (n + threads - 1) / threads;
    return static_cast<int>(std::max<long long>(1, std::min<long long>(want, 8LL * ctx->num_sms)));
}

}  // namespace

hhp_status ensure_transpose(hhp_mat *A) {
    if (A->t) return HHP_OK;
    HHP_TRY(csr_needed(A, "the transpose"));
    hhp_ctx *ctx = A->ctx;
    cudaStream_t st = ctx->stream;
    const int m = A->m, n = A->n, nnz = A->nnz;
    hhp_mat *T = nullptr;
    HHP_TRY(mat_create_dev(ctx, n, m, nnz, &T));
    int *rowidx = nullptr, *k1 = nullptr, *v1 = nullptr, *k2 = nullptr, *v2 = nullptr, *hist = nullptr, *scr = nullptr;
    int scr_n = 0;
    hhp_status rc = HHP_OK;
    auto fail = [&](hhp_status s) {
        cudaFree(k1); cudaFree(v1); cudaFree(k2); cudaFree(v2); cudaFree(hist); cudaFree(scr);
        if (s != HHP_OK) { cudaFree(rowidx); hhp_mat_destroy(T); }
        return s;
    };
    const size_t nz = static_cast<size_t>(std::max(nnz, 1));
    if (cudaMalloc(&rowidx, nz * 4) || cudaMalloc(&k1, nz * 4) || cudaMalloc(&v1, nz * 4) || cudaMalloc(&k2, nz * 4) ||
        cudaMalloc(&v2, nz * 4)) {
        set_error("transpose: out of device memory");
        return fail(HHP_ERR_OOM);
    }
    const int thr = 256;
    if (m > 0) k_rowidx<<<grid_for(ctx, static_cast<long long>(m) * 32, thr), thr, 0, st>>>(A->rowptr, m, rowidx);
    // column counts -> row pointers of A^T (rowptr scratch holds counts, then the scan)
    int *cnt = nullptr;
    if (cudaMalloc(&cnt, sizeof(int) * (static_cast<size_t>(n) + 1))) return fail(HHP_ERR_OOM);
    cudaMemsetAsync(cnt, 0, sizeof(int) * (static_cast<size_t>(n) + 1), st);
    if (nnz > 0) k_col_count<<<grid_for(ctx, nnz, thr), thr, 0, st>>>(A->col, nnz, cnt);
    rc = exclusive_scan(cnt, T->rowptr, n + 1, st, &scr, &scr_n);
    cudaFree(cnt);
    if (rc != HHP_OK) return fail(rc);
    // stable radix sort of k by column
    if (nnz > 0) {
        const int n_tiles = (nnz + kTile - 1) / kTile;
        if (cudaMalloc(&hist, sizeof(int) * 256 * static_cast<size_t>(n_tiles))) return fail(HHP_ERR_OOM);
        k_iota_keys<<<grid_for(ctx, nnz, thr), thr, 0, st>>>(A->col, k1, v1, nnz);
        int bits = 0;
        while (bits < 31 && ((n - 1) >> bits) > 0) bits += 8;
        for (int shift = 0; shift < bits; shift += 8) {
            k_digit_hist<<<n_tiles, 256, 0, st>>>(k1, nnz, shift, n_tiles, hist);
            rc = exclusive_scan(hist, hist, 256 * n_tiles, st, &scr, &scr_n);
            if (rc != HHP_OK) return fail(rc);
            k_digit_scatter<<<n_tiles, 32, 0, st>>>(k1, v1, nnz, shift, n_tiles, hist, k2, v2);
            std::swap(k1, k2);
            std::swap(v1, v2);
        }
        k_t_fill<<<grid_for(ctx, nnz, thr), thr, 0, st>>>(v1, rowidx, A->val, nnz, T->col, T->val);
    }
    if (cudaGetLastError() != cudaSuccess || cudaStreamSynchronize(st) != cudaSuccess) {
        set_error("transpose kernels failed");
        return fail(HHP_ERR_CUDA);
    }
    T->rowptr_host.resize(static_cast<size_t>(n) + 1);
    if (cudaMemcpy(T->rowptr_host.data(), T->rowptr, sizeof(int) * (static_cast<size_t>(n) + 1),
                   cudaMemcpyDeviceToHost) != cudaSuccess)
        return fail(HHP_ERR_CUDA);
    // v1 holds the map; keep it, free the rest
    A->t_map = v1;
    v1 = nullptr;
    A->t = T;
    A->rowidx = rowidx;
    fail(HHP_OK);
    if (A->val32) HHP_TRY(mat_refresh_derived(T));
    return HHP_OK;
}

hhp_status refresh_transpose_values(hhp_mat *A) {
    if (!A->t) return HHP_OK;
    if (A->nnz > 0)
        k_t_vals<<<grid_for(A->ctx, A->nnz, 256), 256, 0, A->ctx->stream>>>(A->t_map, A->val, A->nnz, A->t->val);
    HHP_CUDA(cudaGetLastError());
    return mat_refresh_derived(A->t);
}

hhp_status launch_dlda(hhp_mat *A, cudaStream_t s, const double *lambda, const double *x, double *dlda) {
    if (A->nnz == 0) return HHP_OK;
    HHP_TRY(csr_needed(A, "dL/dA"));
    k_dlda<<<grid_for(A->ctx, A->nnz, 256), 256, 0, s>>>(A->rowidx, A->col, lambda, x, A->nnz, dlda);
    A->ctx->kernel_launches += 1;
    HHP_CUDA(cudaGetLastError());
    return HHP_OK;
}

}  // namespace hhp
