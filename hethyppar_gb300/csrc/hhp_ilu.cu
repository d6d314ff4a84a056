// hhp_ilu.cu -- ILU(0) preconditioning: M = L U with L unit lower and U upper on A's pattern.
//
// This is the preconditioner of the SpSV path of gpu_BiCGStab (src/entry/bicgstab_gpu.c:185-201
// and 238-254, commented out there), where cuSPARSE's csrilu02 would factor A and two SpSV calls
// per application would solve with L and U. Both steps are sequential along the dependency
// levels of the triangles (row i of L waits for every row k < i it references), so here:
//
// * A host pass puts every row in ascending column order (a reordered matrix keeps its rows'
//   entry order), finds each row's diagonal, the levels of L (forward) and of U (backward), and
//   lays every triangle out by level: rows with at most kIluLong entries in 32-row slices
//   (column-major inside a slice, so a warp's lanes read consecutive slots, rows sorted by
//   length inside a level so a slice's lanes have similar lengths), longer rows on a list that
//   a whole warp sums, rows past kIluBig entries on one that a whole block sums.
// * One cooperative kernel factors A (IKJ order, a warp per row) and one kernel per triangle
//   solves it, each walking the levels in order with a grid barrier between levels (levels 0
//   and 1 share a pass, so a two-level triangle needs no barrier and gets an ordinary launch):
//   two launches per application whatever the level count, so the solve graph stays small.
//   Every barrier wait is bounded; a wait that runs out sets the context's error word and the
//   kernel returns, which ends the solve with HHP_ERR_TIMEOUT.
// * Values written inside a kernel by other blocks are read with ld.global.cg (L2), never from
//   L1, which may hold a stale copy of the same line.
//
// A level costs a grid barrier (about a microsecond), so the natural order of a 2D stencil
// (2N - 1 levels) is slow; a multicoloured order (hhp_reorder_color) makes the levels the
// colours -- two for the 5- and 7-point stencils.
//
// Summation orders: a short row is summed sequentially in ascending column order,
// acc = fma(-v, z, acc) from the right-hand value; a long row accumulates 32 lane partials
// (entry e on lane e mod 32) added by a butterfly and subtracted from the right-hand value, a
// very long row 1024 thread partials reduced by warp butterflies and then in warp order; the
// backward solve multiplies by the stored 1 / u_ii (an FP64 division per row per application
// would cost more than the row's FMAs on GB300's FP64 pipe). The oracle restates exactly these
// orders.
#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstring>
#include <numeric>

#include "hhp_device.cuh"
#include "hhp_internal.h"

namespace hhp {

constexpr int kIluLong = 64;           // triangle entries above which a row is summed by a warp
constexpr int kIluBig = 2048;          // ... and above which by a whole block
constexpr int kIluThreads = 1024;      // threads per block of the cooperative kernels (32 warps)
constexpr unsigned kBarrierSpins = 1u << 22;  // bounded wait (x ~64 ns sleeps: well under a second)

struct IluTri {
    int n_levels = 0, n_slices = 0, n_long = 0, n_big = 0;
    int head_slice = 0, head_long = 0, head_big = 0;  // lev_*[min(2, n_levels)], kept on the host
    int lev1_slice = 0;                               // lev_slice[1]: the first level-1 slice
    long long slots = 0;
    int *lev_slice = nullptr;        // n_levels + 1: the slices of each level
    int *lev_long = nullptr;         // n_levels + 1: the long rows of each level
    int *lev_big = nullptr;          // n_levels + 1: the block-summed rows of each level
    long long *slice_ptr = nullptr;  // n_slices + 1: slot (k, lane) of slice s at slice_ptr[s] + 32 k + lane
    int *slice_row = nullptr;        // n_slices * 32 rows (-1: padding)
    int *slice_len = nullptr;        // n_slices * 32 entry counts
    int *scol = nullptr;             // slots: columns
    double *sval = nullptr;          // slots: factor values (filled after the factorization)
    int *long_row = nullptr;         // n_long
    int *big_row = nullptr;          // n_big
    void release() {
        cudaFree(lev_slice);
        cudaFree(lev_long);
        cudaFree(lev_big);
        cudaFree(big_row);
        cudaFree(slice_ptr);
        cudaFree(slice_row);
        cudaFree(slice_len);
        cudaFree(scol);
        cudaFree(sval);
        cudaFree(long_row);
        *this = IluTri();
    }
};

struct IluDev {
    int m = 0, grid = 0;
    long long gen = 0;        // distinct for every factorization built in this process
    int *dpos = nullptr;      // m: position of each row's diagonal in the CSR arrays
    double *lu = nullptr;     // nnz: L's multipliers below the diagonal, U on and above, CSR order
    double *dinv = nullptr;   // m: 1 / u_ii
    double *y = nullptr;      // m: L^-1 r, between the two solves
    int *frow = nullptr;      // m: rows grouped by L level (the factorization's schedule)
    int *flev = nullptr;      // levels_L + 1
    IluTri L, U;
    // Two colours: every row is on level 1 of exactly one triangle (L's level-1 rows are U's
    // level-0 rows and the other way round). An application is then two passes over half the
    // rows each (see launch_ilu_apply).
    bool two_colour = false;
    unsigned *bar = nullptr;  // barrier counters: forward, backward, factorization
    int *bad = nullptr;       // first row with a zero or non-finite pivot (INT_MAX: none)
    // A row whose columns are not ascending (a matrix reordered by csr_permute keeps its rows'
    // entry order) is factored in ascending column order: col holds the sorted columns and src[q]
    // the CSR position of sorted entry q (both empty / null when every row is already sorted).
    // After hhp_mat_drop_csr, col is the matrix's own column array, taken over (ilu_keep_col).
    int *col = nullptr;
    std::vector<int> src;
};

namespace {

struct TriArgs {
    int n_levels;
    int head_slice, head_long, head_big;  // ends of the first pass's ranges (levels 0 and 1)
    int first_slice;  // where the first pass's slices start (lev1_slice: level-0 rows skipped)
    int scale;        // forward solve of two colours: out = (in - sum) * (1 / u_ii)
    int dep_out;      // backward solve of two colours: level-1 dependencies read from out
    const int *lev_slice, *lev_long, *lev_big;
    const long long *slice_ptr;
    const int *slice_row, *slice_len, *scol;
    const double *sval;
    const int *long_row, *big_row;
};

TriArgs args_of(const IluTri &t) {
    return TriArgs{t.n_levels, t.head_slice, t.head_long, t.head_big, 0, 0, 0, t.lev_slice, t.lev_long, t.lev_big,
                   t.slice_ptr, t.slice_row, t.slice_len, t.scol, t.sval, t.long_row, t.big_row};
}

__device__ __forceinline__ unsigned ld_acquire(const unsigned *p) {
    unsigned v;
    asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}

// Grid barrier number `gen` (1, 2, ...) on a counter that starts the launch at zero: every block
// adds one arrival and waits for gen * gridDim.x. Returns false (and the block must return) when
// the wait runs out or another block's did.
__device__ bool grid_barrier(unsigned *bar, unsigned gen, int *dev_err) {
    __shared__ int ok;
    __syncthreads();
    if (threadIdx.x == 0) {
        __threadfence();
        atomicAdd(bar, 1u);
        const unsigned target = gen * gridDim.x;
        int good = 1;
        unsigned spins = 0;
        while (ld_acquire(bar) < target) {
            if (*reinterpret_cast<volatile int *>(dev_err) != DEV_OK) {
                good = 0;
                break;
            }
            if (++spins > kBarrierSpins) {
                atomicExch(dev_err, DEV_ERR_TIMEOUT);
                good = 0;
                break;
            }
            __nanosleep(64);
        }
        __threadfence();
        ok = good;
    }
    __syncthreads();
    return ok != 0;
}

__device__ __forceinline__ int lower_bound(const int *col, int lo, int hi, int j) {
    while (lo < hi) {
        const int mid = lo + ((hi - lo) >> 1);
        if (col[mid] < j) lo = mid + 1;
        else hi = mid;
    }
    return lo;
}

// IKJ ILU(0), a warp per row, rows of one L level at a time. For each k < i stored in row i
// (ascending): l_ik = a_ik / u_kk, then a_ij -= l_ik u_kj for every j > k stored in both rows; the
// lanes walk the shorter of the two lists and binary-search the other. Rows of earlier levels
// (u_kk, u_kj) are final; row i's own entries change only inside its warp, ordered by __syncwarp.
__global__ void __launch_bounds__(kIluThreads) k_ilu_factor(const int *__restrict__ rowptr,
                                                            const int *__restrict__ col,
                                                            const int *__restrict__ dpos, double *lu,
                                                            const int *__restrict__ frow,
                                                            const int *__restrict__ flev, int n_levels,
                                                            unsigned *bar, int *bad, int *dev_err) {
    const int lane = threadIdx.x & 31;
    const int gw = static_cast<int>((blockIdx.x * blockDim.x + threadIdx.x) >> 5);
    const int W = static_cast<int>((gridDim.x * blockDim.x) >> 5);
    for (int lev = 0; lev < n_levels; ++lev) {
        for (int t = flev[lev] + gw; t < flev[lev + 1]; t += W) {
            const int i = frow[t];
            const int re = rowptr[i + 1], di = dpos[i];
            for (int p = rowptr[i]; p < di; ++p) {
                const int k = col[p];
                const double l = __ldcg(lu + p) / __ldcg(lu + dpos[k]);
                __syncwarp();  // every lane has read a_ik before it is overwritten
                if (lane == 0) __stcg(lu + p, l);
                const int kb = dpos[k] + 1, ke = rowptr[k + 1];
                if (re - (p + 1) <= ke - kb) {
                    for (int q = p + 1 + lane; q < re; q += 32) {
                        const int j = col[q];
                        const int t2 = lower_bound(col, kb, ke, j);
                        if (t2 < ke && col[t2] == j) __stcg(lu + q, fma(-l, __ldcg(lu + t2), __ldcg(lu + q)));
                    }
                } else {
                    for (int t2 = kb + lane; t2 < ke; t2 += 32) {
                        const int j = col[t2];
                        const int q = lower_bound(col, p + 1, re, j);
                        if (q < re && col[q] == j) __stcg(lu + q, fma(-l, __ldcg(lu + t2), __ldcg(lu + q)));
                    }
                }
                __syncwarp();
            }
            if (lane == 0) {
                const double u = __ldcg(lu + di);
                if (u == 0.0 || !isfinite(u)) atomicMin(bad, i);
            }
        }
        if (lev + 1 < n_levels && !grid_barrier(bar, static_cast<unsigned>(lev + 1), dev_err)) return;
    }
}

// The value of dependency c: out[c], written by this kernel at an earlier level (read from L2:
// another SM wrote it), except on level 1, whose dependencies are all level-0 rows -- rows with
// no entries in this triangle, out[c] = in[c] (forward) or in[c] * (1 / u_cc) (backward) --
// formed straight from `in`, so levels 0 and 1 share one pass with no grid barrier between them.
// Both ways give the same bits.
template <bool UPPER>
struct Dep {
    const double *in, *dinv, *out;
    bool from_in;
    __device__ __forceinline__ double operator()(int c) const {
        if (from_in) return UPPER ? in[c] * dinv[c] : in[c];
        return __ldcg(out + c);
    }
};

// sum over p in [b, e) step `stride`, starting at `first`, of lu[p] * z(col[p]), one fused
// multiply-add per entry in ascending p; four entries' loads are issued before their FMAs
template <typename Z>
__device__ __forceinline__ double strided_dot(const double *__restrict__ lu, const int *__restrict__ col, const Z &z,
                                              int first, int e, int stride) {
    double acc = 0.0;
    int p = first;
    for (; p + 3 * stride < e; p += 4 * stride) {
        const int c0 = col[p], c1 = col[p + stride], c2 = col[p + 2 * stride], c3 = col[p + 3 * stride];
        const double v0 = lu[p], v1 = lu[p + stride], v2 = lu[p + 2 * stride], v3 = lu[p + 3 * stride];
        const double z0 = z(c0), z1 = z(c1), z2 = z(c2), z3 = z(c3);
        acc = fma(v0, z0, acc);
        acc = fma(v1, z1, acc);
        acc = fma(v2, z2, acc);
        acc = fma(v3, z3, acc);
    }
    for (; p < e; p += stride) acc = fma(lu[p], z(col[p]), acc);
    return acc;
}

// One triangular solve, level by level. Forward (UPPER false): out_i = in_i - sum l_ik out_k.
// Backward (UPPER true): out_i = (in_i - sum u_ij out_j) * (1 / u_ii). Per level: rows with more
// than kIluBig entries a block each (thread t sums entries t, t + blockDim, ...; warp
// butterflies, then the warp sums in warp order), rows with more than kIluLong a warp each
// (lane l sums entries l, l + 32, ...; a butterfly), the rest a lane each in 32-row slices
// (sequential, from the right-hand value). Levels 0 and 1 run in one pass (see Dep), every later
// level after a grid barrier: a two-level (two-colour) triangle needs none. Returns at once when
// the solver's status word says the loop has ended. The kernel clears the other triangle's
// barrier counter (that kernel is not running: launches are stream-ordered), so a forward and a
// backward solve alternate with no reset of their own.
template <bool UPPER>
__global__ void __launch_bounds__(kIluThreads, 1) k_ilu_tri(TriArgs t, const int *__restrict__ rowptr,
                                                         const int *__restrict__ col,
                                                         const int *__restrict__ dpos,
                                                         const double *__restrict__ lu,
                                                         const double *__restrict__ dinv,
                                                         const double *__restrict__ in, double *out,
                                                         unsigned *bar, unsigned *bar_other, const int *stop,
                                                         int *dev_err) {
    __shared__ double wsum[kIluThreads / 32];
    if (blockIdx.x == 0 && threadIdx.x == 0) *bar_other = 0u;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int gw = static_cast<int>((blockIdx.x * blockDim.x + threadIdx.x) >> 5);
    const int W = static_cast<int>((gridDim.x * blockDim.x) >> 5);
    // The first pass's bounds are arguments, so this warp's first slices' row data is pulled into
    // L1 while the two status words (written by earlier launches) are read together.
    for (int s = t.first_slice + gw; s < t.head_slice && s < t.first_slice + gw + 2 * W; s += W) {
        asm volatile("prefetch.global.L1 [%0];" ::"l"(t.slice_row + 32LL * s + lane));
        asm volatile("prefetch.global.L1 [%0];" ::"l"(t.slice_len + 32LL * s + lane));
        asm volatile("prefetch.global.L1 [%0];" ::"l"(t.slice_ptr + s));
    }
    const int run = stop ? *reinterpret_cast<volatile const int *>(stop) : ST_RUNNING;
    const int err = *reinterpret_cast<volatile int *>(dev_err);
    if (run != ST_RUNNING || err != DEV_OK) return;
    unsigned barriers = 0;
    for (int lev = 0; lev < t.n_levels; ++lev) {
        // levels 0 and 1 as one range of rows (level-0 rows have no entries, so `z` is never
        // called for them): a warp's slices of both levels are in flight together
        const bool head = lev == 0;
        const int le = head && t.n_levels > 1 ? 2 : lev + 1;
        const Dep<UPPER> z{in, dinv, out, le == 2 && !t.dep_out};
        const bool scale = UPPER || t.scale;
        const int big_lo = head ? 0 : t.lev_big[lev], big_hi = head ? t.head_big : t.lev_big[le];
        for (int q = big_lo + blockIdx.x; q < big_hi; q += gridDim.x) {
            const int row = t.big_row[q];
            const int b = UPPER ? dpos[row] + 1 : rowptr[row];
            const int e = UPPER ? rowptr[row + 1] : dpos[row];
            const double acc = warp_sum(strided_dot(lu, col, z, b + threadIdx.x, e, kIluThreads));
            if (lane == 0) wsum[warp] = acc;
            __syncthreads();
            if (threadIdx.x == 0) {
                double tot = 0.0;
                for (int w = 0; w < kIluThreads / 32; ++w) tot += wsum[w];
                double r = in[row] - tot;
                if (scale) r = r * dinv[row];
                __stcg(out + row, r);
            }
            __syncthreads();
        }
        const int long_lo = head ? 0 : t.lev_long[lev], long_hi = head ? t.head_long : t.lev_long[le];
        for (int q = long_lo + gw; q < long_hi; q += W) {
            const int row = t.long_row[q];
            const int b = UPPER ? dpos[row] + 1 : rowptr[row];
            const int e = UPPER ? rowptr[row + 1] : dpos[row];
            const double acc = warp_sum(strided_dot(lu, col, z, b + lane, e, 32));
            if (lane == 0) {
                double r = in[row] - acc;
                if (scale) r = r * dinv[row];
                __stcg(out + row, r);
            }
        }
        // Two slices per pass (s and s + W), four steps at a time: every load of a group is issued
        // before its FMAs, so a warp has two slices' chains of dependent requests (row data, then
        // slots, then gathers) in flight at once. A step past a lane's row length loads nothing
        // and adds fma(-0, 0, acc), which leaves acc unchanged bit for bit.
        const int s_hi = head ? t.head_slice : t.lev_slice[le];
        for (int s = (head ? t.first_slice : t.lev_slice[lev]) + gw; s < s_hi; s += 2 * W) {
            const int sb = s + W;
            const bool two = sb < s_hi;
            const int r0 = t.slice_row[32 * s + lane];
            const int n0 = t.slice_len[32 * s + lane];
            const long long q0 = t.slice_ptr[s] + lane;
            const int r1 = two ? t.slice_row[32 * sb + lane] : -1;
            const int n1 = two ? t.slice_len[32 * sb + lane] : 0;
            const long long q1 = two ? t.slice_ptr[sb] + lane : 0;
            double a0 = r0 >= 0 ? in[r0] : 0.0, a1 = r1 >= 0 ? in[r1] : 0.0;
            const int len = max(n0, n1);
            for (int k = 0; k < len; k += 4) {
                int c[8];
                double v[8], zz[8];
#pragma unroll
                for (int j = 0; j < 4; ++j) {
                    const bool p0 = k + j < n0, p1 = k + j < n1;
                    c[j] = p0 ? t.scol[q0 + 32LL * (k + j)] : 0;
                    v[j] = p0 ? t.sval[q0 + 32LL * (k + j)] : 0.0;
                    c[4 + j] = p1 ? t.scol[q1 + 32LL * (k + j)] : 0;
                    v[4 + j] = p1 ? t.sval[q1 + 32LL * (k + j)] : 0.0;
                }
#pragma unroll
                for (int j = 0; j < 4; ++j) {
                    zz[j] = k + j < n0 ? z(c[j]) : 0.0;
                    zz[4 + j] = k + j < n1 ? z(c[4 + j]) : 0.0;
                }
#pragma unroll
                for (int j = 0; j < 4; ++j) a0 = fma(-v[j], zz[j], a0);
#pragma unroll
                for (int j = 0; j < 4; ++j) a1 = fma(-v[4 + j], zz[4 + j], a1);
            }
            if (r0 >= 0) __stcg(out + r0, scale ? a0 * dinv[r0] : a0);
            if (r1 >= 0) __stcg(out + r1, scale ? a1 * dinv[r1] : a1);
        }
        lev = le - 1;
        if (lev >= 1 && lev + 1 < t.n_levels && !grid_barrier(bar, ++barriers, dev_err)) return;
    }
}

// Slot values and u_ii from the factor (sidx: the CSR position of every slot).
__global__ void k_ilu_fill(const double *__restrict__ lu, const int *__restrict__ sidx, long long slots,
                           double *__restrict__ sval) {
    for (long long q = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; q < slots;
         q += static_cast<long long>(gridDim.x) * blockDim.x) {
        const int p = sidx[q];
        sval[q] = p >= 0 ? lu[p] : 0.0;
    }
}
__global__ void k_ilu_gather(const double *__restrict__ val, const int *__restrict__ src, int nnz,
                             double *__restrict__ lu) {
    for (int q = blockIdx.x * blockDim.x + threadIdx.x; q < nnz; q += gridDim.x * blockDim.x) lu[q] = val[src[q]];
}
__global__ void k_ilu_diag(const double *__restrict__ lu, const int *__restrict__ dpos, int m,
                           double *__restrict__ dinv) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < m; i += gridDim.x * blockDim.x) dinv[i] = 1.0 / lu[dpos[i]];
}

// ---- host analysis -----------------------------------------------------------------------------
struct TriHost {
    int n_levels = 0;
    std::vector<int> lev_slice, lev_long, lev_big, slice_row, slice_len, scol, sidx, long_row, big_row;
    std::vector<long long> slice_ptr;
};

// Rows grouped by level (lev[i] in [0, nlev)), each level's rows by descending entry count
// (ties by row), then cut into 32-row slices; rows with more than kIluBig entries go to the big
// list, the others with more than kIluLong to the long list. first(i) / count(i): the row's
// entries in this triangle.
template <typename First, typename Count>
void layout_triangle(int m, const std::vector<int> &lev, int nlev, const int *col, First first, Count count,
                     TriHost &T) {
    T.n_levels = nlev;
    std::vector<int> start(static_cast<size_t>(nlev) + 1, 0);
    for (int i = 0; i < m; ++i) ++start[static_cast<size_t>(lev[static_cast<size_t>(i)]) + 1];
    std::partial_sum(start.begin(), start.end(), start.begin());
    std::vector<int> rows(static_cast<size_t>(m)), fill(start.begin(), start.end() - 1);
    for (int i = 0; i < m; ++i) rows[static_cast<size_t>(fill[static_cast<size_t>(lev[static_cast<size_t>(i)])]++)] = i;
    T.lev_slice.assign(1, 0);
    T.lev_long.assign(1, 0);
    T.lev_big.assign(1, 0);
    T.slice_ptr.assign(1, 0);
    for (int l = 0; l < nlev; ++l) {
        auto b = rows.begin() + start[static_cast<size_t>(l)], e = rows.begin() + start[static_cast<size_t>(l) + 1];
        std::stable_sort(b, e, [&](int x, int y) { return count(x) > count(y); });
        auto it = b;
        for (; it != e && count(*it) > kIluBig; ++it) T.big_row.push_back(*it);
        for (; it != e && count(*it) > kIluLong; ++it) T.long_row.push_back(*it);
        for (; it != e; it += std::min<std::ptrdiff_t>(32, e - it)) {
            const int nr = static_cast<int>(std::min<std::ptrdiff_t>(32, e - it));
            const int width = count(*it);
            const long long base = T.slice_ptr.back();
            T.slice_ptr.push_back(base + 32LL * width);
            T.scol.resize(static_cast<size_t>(base + 32LL * width), 0);
            T.sidx.resize(static_cast<size_t>(base + 32LL * width), -1);
            for (int j = 0; j < 32; ++j) {
                const int row = j < nr ? it[j] : -1;
                T.slice_row.push_back(row);
                T.slice_len.push_back(row >= 0 ? count(row) : 0);
                if (row < 0) continue;
                const int f = first(row), c = count(row);
                for (int k = 0; k < c; ++k) {
                    const size_t q = static_cast<size_t>(base + 32LL * k + j);
                    T.scol[q] = col[f + k];
                    T.sidx[q] = f + k;
                }
            }
        }
        T.lev_slice.push_back(static_cast<int>(T.slice_ptr.size()) - 1);
        T.lev_long.push_back(static_cast<int>(T.long_row.size()));
        T.lev_big.push_back(static_cast<int>(T.big_row.size()));
    }
}

// Host array -> new device array, ordered on the context's (non-blocking) stream like every other
// upload of the library: a legacy-stream copy from pageable memory may still be in flight when the
// call returns, unordered against that stream's kernels. (A pageable source is staged before the
// call returns, so the host vector may go right after.)
template <typename V>
hhp_status upload(V **dst, const std::vector<V> &src, cudaStream_t st) {
    if (src.empty()) return HHP_OK;
    HHP_CUDA(cudaMalloc(dst, sizeof(V) * src.size()));
    HHP_CUDA(cudaMemcpyAsync(*dst, src.data(), sizeof(V) * src.size(), cudaMemcpyHostToDevice, st));
    return HHP_OK;
}

hhp_status upload_tri(const TriHost &h, IluTri &d, int **sidx_dev, cudaStream_t st) {
    d.n_levels = h.n_levels;
    d.n_slices = static_cast<int>(h.slice_ptr.size()) - 1;
    d.n_long = static_cast<int>(h.long_row.size());
    d.n_big = static_cast<int>(h.big_row.size());
    d.slots = h.slice_ptr.back();
    const size_t head = static_cast<size_t>(std::min(2, h.n_levels));
    d.head_slice = h.lev_slice[head];
    d.head_long = h.lev_long[head];
    d.head_big = h.lev_big[head];
    d.lev1_slice = h.n_levels >= 2 ? h.lev_slice[1] : 0;
    HHP_TRY(upload(&d.lev_slice, h.lev_slice, st));
    HHP_TRY(upload(&d.lev_long, h.lev_long, st));
    HHP_TRY(upload(&d.slice_ptr, h.slice_ptr, st));
    HHP_TRY(upload(&d.slice_row, h.slice_row, st));
    HHP_TRY(upload(&d.slice_len, h.slice_len, st));
    HHP_TRY(upload(&d.scol, h.scol, st));
    HHP_TRY(upload(&d.long_row, h.long_row, st));
    HHP_TRY(upload(&d.lev_big, h.lev_big, st));
    HHP_TRY(upload(&d.big_row, h.big_row, st));
    HHP_TRY(upload(sidx_dev, h.sidx, st));
    if (d.slots > 0) HHP_CUDA(cudaMalloc(&d.sval, sizeof(double) * static_cast<size_t>(d.slots)));
    return HHP_OK;
}

// A launch whose blocks wait on one another (coop) is cooperative: the runtime guarantees that
// all of them are resident together. A triangle of at most two levels has no barrier (levels 0
// and 1 share a pass), so its launch is an ordinary one.
cudaError_t launch_coop(const void *func, int grid, void **args, cudaStream_t st, bool coop = true) {
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(static_cast<unsigned>(grid));
    cfg.blockDim = dim3(kIluThreads);
    cfg.stream = st;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeCooperative;
    attr[0].val.cooperative = 1;
    cfg.attrs = coop ? attr : nullptr;
    cfg.numAttrs = coop ? 1 : 0;
    return cudaLaunchKernelExC(&cfg, func, args);
}

hhp_status build_ilu(hhp_mat *A, IluDev *I, int *levels_out) {
    const int m = A->m;
    cudaStream_t st = A->ctx->stream;
    const std::vector<int> &rp = A->rowptr_host;
    std::vector<int> col(static_cast<size_t>(A->nnz));
    HHP_CUDA(cudaStreamSynchronize(st));
    if (A->nnz) HHP_CUDA(cudaMemcpy(col.data(), A->col, sizeof(int) * col.size(), cudaMemcpyDeviceToHost));
    // rows in ascending column order (a stable sort of the rows that are not), then the
    // diagonal positions; a column stored twice in a row is refused
    bool sorted = true;
    for (int i = 0; i < m && sorted; ++i)
        for (int p = rp[static_cast<size_t>(i)] + 1; p < rp[static_cast<size_t>(i) + 1]; ++p)
            if (col[static_cast<size_t>(p)] <= col[static_cast<size_t>(p) - 1]) {
                sorted = false;
                break;
            }
    if (!sorted) {
        I->src.resize(col.size());
        std::iota(I->src.begin(), I->src.end(), 0);
        std::vector<int> sc(col.size());
        for (int i = 0; i < m; ++i) {
            auto b = I->src.begin() + rp[static_cast<size_t>(i)], e = I->src.begin() + rp[static_cast<size_t>(i) + 1];
            std::stable_sort(b, e, [&](int x, int y) { return col[static_cast<size_t>(x)] < col[static_cast<size_t>(y)]; });
        }
        for (size_t q = 0; q < col.size(); ++q) sc[q] = col[static_cast<size_t>(I->src[q])];
        col.swap(sc);
    }
    std::vector<int> dpos(static_cast<size_t>(m), -1);
    for (int i = 0; i < m; ++i) {
        for (int p = rp[static_cast<size_t>(i)]; p < rp[static_cast<size_t>(i) + 1]; ++p) {
            const int c = col[static_cast<size_t>(p)];
            if (p > rp[static_cast<size_t>(i)] && c == col[static_cast<size_t>(p) - 1]) {
                set_error("ilu0: row %d stores column %d twice", i, c);
                return HHP_ERR_ARG;
            }
            if (c == i) dpos[static_cast<size_t>(i)] = p;
        }
        if (dpos[static_cast<size_t>(i)] < 0) {
            set_error("ilu0 needs every diagonal entry stored; row %d has none", i);
            return HHP_ERR_ARG;
        }
    }
    // levels: L forward (rows ascending), U backward (rows descending)
    std::vector<int> levL(static_cast<size_t>(m)), levU(static_cast<size_t>(m));
    int nL = 0, nU = 0;
    for (int i = 0; i < m; ++i) {
        int lv = 0;
        for (int p = rp[static_cast<size_t>(i)]; p < dpos[static_cast<size_t>(i)]; ++p)
            lv = std::max(lv, levL[static_cast<size_t>(col[static_cast<size_t>(p)])] + 1);
        levL[static_cast<size_t>(i)] = lv;
        nL = std::max(nL, lv + 1);
    }
    for (int i = m - 1; i >= 0; --i) {
        int lv = 0;
        for (int p = dpos[static_cast<size_t>(i)] + 1; p < rp[static_cast<size_t>(i) + 1]; ++p)
            lv = std::max(lv, levU[static_cast<size_t>(col[static_cast<size_t>(p)])] + 1);
        levU[static_cast<size_t>(i)] = lv;
        nU = std::max(nU, lv + 1);
    }
    if (levels_out) {
        levels_out[0] = nL;
        levels_out[1] = nU;
    }
    I->two_colour = nL == 2 && nU == 2;
    for (int i = 0; i < m && I->two_colour; ++i)
        I->two_colour = levL[static_cast<size_t>(i)] + levU[static_cast<size_t>(i)] == 1;
    TriHost TL, TU;
    const int *cp = col.data();
    layout_triangle(
        m, levL, nL, cp, [&](int i) { return rp[static_cast<size_t>(i)]; },
        [&](int i) { return dpos[static_cast<size_t>(i)] - rp[static_cast<size_t>(i)]; }, TL);
    layout_triangle(
        m, levU, nU, cp, [&](int i) { return dpos[static_cast<size_t>(i)] + 1; },
        [&](int i) { return rp[static_cast<size_t>(i) + 1] - dpos[static_cast<size_t>(i)] - 1; }, TU);
    // factorization schedule: rows by L level, ascending inside a level
    std::vector<int> flev(static_cast<size_t>(nL) + 1, 0), frow(static_cast<size_t>(m));
    for (int i = 0; i < m; ++i) ++flev[static_cast<size_t>(levL[static_cast<size_t>(i)]) + 1];
    std::partial_sum(flev.begin(), flev.end(), flev.begin());
    {
        std::vector<int> f(flev.begin(), flev.end() - 1);
        for (int i = 0; i < m; ++i) frow[static_cast<size_t>(f[static_cast<size_t>(levL[static_cast<size_t>(i)])]++)] = i;
    }
    // device copies
    I->m = m;
    int *sidxL = nullptr, *sidxU = nullptr;
    hhp_status rc = HHP_OK;
    do {
        if (!sorted && (rc = upload(&I->col, col, st)) != HHP_OK) break;
        if ((rc = upload(&I->dpos, dpos, st)) != HHP_OK) break;
        if ((rc = upload(&I->frow, frow, st)) != HHP_OK) break;
        if ((rc = upload(&I->flev, flev, st)) != HHP_OK) break;
        if ((rc = upload_tri(TL, I->L, &sidxL, st)) != HHP_OK) break;
        if ((rc = upload_tri(TU, I->U, &sidxU, st)) != HHP_OK) break;
        if (cudaMalloc(&I->lu, sizeof(double) * (static_cast<size_t>(A->nnz) + 1)) != cudaSuccess ||
            cudaMalloc(&I->dinv, sizeof(double) * static_cast<size_t>(m)) != cudaSuccess ||
            cudaMalloc(&I->y, sizeof(double) * static_cast<size_t>(m)) != cudaSuccess ||
            cudaMalloc(&I->bar, 4 * sizeof(unsigned)) != cudaSuccess || cudaMalloc(&I->bad, sizeof(int)) != cudaSuccess) {
            set_error("out of device memory for the ILU(0) factors");
            rc = HHP_ERR_OOM;
            break;
        }
        // cooperative grid: every block resident at once (the blocks wait on one another)
        int occ_f = 0, occ_l = 0, occ_u = 0;
        if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ_f, k_ilu_factor, kIluThreads, 0) != cudaSuccess ||
            cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ_l, k_ilu_tri<false>, kIluThreads, 0) != cudaSuccess ||
            cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ_u, k_ilu_tri<true>, kIluThreads, 0) != cudaSuccess) {
            rc = HHP_ERR_CUDA;
            break;
        }
        // one 1024-thread block per SM (64 registers a thread, no spills); measured against 2 x 512,
        // 4 x 512 (32 registers, spilling) and 4 x 256: within 5 % on the stencils, best on the
        // power-law system, whose longest rows are summed block-wide
        const int per_sm = std::min(occ_f, std::min(occ_l, occ_u));
        if (per_sm < 1) {
            set_error("ilu0: the triangular-solve kernels cannot be resident on an SM");
            rc = HHP_ERR_CUDA;
            break;
        }
        I->grid = per_sm * A->ctx->num_sms;
        // factor: lu = val, then the cooperative level walk
        const int none = 0x7fffffff;
        if (cudaMemsetAsync(I->bar, 0, 4 * sizeof(unsigned), st) != cudaSuccess ||
            cudaMemcpyAsync(I->bad, &none, sizeof(int), cudaMemcpyHostToDevice, st) != cudaSuccess ||
            cudaMemsetAsync(A->ctx->dev_err, 0, sizeof(int), st) != cudaSuccess) {
            rc = HHP_ERR_CUDA;
            break;
        }
        if (sorted) {
            if (A->nnz && cudaMemcpyAsync(I->lu, A->val, sizeof(double) * static_cast<size_t>(A->nnz),
                                          cudaMemcpyDeviceToDevice, st) != cudaSuccess) {
                rc = HHP_ERR_CUDA;
                break;
            }
        } else {
            int *src_dev = nullptr;
            if ((rc = upload(&src_dev, I->src, st)) != HHP_OK) break;
            k_ilu_gather<<<4 * A->ctx->num_sms, 256, 0, st>>>(A->val, src_dev, A->nnz, I->lu);
            const cudaError_t ge = cudaGetLastError();
            const cudaError_t se = cudaStreamSynchronize(st);
            cudaFree(src_dev);
            A->ctx->kernel_launches += 1;
            if (ge != cudaSuccess || se != cudaSuccess) {
                rc = HHP_ERR_CUDA;
                break;
            }
        }
        {
            const int *a_rp = A->rowptr, *a_col = I->col ? I->col : A->col, *a_dpos = I->dpos, *a_frow = I->frow,
                      *a_flev = I->flev;
            double *a_lu = I->lu;
            int nlev = nL;
            unsigned *a_bar = I->bar + 2;
            int *a_bad = I->bad, *a_err = A->ctx->dev_err;
            void *args[] = {&a_rp, &a_col, &a_dpos, &a_lu, &a_frow, &a_flev, &nlev, &a_bar, &a_bad, &a_err};
            if (launch_coop(reinterpret_cast<const void *>(k_ilu_factor), I->grid, args, st) != cudaSuccess) {
                rc = HHP_ERR_CUDA;
                break;
            }
            A->ctx->kernel_launches += 1;
        }
        int first_bad = none, err = DEV_OK;
        if (cudaMemcpyAsync(&first_bad, I->bad, sizeof(int), cudaMemcpyDeviceToHost, st) != cudaSuccess ||
            cudaMemcpyAsync(&err, A->ctx->dev_err, sizeof(int), cudaMemcpyDeviceToHost, st) != cudaSuccess ||
            cudaStreamSynchronize(st) != cudaSuccess) {
            rc = HHP_ERR_CUDA;
            break;
        }
        if (err != DEV_OK) {
            set_error("ilu0: a bounded wait of the factorization timed out");
            rc = HHP_ERR_TIMEOUT;
            break;
        }
        if (first_bad != none) {
            set_error("ilu0: zero or non-finite pivot u_ii at row %d", first_bad);
            rc = HHP_ERR_BREAKDOWN;
            break;
        }
        const int g = 4 * A->ctx->num_sms;
        if (I->L.slots) k_ilu_fill<<<g, 256, 0, st>>>(I->lu, sidxL, I->L.slots, I->L.sval);
        if (I->U.slots) k_ilu_fill<<<g, 256, 0, st>>>(I->lu, sidxU, I->U.slots, I->U.sval);
        k_ilu_diag<<<g, 256, 0, st>>>(I->lu, I->dpos, m, I->dinv);
        A->ctx->kernel_launches += 3;
        if (cudaGetLastError() != cudaSuccess || cudaStreamSynchronize(st) != cudaSuccess) rc = HHP_ERR_CUDA;
    } while (0);
    cudaFree(sidxL);
    cudaFree(sidxU);
    if (rc == HHP_ERR_CUDA) set_error("building the ILU(0) factors failed: %s", cudaGetErrorString(cudaGetLastError()));
    return rc;
}

void free_ilu(IluDev *I) {
    if (!I) return;
    I->L.release();
    I->U.release();
    cudaFree(I->dpos);
    cudaFree(I->lu);
    cudaFree(I->dinv);
    cudaFree(I->y);
    cudaFree(I->frow);
    cudaFree(I->flev);
    cudaFree(I->bar);
    cudaFree(I->bad);
    cudaFree(I->col);
    delete I;
}

}  // namespace

hhp_status ensure_ilu(hhp_mat *A, int *levels) {
    if (A->ilu) {
        if (levels) {
            levels[0] = A->ilu->L.n_levels;
            levels[1] = A->ilu->U.n_levels;
        }
        return HHP_OK;
    }
    if (A->m != A->n || A->m == 0) {
        set_error("ilu0 needs a square, non-empty matrix");
        return HHP_ERR_ARG;
    }
    HHP_TRY(csr_needed(A, "ILU(0)"));
    IluDev *I = new IluDev();
    hhp_status rc;
    try {
        rc = build_ilu(A, I, levels);
    } catch (...) {  // host allocation failure: release the device arrays, then report
        free_ilu(I);
        throw;
    }
    if (rc != HHP_OK) {
        free_ilu(I);
        return rc;
    }
    static std::atomic<long long> builds{0};
    I->gen = ++builds;
    A->ilu = I;
    return HHP_OK;
}

long long ilu_generation(const hhp_mat *A) { return A->ilu ? A->ilu->gen : 0; }

void release_ilu(hhp_mat *A) {
    free_ilu(A->ilu);
    A->ilu = nullptr;
}

void ilu_keep_col(hhp_mat *A) {
    // the warp- and block-summed rows of the triangles read their columns from this array
    if (A->ilu && !A->ilu->col) {
        A->ilu->col = A->col;
        A->col = nullptr;
    }
}

hhp_status launch_ilu_apply(hhp_mat *A, cudaStream_t st, const double *in, double *out, const int *stop) {
    IluDev *I = A->ilu;
    if (!I) {
        set_error("ilu0: no factorization");
        return HHP_ERR_STATE;
    }
    const int *rp = A->rowptr, *col = I->col ? I->col : A->col, *dpos = I->dpos;
    const double *lu = I->lu, *dinv = I->dinv;
    int *err = A->ctx->dev_err;
    if (I->two_colour) {
        // L's level-1 rows are U's level-0 rows: their final value is (r_i - sum l_ik r_k) / u_ii,
        // which the forward pass writes straight to out. U's level-1 rows are L's level-0 rows,
        // whose y is r itself: the backward pass reads r and the forward pass's results. Each
        // pass walks half the rows, y is not used, and every value is the one the two full
        // solves give, bit for bit (same sums, same order, the same multiplication by 1 / u_ii).
        unsigned *b = I->bar, *bo = I->bar + 1;
        const double *x = in;
        double *y = out;
        {
            TriArgs t = args_of(I->L);
            t.first_slice = I->L.lev1_slice;
            t.scale = 1;
            void *args[] = {&t, &rp, &col, &dpos, &lu, &dinv, &x, &y, &b, &bo, &stop, &err};
            HHP_CUDA(launch_coop(reinterpret_cast<const void *>(k_ilu_tri<false>), I->grid, args, st, false));
        }
        {
            TriArgs t = args_of(I->U);
            t.first_slice = I->U.lev1_slice;
            t.dep_out = 1;
            void *args[] = {&t, &rp, &col, &dpos, &lu, &dinv, &x, &y, &bo, &b, &stop, &err};
            HHP_CUDA(launch_coop(reinterpret_cast<const void *>(k_ilu_tri<true>), I->grid, args, st, false));
        }
        A->ctx->kernel_launches += 2;
        return HHP_OK;
    }
    {  // y = L^-1 in
        TriArgs t = args_of(I->L);
        unsigned *b = I->bar, *bo = I->bar + 1;
        const double *x = in;
        double *y = I->y;
        void *args[] = {&t, &rp, &col, &dpos, &lu, &dinv, &x, &y, &b, &bo, &stop, &err};
        HHP_CUDA(launch_coop(reinterpret_cast<const void *>(k_ilu_tri<false>), I->grid, args, st, I->L.n_levels > 2));
    }
    {  // out = U^-1 y
        TriArgs t = args_of(I->U);
        unsigned *b = I->bar + 1, *bo = I->bar;
        const double *x = I->y;
        double *y = out;
        void *args[] = {&t, &rp, &col, &dpos, &lu, &dinv, &x, &y, &b, &bo, &stop, &err};
        HHP_CUDA(launch_coop(reinterpret_cast<const void *>(k_ilu_tri<true>), I->grid, args, st, I->U.n_levels > 2));
    }
    A->ctx->kernel_launches += 2;
    return HHP_OK;
}

hhp_status ilu_factors(hhp_mat *A, double *lu_host) {
    if (!A->ilu) return HHP_ERR_STATE;
    HHP_CUDA(cudaStreamSynchronize(A->ctx->stream));
    if (!A->nnz) return HHP_OK;
    const std::vector<int> &src = A->ilu->src;
    if (src.empty()) {
        HHP_CUDA(cudaMemcpy(lu_host, A->ilu->lu, sizeof(double) * static_cast<size_t>(A->nnz), cudaMemcpyDeviceToHost));
        return HHP_OK;
    }
    std::vector<double> lu(static_cast<size_t>(A->nnz));
    HHP_CUDA(cudaMemcpy(lu.data(), A->ilu->lu, sizeof(double) * lu.size(), cudaMemcpyDeviceToHost));
    for (size_t q = 0; q < lu.size(); ++q) lu_host[src[q]] = lu[q];  // back to A's entry order
    return HHP_OK;
}

}  // namespace hhp
