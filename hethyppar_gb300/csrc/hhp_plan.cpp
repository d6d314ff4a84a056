// hhp_plan.cpp -- host-side construction of the SpMV work plan (row-length binning + balanced
// contiguous per-warp ranges).
//
// Rows are binned by length:
//   len <= med          -> grouped, in row order, into ROWS items of up to 32 rows and at most
//                          `cap` nonzeros; each lane sums one row sequentially (vector-per-row
//                          degenerates to thread-per-row: no intra-row reduction, so the sum
//                          order equals the CSR order of the reference's CSR_spmxv_seq,
//                          src/util/hhp_cpu.c:445-455, with each step fused)
//   med < len <= cap    -> one VEC item: the row is summed by a whole warp
//   len > cap           -> CHUNK items of `cap` nonzeros (merge-path-style equal-nnz slices),
//                          combined in slice order
// The item list (in row order) is then cut into n_warps contiguous ranges of near-equal work,
// like a merge-path split of the (rows + nonzeros) list: warp g takes the items whose work
// midpoint falls in [g*W/G, (g+1)*W/G).
#include <algorithm>
#include <cmath>

#include "hhp_internal.h"

namespace hhp {

void build_plan(int m, const int *rowptr, int n_warps, int cap, int med, PlanHost &P) {
    P = PlanHost();
    P.n_warps = n_warps;
    P.cap = cap;
    P.med = med;
    std::vector<long long> work;
    P.items.reserve(static_cast<size_t>(m) / 16 + 16);
    work.reserve(static_cast<size_t>(m) / 16 + 16);

    int t_r0 = -1, t_rows = 0, t_k0 = 0, t_k1 = 0;
    auto close_tile = [&]() {
        if (t_rows > 0) {
            P.items.push_back(make_int4(t_r0, (KIND_ROWS << KIND_SHIFT) | t_rows, t_k0, t_k1));
            work.push_back(static_cast<long long>(t_k1 - t_k0) + 2LL * t_rows + 16);
            P.max_item_nnz = std::max<long long>(P.max_item_nnz, t_k1 - t_k0);
        }
        t_rows = 0;
    };
    int n_chunks = 0;
    for (int r = 0; r < m; ++r) {
        const int k0 = rowptr[r], k1 = rowptr[r + 1], len = k1 - k0;
        if (len > cap) {
            close_tile();
            const int l = static_cast<int>(P.long_rows.size());
            P.long_rows.push_back(r);
            P.long_first.push_back(n_chunks);
            for (int a = k0; a < k1; a += cap) {
                const int b = std::min(a + cap, k1);
                P.items.push_back(make_int4(r, (KIND_CHUNK << KIND_SHIFT) | n_chunks, a, b));
                work.push_back(static_cast<long long>(b - a) + 18);
                P.chunk_long.push_back(l);
                P.max_item_nnz = std::max<long long>(P.max_item_nnz, b - a);
                ++n_chunks;
            }
        } else if (len > med) {
            close_tile();
            P.items.push_back(make_int4(r, (KIND_VEC << KIND_SHIFT) | 1, k0, k1));
            work.push_back(static_cast<long long>(len) + 18);
            P.max_item_nnz = std::max<long long>(P.max_item_nnz, len);
        } else {
            if (t_rows == 32 || (t_rows > 0 && (t_k1 - t_k0) + len > cap)) close_tile();
            if (t_rows == 0) {
                t_r0 = r;
                t_k0 = k0;
            }
            t_k1 = k1;
            ++t_rows;
        }
    }
    close_tile();
    P.long_first.push_back(n_chunks);

    // Balanced contiguous split.
    const size_t ni = P.items.size();
    long long total = 0;
    for (long long w : work) total += w;
    P.warp_begin.assign(static_cast<size_t>(n_warps) + 1, static_cast<int>(ni));  // trailing warps: empty
    std::vector<long long> per_warp(static_cast<size_t>(n_warps), 0);
    if (ni > 0 && total > 0) {
        long long prefix = 0;
        int cur = -1;
        for (size_t i = 0; i < ni; ++i) {
            const long double mid = static_cast<long double>(prefix) + 0.5L * static_cast<long double>(work[i]);
            int g = static_cast<int>(mid * n_warps / static_cast<long double>(total));
            g = std::min(std::max(g, 0), n_warps - 1);
            if (g < cur) g = cur;
            while (cur < g) P.warp_begin[static_cast<size_t>(++cur)] = static_cast<int>(i);
            per_warp[static_cast<size_t>(g)] += work[i];
            prefix += work[i];
        }
        P.warp_begin[0] = 0;
        long long mx = *std::max_element(per_warp.begin(), per_warp.end());
        P.imbalance = static_cast<double>(mx) / (static_cast<double>(total) / n_warps);
    } else {
        std::fill(P.warp_begin.begin(), P.warp_begin.end(), 0);  // no items (m == 0)
    }
}

}  // namespace hhp

extern "C" hhp_status hhp_plan_stats(int m, int nnz, const int *rowptr, int n_warps, int cap, int *n_items,
                                     int *n_long_rows, int *n_chunks, int *max_item_nnz, double *imbalance) {
    if (m < 0 || nnz < 0 || !rowptr || n_warps <= 0 || cap < 32) {
        hhp::set_error("hhp_plan_stats: invalid arguments");
        return HHP_ERR_ARG;
    }
    if (rowptr[0] != 0 || rowptr[m] != nnz) {
        hhp::set_error("hhp_plan_stats: rowptr[0] must be 0 and rowptr[m] must equal nnz");
        return HHP_ERR_ARG;
    }
    hhp::PlanHost P;
    hhp::build_plan(m, rowptr, n_warps, cap, std::min(hhp::tuning().med, cap), P);
    if (n_items) *n_items = static_cast<int>(P.items.size());
    if (n_long_rows) *n_long_rows = static_cast<int>(P.long_rows.size());
    if (n_chunks) *n_chunks = static_cast<int>(P.chunk_long.size());
    if (max_item_nnz) *max_item_nnz = static_cast<int>(P.max_item_nnz);
    if (imbalance) *imbalance = P.imbalance;
    return HHP_OK;
}

extern "C" hhp_status hhp_plan_dump(int m, int nnz, const int *rowptr, int n_warps, int cap, int capacity,
                                    int *items_out, int *warp_begin_out, int *n_items) {
    if (m < 0 || nnz < 0 || !rowptr || n_warps <= 0 || cap < 32 || !n_items) {
        hhp::set_error("hhp_plan_dump: invalid arguments");
        return HHP_ERR_ARG;
    }
    if (rowptr[0] != 0 || rowptr[m] != nnz) {
        hhp::set_error("hhp_plan_dump: rowptr[0] must be 0 and rowptr[m] must equal nnz");
        return HHP_ERR_ARG;
    }
    hhp::PlanHost P;
    hhp::build_plan(m, rowptr, n_warps, cap, std::min(hhp::tuning().med, cap), P);
    *n_items = static_cast<int>(P.items.size());
    if (capacity < *n_items || !items_out || !warp_begin_out) {
        hhp::set_error("hhp_plan_dump: capacity %d < %d items", capacity, *n_items);
        return HHP_ERR_ARG;
    }
    for (size_t i = 0; i < P.items.size(); ++i) {
        items_out[4 * i] = P.items[i].x;
        items_out[4 * i + 1] = P.items[i].y;
        items_out[4 * i + 2] = P.items[i].z;
        items_out[4 * i + 3] = P.items[i].w;
    }
    for (size_t g = 0; g < P.warp_begin.size(); ++g) warp_begin_out[g] = P.warp_begin[g];
    return HHP_OK;
}
