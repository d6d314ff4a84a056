// hhp_plan.cpp -- host-side construction of the SpMV work plan: row-length binning into a sliced,
// row-interleaved device layout plus equal-nnz chunks for long rows.
//
// Rows are binned by length:
//   len <= long_thr  -> "slice rows": placed in slices of H = 32*RPL rows (RPL rows per lane).
//                       Inside a slice the j-th nonzero of all H rows are stored next to each
//                       other (step-major), so at every step a warp loads its lanes' values and
//                       column indices with one coalesced vector load per lane; each lane sums
//                       its rows sequentially in CSR order (the order of CSR_spmxv_seq,
//                       src/util/hhp_cpu.c:445-455), one fused multiply-add per nonzero.
//                       Rows keep their natural order unless that would pad the slices by more
//                       than 15%; then rows are sorted by length (descending, stable) inside
//                       windows of `window` rows, so slice-mates have similar lengths.
//   len >  long_thr  -> CHUNK items of at most `cap` nonzeros (equal-nnz slices of the row, as a
//                       merge-path split would cut it), each summed by one warp, the chunk sums
//                       combined in chunk order by whichever warp finishes the row's last chunk.
#include <algorithm>
#include <cmath>
#include <numeric>
#include <queue>

#include "hhp_internal.h"

namespace hhp {

void build_plan(int m, const int *rowptr, int rpl, int long_thr, int cap, int window, SellHost &P) {
    P = SellHost();
    P.rpl = rpl;
    P.H = 32 * rpl;
    P.long_thr = long_thr;
    P.cap = cap;
    const int H = P.H;
    std::vector<int> order;
    order.reserve(static_cast<size_t>(m));
    long long short_nnz = 0;
    int n_chunks = 0;
    for (int r = 0; r < m; ++r) {
        const int len = rowptr[r + 1] - rowptr[r];
        if (len > long_thr) {
            const int l = static_cast<int>(P.long_rows.size());
            P.long_rows.push_back(r);
            P.long_first.push_back(n_chunks);
            for (int a = rowptr[r]; a < rowptr[r + 1]; a += cap) {
                const int b = std::min(a + cap, rowptr[r + 1]);
                P.chunks.push_back(make_int4(r, n_chunks, a, b));
                P.chunk_long.push_back(l);
                ++n_chunks;
            }
        } else {
            order.push_back(r);
            short_nnz += len;
        }
    }
    P.long_first.push_back(n_chunks);
    auto padded = [&](const std::vector<int> &ord) {
        long long tot = 0;
        for (size_t s0 = 0; s0 < ord.size(); s0 += static_cast<size_t>(H)) {
            int mx = 0;
            for (size_t q = s0; q < std::min(ord.size(), s0 + static_cast<size_t>(H)); ++q)
                mx = std::max(mx, rowptr[ord[q] + 1] - rowptr[ord[q]]);
            tot += static_cast<long long>(mx) * H;
        }
        return tot;
    };
    long long tot = padded(order);
    P.sorted = false;
    if (short_nnz > 0 && static_cast<double>(tot) > 1.15 * static_cast<double>(short_nnz)) {
        for (size_t w0 = 0; w0 < order.size(); w0 += static_cast<size_t>(window)) {
            const auto b = order.begin() + static_cast<long>(w0);
            const auto e = order.begin() + static_cast<long>(std::min(order.size(), w0 + static_cast<size_t>(window)));
            std::stable_sort(b, e, [&](int x, int y) {
                return (rowptr[x + 1] - rowptr[x]) > (rowptr[y + 1] - rowptr[y]);
            });
        }
        tot = padded(order);
        P.sorted = true;
    }
    P.has_perm = P.sorted || !P.long_rows.empty();
    const size_t ms = order.size();
    P.n_slices = static_cast<int>((ms + static_cast<size_t>(H) - 1) / static_cast<size_t>(H));
    const size_t npos = static_cast<size_t>(P.n_slices) * static_cast<size_t>(H);
    P.pos_row.assign(npos, -1);
    P.pos_len.assign(npos, 0);
    P.slice_ptr.assign(static_cast<size_t>(P.n_slices) + 1, 0);
    long long off = 0;
    for (int s = 0; s < P.n_slices; ++s) {
        int mx = 0;
        for (int q = 0; q < H; ++q) {
            const size_t p = static_cast<size_t>(s) * H + static_cast<size_t>(q);
            if (p < ms) {
                const int r = order[p];
                P.pos_row[p] = r;
                P.pos_len[p] = rowptr[r + 1] - rowptr[r];
                mx = std::max(mx, P.pos_len[p]);
            }
        }
        P.slice_ptr[static_cast<size_t>(s)] = off;
        off += static_cast<long long>(mx) * H;
    }
    P.slice_ptr[static_cast<size_t>(P.n_slices)] = off;
    P.total = off;
    P.short_nnz = short_nnz;
    P.padding = short_nnz > 0 ? static_cast<double>(off) / static_cast<double>(short_nnz) : 1.0;
}

void assign_units(const SellHost &P, int n_warps, std::vector<int> &warp_ptr, std::vector<int> &warp_units,
                  double *imbalance) {
    // cost of a unit ~ the steps its warp walks: a slice's longest row, a chunk's nonzeros / 32,
    // plus a fixed cost for loading lengths and writing results
    const int ns = P.n_slices, nc = static_cast<int>(P.chunks.size()), nu = ns + nc;
    std::vector<long long> cost(static_cast<size_t>(nu));
    for (int s = 0; s < ns; ++s) {
        const long long steps = (P.slice_ptr[static_cast<size_t>(s) + 1] - P.slice_ptr[static_cast<size_t>(s)]) / P.H;
        cost[static_cast<size_t>(s)] = steps + 4;
    }
    for (int c = 0; c < nc; ++c) {
        const int4 d = P.chunks[static_cast<size_t>(c)];
        cost[static_cast<size_t>(ns + c)] = (d.w - d.z + 31) / 32 + 8;
    }
    // longest processing time first: each unit, largest first (ties by id), goes to the least
    // loaded warp (ties by warp id); deterministic, and for equal costs it deals round-robin
    std::vector<int> order(static_cast<size_t>(nu));
    std::iota(order.begin(), order.end(), 0);
    std::stable_sort(order.begin(), order.end(), [&](int a, int b) { return cost[static_cast<size_t>(a)] > cost[static_cast<size_t>(b)]; });
    using Load = std::pair<long long, int>;
    std::priority_queue<Load, std::vector<Load>, std::greater<Load>> heap;
    for (int w = 0; w < n_warps; ++w) heap.push({0LL, w});
    std::vector<int> owner(static_cast<size_t>(nu));
    std::vector<long long> load(static_cast<size_t>(n_warps), 0);
    for (int u : order) {
        Load l = heap.top();
        heap.pop();
        owner[static_cast<size_t>(u)] = l.second;
        l.first += cost[static_cast<size_t>(u)];
        load[static_cast<size_t>(l.second)] = l.first;
        heap.push(l);
    }
    warp_ptr.assign(static_cast<size_t>(n_warps) + 1, 0);
    for (int u = 0; u < nu; ++u) warp_ptr[static_cast<size_t>(owner[static_cast<size_t>(u)]) + 1]++;
    for (int w = 0; w < n_warps; ++w) warp_ptr[static_cast<size_t>(w) + 1] += warp_ptr[static_cast<size_t>(w)];
    warp_units.assign(static_cast<size_t>(nu), 0);
    std::vector<int> fill(warp_ptr.begin(), warp_ptr.end() - 1);
    for (int u = 0; u < nu; ++u) {  // ascending unit id within each warp
        const int w = owner[static_cast<size_t>(u)];
        warp_units[static_cast<size_t>(fill[static_cast<size_t>(w)]++)] = u;
    }
    if (imbalance) {
        long long tot = 0, mx = 0;
        for (long long v : load) {
            tot += v;
            mx = std::max(mx, v);
        }
        *imbalance = tot > 0 ? static_cast<double>(mx) * n_warps / static_cast<double>(tot) : 1.0;
    }
}

namespace {
bool rows_ascending(int m, const int *rowptr) {
    for (int i = 0; i < m; ++i)
        if (rowptr[i + 1] < rowptr[i]) return false;
    return true;
}
}  // namespace

}  // namespace hhp

extern "C" hhp_status hhp_plan_stats(int m, int nnz, const int *rowptr, int rows_per_lane, int cap, int *n_slices,
                                     int *n_long_rows, int *n_chunks, int *sorted, double *padding) {
    if (m < 0 || nnz < 0 || !rowptr || (rows_per_lane != 1 && rows_per_lane != 2 && rows_per_lane != 4) ||
        cap < 32) {
        hhp::set_error("hhp_plan_stats: invalid arguments");
        return HHP_ERR_ARG;
    }
    if (rowptr[0] != 0 || rowptr[m] != nnz || !hhp::rows_ascending(m, rowptr)) {
        hhp::set_error("hhp_plan_stats: rowptr must rise from 0 to nnz");
        return HHP_ERR_ARG;
    }
    hhp::SellHost P;
    const hhp::Tuning &t = hhp::tuning();
    hhp::build_plan(m, rowptr, rows_per_lane, t.long_thr, cap, t.window, P);
    if (n_slices) *n_slices = P.n_slices;
    if (n_long_rows) *n_long_rows = static_cast<int>(P.long_rows.size());
    if (n_chunks) *n_chunks = static_cast<int>(P.chunks.size());
    if (sorted) *sorted = P.sorted ? 1 : 0;
    if (padding) *padding = P.padding;
    return HHP_OK;
}

extern "C" hhp_status hhp_plan_dump(int m, int nnz, const int *rowptr, int rows_per_lane, int cap, int capacity,
                                    int *slice_rows, int *chunks, int *n_slices, int *n_chunks) {
    if (m < 0 || nnz < 0 || !rowptr || (rows_per_lane != 1 && rows_per_lane != 2 && rows_per_lane != 4) ||
        cap < 32 || !n_slices || !n_chunks) {
        hhp::set_error("hhp_plan_dump: invalid arguments");
        return HHP_ERR_ARG;
    }
    if (rowptr[0] != 0 || rowptr[m] != nnz || !hhp::rows_ascending(m, rowptr)) {
        hhp::set_error("hhp_plan_dump: rowptr must rise from 0 to nnz");
        return HHP_ERR_ARG;
    }
    hhp::SellHost P;
    const hhp::Tuning &t = hhp::tuning();
    hhp::build_plan(m, rowptr, rows_per_lane, t.long_thr, cap, t.window, P);
    *n_slices = P.n_slices;
    *n_chunks = static_cast<int>(P.chunks.size());
    const long long need = static_cast<long long>(P.pos_row.size()) + 4LL * static_cast<long long>(P.chunks.size());
    if (capacity < need || !slice_rows || !chunks) {
        hhp::set_error("hhp_plan_dump: capacity %d < %lld", capacity, need);
        return HHP_ERR_ARG;
    }
    std::copy(P.pos_row.begin(), P.pos_row.end(), slice_rows);
    for (size_t c = 0; c < P.chunks.size(); ++c) {
        chunks[4 * c] = P.chunks[c].x;
        chunks[4 * c + 1] = P.chunks[c].y;
        chunks[4 * c + 2] = P.chunks[c].z;
        chunks[4 * c + 3] = P.chunks[c].w;
    }
    return HHP_OK;
}
