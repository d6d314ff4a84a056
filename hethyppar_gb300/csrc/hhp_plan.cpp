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
#include <system_error>
#include <thread>

#include "hhp_internal.h"

namespace hhp {

namespace {

// fn(begin, end) over [0, n) split into contiguous ranges, one per host thread (serial for small
// n). Every range is processed exactly as the serial loop would process it, so the result does
// not depend on the thread count.
template <typename Fn>
void parallel_ranges(size_t n, size_t min_per_thread, Fn fn) {
    const size_t hw = std::max(1u, std::thread::hardware_concurrency());
    const size_t nt = std::min({hw, size_t{32}, std::max<size_t>(1, n / std::max<size_t>(min_per_thread, 1))});
    if (nt <= 1) {
        fn(size_t{0}, n);
        return;
    }
    std::vector<std::thread> pool;
    pool.reserve(nt - 1);
    const size_t step = (n + nt - 1) / nt;
    for (size_t t = 1; t < nt; ++t) {
        const size_t b = std::min(n, t * step), e = std::min(n, b + step);
        try {
            pool.emplace_back([=, &fn] { fn(b, e); });
        } catch (const std::system_error &) {
            fn(b, e);  // no thread to be had: this range runs here
        }
    }
    fn(size_t{0}, std::min(n, step));
    for (auto &th : pool) th.join();
}

}  // namespace

void build_plan(int m, const int *rowptr, int rpl, int long_thr, int cap, int window, SellHost &P) {
    P = SellHost();
    P.rpl = rpl;
    P.H = 32 * rpl;
    P.long_thr = long_thr;
    P.cap = cap;
    const int H = P.H;
    // rows up to long_thr go to slices in row order, longer ones to chunks: counted per range of
    // rows, then placed at each range's offset
    const size_t nr = static_cast<size_t>(m), kRange = 1 << 16;
    const size_t nrange = (nr + kRange - 1) / kRange;
    std::vector<size_t> n_short(nrange + 1, 0);
    std::vector<long long> nnz_short(nrange, 0);
    parallel_ranges(nrange, 4, [&](size_t gb, size_t ge) {
        for (size_t g = gb; g < ge; ++g) {
            size_t c = 0;
            long long z = 0;
            for (size_t r = g * kRange; r < std::min(nr, (g + 1) * kRange); ++r) {
                const int len = rowptr[r + 1] - rowptr[r];
                if (len <= long_thr) {
                    ++c;
                    z += len;
                }
            }
            n_short[g + 1] = c;
            nnz_short[g] = z;
        }
    });
    long long short_nnz = 0;
    for (size_t g = 0; g < nrange; ++g) {
        n_short[g + 1] += n_short[g];
        short_nnz += nnz_short[g];
    }
    std::vector<int> order(n_short[nrange]);
    parallel_ranges(nrange, 4, [&](size_t gb, size_t ge) {
        for (size_t g = gb; g < ge; ++g) {
            size_t o = n_short[g];
            for (size_t r = g * kRange; r < std::min(nr, (g + 1) * kRange); ++r)
                if (rowptr[r + 1] - rowptr[r] <= long_thr) order[o++] = static_cast<int>(r);
        }
    });
    int n_chunks = 0;
    if (order.size() < nr)
        for (int r = 0; r < m; ++r) {
            if (rowptr[r + 1] - rowptr[r] <= long_thr) continue;
            const int l = static_cast<int>(P.long_rows.size());
            P.long_rows.push_back(r);
            P.long_first.push_back(n_chunks);
            for (int a = rowptr[r]; a < rowptr[r + 1]; a += cap) {
                const int b = std::min(a + cap, rowptr[r + 1]);
                P.chunks.push_back(make_int4(r, n_chunks, a, b));
                P.chunk_long.push_back(l);
                ++n_chunks;
            }
        }
    P.long_first.push_back(n_chunks);
    // slice widths of an order (H rows per slice, the longest row sets the width), in parallel
    auto widths = [&](const std::vector<int> &ord, std::vector<int> &w) {
        const size_t ns = (ord.size() + static_cast<size_t>(H) - 1) / static_cast<size_t>(H);
        w.assign(ns, 0);
        parallel_ranges(ns, 2048, [&](size_t b, size_t e) {
            for (size_t s = b; s < e; ++s) {
                int mx = 0;
                const size_t q1 = std::min(ord.size(), (s + 1) * static_cast<size_t>(H));
                for (size_t q = s * static_cast<size_t>(H); q < q1; ++q)
                    mx = std::max(mx, rowptr[ord[q] + 1] - rowptr[ord[q]]);
                w[s] = mx;
            }
        });
    };
    std::vector<int> width;
    auto padded = [&](const std::vector<int> &ord) {
        widths(ord, width);
        long long tot = 0;
        for (int x : width) tot += static_cast<long long>(x) * H;
        return tot;
    };
    long long tot = padded(order);
    P.sorted = false;
    if (short_nnz > 0 && static_cast<double>(tot) > 1.15 * static_cast<double>(short_nnz)) {
        const size_t nwin = (order.size() + static_cast<size_t>(window) - 1) / static_cast<size_t>(window);
        parallel_ranges(nwin, 4, [&](size_t wb, size_t we) {
            for (size_t wi = wb; wi < we; ++wi) {
                const size_t w0 = wi * static_cast<size_t>(window);
                const auto b = order.begin() + static_cast<long>(w0);
                const auto e = order.begin() + static_cast<long>(std::min(order.size(), w0 + static_cast<size_t>(window)));
                std::stable_sort(b, e, [&](int x, int y) {
                    return (rowptr[x + 1] - rowptr[x]) > (rowptr[y + 1] - rowptr[y]);
                });
            }
        });
        tot = padded(order);
        P.sorted = true;
    }
    P.has_perm = P.sorted || !P.long_rows.empty();
    const size_t ms = order.size();
    P.n_slices = static_cast<int>((ms + static_cast<size_t>(H) - 1) / static_cast<size_t>(H));
    const size_t npos = static_cast<size_t>(P.n_slices) * static_cast<size_t>(H);
    P.pos_row.resize(npos);
    P.pos_len.resize(npos);
    P.slice_ptr.assign(static_cast<size_t>(P.n_slices) + 1, 0);
    // `width` holds the widths of the final order (padded() ran last on it)
    long long off = 0;
    for (int s = 0; s < P.n_slices; ++s) {
        P.slice_ptr[static_cast<size_t>(s)] = off;
        off += static_cast<long long>(width[static_cast<size_t>(s)]) * H;
    }
    parallel_ranges(npos, 65536, [&](size_t b, size_t e) {
        for (size_t p = b; p < e; ++p) {
            if (p < ms) {
                const int r = order[p];
                P.pos_row[p] = r;
                P.pos_len[p] = rowptr[r + 1] - rowptr[r];
            } else {
                P.pos_row[p] = -1;
                P.pos_len[p] = 0;
            }
        }
    });
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


// Uniform diagonals. A matrix whose entries all lie on at most max_k diagonals (offsets col - row;
// stencils: 5 or 7) needs no per-entry index in its slices: step k of every slice row holds the
// entry on diagonal doff[k] (zero where the row has none, marked absent in the row's bit mask),
// and the kernel forms the column as row + doff[k]. Accepted when every row's columns ascend
// (the steps then keep the CSR order of each row's sum), there are at most max_k distinct offsets,
// and padding all rows to all of them adds at most max_pad of the nonzeros. The distinct offsets
// are found per host thread and merged; a range that meets more than max_k stops at once.
bool uniform_diagonals(int m, const int *rowptr, const int *col, int max_k, double max_pad, int *doff, int &K,
                       std::vector<int> &mask) {
    K = 0;
    if (m <= 0 || max_k <= 0 || max_k > 31) return false;
    const long long nnz = rowptr[m];
    if (nnz <= 0) return false;
    const size_t n = static_cast<size_t>(m);
    const size_t hw = std::max(1u, std::thread::hardware_concurrency());
    const size_t nt = std::min({hw, size_t{32}, std::max<size_t>(1, n / 65536)});
    std::vector<std::vector<int>> sets(nt);
    std::vector<char> ok(nt, 1);
    const size_t step = (n + nt - 1) / nt;
    parallel_ranges(n, 65536, [&](size_t b, size_t e) {
        // parallel_ranges derives nt and step exactly as above and gives range t the rows
        // [t * step, (t + 1) * step): b / step is the range's own index, one set per range
        const size_t id = step ? b / step : 0;
        std::vector<int> &d = sets[std::min(id, nt - 1)];
        for (size_t i = b; i < e; ++i) {
            const int r = static_cast<int>(i);
            for (int p = rowptr[i]; p < rowptr[i + 1]; ++p) {
                if (p > rowptr[i] && col[p] <= col[p - 1]) {
                    ok[std::min(id, nt - 1)] = 0;
                    return;
                }
                const int o = col[p] - r;
                if (std::find(d.begin(), d.end(), o) == d.end()) {
                    if (static_cast<int>(d.size()) == max_k) {
                        ok[std::min(id, nt - 1)] = 0;
                        return;
                    }
                    d.push_back(o);
                }
            }
        }
    });
    std::vector<int> all;
    for (size_t t = 0; t < nt; ++t) {
        if (!ok[t]) return false;
        for (int o : sets[t])
            if (std::find(all.begin(), all.end(), o) == all.end()) all.push_back(o);
        if (static_cast<int>(all.size()) > max_k) return false;
    }
    std::sort(all.begin(), all.end());
    if (static_cast<double>(all.size()) * static_cast<double>(m) > (1.0 + max_pad) * static_cast<double>(nnz)) return false;
    K = static_cast<int>(all.size());
    std::copy(all.begin(), all.end(), doff);
    mask.assign(n, 0);
    parallel_ranges(n, 65536, [&](size_t b, size_t e) {
        for (size_t i = b; i < e; ++i) {
            int mk = 0;
            for (int p = rowptr[i]; p < rowptr[i + 1]; ++p) {
                const int o = col[p] - static_cast<int>(i);
                mk |= 1 << static_cast<int>(std::lower_bound(all.begin(), all.end(), o) - all.begin());
            }
            mask[i] = mk;
        }
    });
    return true;
}

}  // namespace hhp

extern "C" hhp_status hhp_plan_stats(int m, int nnz, const int *rowptr, int rows_per_lane, int cap, int *n_slices,
                                     int *n_long_rows, int *n_chunks, int *sorted, double *padding) {
    HHP_API_BEGIN
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
    HHP_API_END
}

extern "C" hhp_status hhp_plan_dump(int m, int nnz, const int *rowptr, int rows_per_lane, int cap, int capacity,
                                    int *slice_rows, int *chunks, int *n_slices, int *n_chunks) {
    HHP_API_BEGIN
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
    HHP_API_END
}
