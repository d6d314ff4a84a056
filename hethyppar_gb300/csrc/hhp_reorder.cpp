// hhp_reorder.cpp -- reverse Cuthill-McKee and multicolour orderings of a square CSR pattern, host
// side (the multicolour order, for ILU(0), is at the end of the file).
//
// The reference reorders rows by a partition vector (csr_permute, src/util/hhp_dp_helpers.c:18-37,
// grouped GPU-part first as src/entry/bicgstab_hybrid_dist_dp.c:221-233 does) that PaToH computed
// offline. This computes a locality ordering with no partitioner: the reverse Cuthill-McKee order
// of the symmetrised pattern A + A^T (diagonal ignored). Rows whose columns lie close together
// keep the SpMV's x gathers within a few cache lines and often let the slice layout store 16-bit
// column offsets. The result is a permutation in csr_permute's convention (row i of the reordered
// matrix is row perm[i] of A, column j becomes perm_inv[j]), as hhp_mat_from_csr's perm takes it.
//
// Algorithm (Cuthill & McKee 1969; pseudo-peripheral start nodes after Gibbs, Poole & Stockmeyer
// 1976 and George & Liu 1979), deterministic, every tie broken by the lower node number:
//  * components are taken in order of their lowest-numbered node;
//  * a component's start node: from its lowest-degree node r, build the BFS level structure; take
//    the lowest-degree node x of the last level; if x's level structure is deeper, r = x, repeat
//    (at most 8 rounds);
//  * Cuthill-McKee: breadth-first from the start node, each dequeued node enqueueing its
//    unvisited neighbours by increasing degree;
//  * the concatenated order is reversed.
// Degrees count distinct neighbours in A + A^T. O(nnz log(max degree)) time, O(nnz) memory.
#include <algorithm>
#include <cstring>
#include <vector>

#include "hhp_internal.h"

namespace hhp {

namespace {

struct Graph {
    std::vector<long long> ptr;  // m + 1
    std::vector<int> adj;        // distinct neighbours of each node, ascending
    int deg(int v) const { return static_cast<int>(ptr[static_cast<size_t>(v) + 1] - ptr[static_cast<size_t>(v)]); }
};

// A + A^T without the diagonal, duplicates merged.
Graph symmetrise(int m, const int *rowptr, const int *col) {
    Graph g;
    std::vector<long long> cnt(static_cast<size_t>(m) + 1, 0);
    for (int i = 0; i < m; ++i)
        for (int k = rowptr[i]; k < rowptr[i + 1]; ++k) {
            const int j = col[k];
            if (j == i) continue;
            ++cnt[static_cast<size_t>(i) + 1];
            ++cnt[static_cast<size_t>(j) + 1];
        }
    for (int i = 0; i < m; ++i) cnt[static_cast<size_t>(i) + 1] += cnt[static_cast<size_t>(i)];
    std::vector<int> raw(static_cast<size_t>(cnt[static_cast<size_t>(m)]));
    std::vector<long long> fill(cnt.begin(), cnt.end() - 1);
    for (int i = 0; i < m; ++i)
        for (int k = rowptr[i]; k < rowptr[i + 1]; ++k) {
            const int j = col[k];
            if (j == i) continue;
            raw[static_cast<size_t>(fill[static_cast<size_t>(i)]++)] = j;
            raw[static_cast<size_t>(fill[static_cast<size_t>(j)]++)] = i;
        }
    g.ptr.assign(static_cast<size_t>(m) + 1, 0);
    g.adj.reserve(raw.size());
    for (int i = 0; i < m; ++i) {
        auto b = raw.begin() + cnt[static_cast<size_t>(i)], e = raw.begin() + cnt[static_cast<size_t>(i) + 1];
        std::sort(b, e);
        e = std::unique(b, e);
        g.adj.insert(g.adj.end(), b, e);
        g.ptr[static_cast<size_t>(i) + 1] = static_cast<long long>(g.adj.size());
    }
    return g;
}

// Breadth-first level structure of the component containing `root` (nodes with mark == stamp are
// treated as visited). Returns the number of levels; `last` receives the nodes of the last level.
int levels(const Graph &g, int root, std::vector<int> &mark, int stamp, std::vector<int> &queue,
           std::vector<int> &last) {
    queue.clear();
    queue.push_back(root);
    mark[static_cast<size_t>(root)] = stamp;
    size_t head = 0;
    int depth = 0;
    while (head < queue.size()) {
        const size_t level_end = queue.size();
        last.assign(queue.begin() + static_cast<long>(head), queue.begin() + static_cast<long>(level_end));
        ++depth;
        for (; head < level_end; ++head) {
            const int u = queue[head];
            for (long long k = g.ptr[static_cast<size_t>(u)]; k < g.ptr[static_cast<size_t>(u) + 1]; ++k) {
                const int v = g.adj[static_cast<size_t>(k)];
                if (mark[static_cast<size_t>(v)] == stamp) continue;
                mark[static_cast<size_t>(v)] = stamp;
                queue.push_back(v);
            }
        }
    }
    return depth;
}

int lowest_degree(const Graph &g, const std::vector<int> &nodes) {
    int best = nodes.front();
    for (int v : nodes)
        if (g.deg(v) < g.deg(best) || (g.deg(v) == g.deg(best) && v < best)) best = v;
    return best;
}

}  // namespace

}  // namespace hhp

using namespace hhp;

namespace hhp {
namespace {
hhp_status check_square_csr(const char *who, int m, const int *rowptr, const int *col, const int *perm) {
    if (m < 0 || (m > 0 && (!rowptr || !perm)) || (m > 0 && rowptr[m] > 0 && !col)) {
        set_error("%s: null argument or negative size", who);
        return HHP_ERR_ARG;
    }
    if (m == 0) return HHP_OK;
    if (rowptr[0] != 0) {
        set_error("%s: rowptr[0] must be 0", who);
        return HHP_ERR_ARG;
    }
    for (int i = 0; i < m; ++i) {
        if (rowptr[i + 1] < rowptr[i]) {
            set_error("%s: rowptr decreases at row %d", who, i);
            return HHP_ERR_ARG;
        }
        for (int k = rowptr[i]; k < rowptr[i + 1]; ++k)
            if (col[k] < 0 || col[k] >= m) {
                set_error("%s: column %d of row %d outside [0, %d)", who, col[k], i, m);
                return HHP_ERR_ARG;
            }
    }
    return HHP_OK;
}
}  // namespace
}  // namespace hhp

hhp_status hhp_reorder_rcm(int m, const int *rowptr, const int *col, int *perm) {
    HHP_API_BEGIN
    HHP_TRY(check_square_csr("reorder_rcm", m, rowptr, col, perm));
    if (m == 0) return HHP_OK;
    const Graph g = symmetrise(m, rowptr, col);
    std::vector<int> order;
    order.reserve(static_cast<size_t>(m));
    std::vector<char> placed(static_cast<size_t>(m), 0);
    std::vector<int> mark(static_cast<size_t>(m), 0), queue, last, nbr;
    queue.reserve(static_cast<size_t>(m));
    int stamp = 0;
    for (int seed = 0; seed < m; ++seed) {
        if (placed[static_cast<size_t>(seed)]) continue;
        // the component's nodes, then its lowest-degree node
        levels(g, seed, mark, ++stamp, queue, last);
        int r = lowest_degree(g, queue);
        int depth = levels(g, r, mark, ++stamp, queue, last);
        for (int round = 0; round < 8; ++round) {
            const int x = lowest_degree(g, last);
            std::vector<int> last_x;
            const int dx = levels(g, x, mark, ++stamp, queue, last_x);
            if (dx <= depth) break;
            r = x;
            depth = dx;
            last.swap(last_x);
        }
        // Cuthill-McKee from r
        const size_t first = order.size();
        order.push_back(r);
        placed[static_cast<size_t>(r)] = 1;
        for (size_t head = first; head < order.size(); ++head) {
            const int u = order[head];
            nbr.clear();
            for (long long k = g.ptr[static_cast<size_t>(u)]; k < g.ptr[static_cast<size_t>(u) + 1]; ++k) {
                const int v = g.adj[static_cast<size_t>(k)];
                if (!placed[static_cast<size_t>(v)]) {
                    placed[static_cast<size_t>(v)] = 1;
                    nbr.push_back(v);
                }
            }
            std::sort(nbr.begin(), nbr.end(), [&](int a, int b) {
                return g.deg(a) != g.deg(b) ? g.deg(a) < g.deg(b) : a < b;
            });
            order.insert(order.end(), nbr.begin(), nbr.end());
        }
    }
    for (int i = 0; i < m; ++i) perm[i] = order[static_cast<size_t>(m - 1 - i)];
    return HHP_OK;
    HHP_API_END
}

// Greedy multicolouring (the first-fit colouring of graph-colouring practice, in natural node
// order) of A + A^T: rows of one colour share no entry, so in the reordered matrix the rows of a
// colour depend only on rows of earlier colours and the triangles of ILU(0) have at most as many
// dependency levels as there are colours.
hhp_status hhp_reorder_color(int m, const int *rowptr, const int *col, int *perm, int *n_colors) {
    HHP_API_BEGIN
    HHP_TRY(check_square_csr("reorder_color", m, rowptr, col, perm));
    if (n_colors) *n_colors = 0;
    if (m == 0) return HHP_OK;
    const Graph g = symmetrise(m, rowptr, col);
    std::vector<int> color(static_cast<size_t>(m), -1), taken;
    int nc = 0;
    for (int v = 0; v < m; ++v) {
        // taken[c] == v: a neighbour coloured before v has colour c
        for (long long k = g.ptr[static_cast<size_t>(v)]; k < g.ptr[static_cast<size_t>(v) + 1]; ++k) {
            const int c = color[static_cast<size_t>(g.adj[static_cast<size_t>(k)])];
            if (c >= 0) taken[static_cast<size_t>(c)] = v;
        }
        int c = 0;
        while (c < nc && taken[static_cast<size_t>(c)] == v) ++c;
        if (c == nc) {
            ++nc;
            taken.push_back(-1);
        }
        color[static_cast<size_t>(v)] = c;
    }
    std::vector<int> start(static_cast<size_t>(nc) + 1, 0);
    for (int v = 0; v < m; ++v) ++start[static_cast<size_t>(color[static_cast<size_t>(v)]) + 1];
    for (int c = 0; c < nc; ++c) start[static_cast<size_t>(c) + 1] += start[static_cast<size_t>(c)];
    for (int v = 0; v < m; ++v) perm[start[static_cast<size_t>(color[static_cast<size_t>(v)])]++] = v;
    if (n_colors) *n_colors = nc;
    return HHP_OK;
    HHP_API_END
}
