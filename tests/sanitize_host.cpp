// sanitize_host.cpp -- drives the library's host-only code (Matrix Market and binary CSR reader,
// vector files, SpMV work plan and its uniform-diagonal check, reverse Cuthill-McKee, multicolour
// order) with ordinary, malformed and large inputs.
// tests/test_sanitize_cpu.py compiles it with hhp_io.cpp, hhp_plan.cpp and hhp_reorder.cpp under
// AddressSanitizer + UndefinedBehaviorSanitizer, and again under ThreadSanitizer for the parallel
// reader; any report, leak or failed check ends the run with a nonzero status. No CUDA call is
// made. Usage: sanitize_host <scratch dir>
#include <cstdarg>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <random>
#include <string>
#include <vector>

#include "hhp_gpu.h"
#include "hhp_internal.h"

// The three definitions the library's hhp_api.cu provides for these sources.
namespace hhp {
namespace {
thread_local char g_err[512];
}
void set_error(const char *fmt, ...) {
    va_list ap;
    va_start(ap, fmt);
    std::vsnprintf(g_err, sizeof g_err, fmt, ap);
    va_end(ap);
}
int env_int(const char *, int dflt) { return dflt; }
const Tuning &tuning() {
    static const Tuning t;
    return t;
}
}  // namespace hhp

namespace {

int g_fail = 0;
#define CHECK(cond)                                                                  \
    do {                                                                             \
        if (!(cond)) {                                                               \
            std::fprintf(stderr, "check failed at line %d: %s\n", __LINE__, #cond);  \
            ++g_fail;                                                                \
        }                                                                            \
    } while (0)

std::string g_dir;

std::string write_file(const char *name, const std::string &text) {
    const std::string p = g_dir + "/" + name;
    FILE *f = std::fopen(p.c_str(), "wb");
    if (!f) {
        std::fprintf(stderr, "cannot write %s\n", p.c_str());
        std::exit(2);
    }
    std::fwrite(text.data(), 1, text.size(), f);
    std::fclose(f);
    return p;
}

struct Csr {
    int m = 0, n = 0, nnz = 0;
    int *rowptr = nullptr, *col = nullptr;
    double *val = nullptr;
    ~Csr() {
        hhp_free(rowptr);
        hhp_free(col);
        hhp_free(val);
    }
};

hhp_status read(const std::string &p, Csr &c) {
    return hhp_mtx_read(p.c_str(), &c.m, &c.n, &c.nnz, &c.rowptr, &c.col, &c.val);
}

bool well_formed(const Csr &c) {
    if (c.rowptr[0] != 0 || c.rowptr[c.m] != c.nnz) return false;
    for (int i = 0; i < c.m; ++i)
        if (c.rowptr[i + 1] < c.rowptr[i]) return false;
    for (int k = 0; k < c.nnz; ++k)
        if (c.col[k] < 0 || c.col[k] >= c.n) return false;
    return true;
}

void small_matrix_market() {
    // unsorted entries, a duplicate, comments, an integer field
    const std::string ok = write_file("ok.mtx",
                                      "%%MatrixMarket matrix coordinate real general\n% c\n3 4 5\n"
                                      "3 1 1.5\n1 4 -2\n2 2 3e0\n1 1 4\n1 4 5\n");
    {
        Csr c;
        CHECK(read(ok, c) == HHP_OK);
        CHECK(c.m == 3 && c.n == 4 && c.nnz == 5 && well_formed(c));
        // rows ordered, file order kept within a row: row 0 = (3, -2), (0, 4), (3, 5)
        CHECK(c.rowptr[1] == 3 && c.col[0] == 3 && c.col[1] == 0 && c.col[2] == 3 && c.val[2] == 5.0);
    }
    const char *bad[] = {
        "%%MatrixMarket matrix coordinate real symmetric\n2 2 1\n1 1 1.0\n",
        "%%MatrixMarket matrix coordinate pattern general\n2 2 1\n1 1\n",
        "%%MatrixMarket matrix coordinate complex general\n2 2 1\n1 1 1 0\n",
        "2 2 1\n1 1 1.0\n",
        "%%MatrixMarket matrix coordinate real general\n2 2 2\n1 1 1.0\n",
        "%%MatrixMarket matrix coordinate real general\n2 2 1\n1 3 1.0\n",
        "%%MatrixMarket matrix coordinate real general\n2 2 1\n0 1 1.0\n",
        "%%MatrixMarket matrix coordinate real general\n2147483647 2147483647 1\n1 1 1.0\n",
        "%%MatrixMarket matrix coordinate real general\n-1 2 0\n",
        "%%MatrixMarket matrix coordinate real general\n2 2 1\n1 1 x\n",
        "%%MatrixMarket matrix coordinate real general\n",
        "",
    };
    for (const char *t : bad) {
        Csr c;
        const hhp_status s = read(write_file("bad.mtx", t), c);
        CHECK(s != HHP_OK);
        CHECK(c.rowptr == nullptr && c.col == nullptr && c.val == nullptr);
    }
    Csr c;
    CHECK(read(g_dir + "/does-not-exist.mtx", c) == HHP_ERR_IO);
    CHECK(hhp_mtx_read(nullptr, &c.m, &c.n, &c.nnz, &c.rowptr, &c.col, &c.val) != HHP_OK);
    CHECK(hhp_mtx_read(ok.c_str(), nullptr, &c.n, &c.nnz, &c.rowptr, &c.col, &c.val) == HHP_ERR_ARG);
}

// A file above the reader's parallel threshold, rows in random order, checked against a serial
// stable counting sort of the same entries.
void large_matrix_market() {
    const int m = 70000, n = 50000, nz = 600000;
    std::mt19937 rng(7);
    std::vector<int> ri(nz), ci(nz);
    std::vector<double> vi(nz);
    std::string text = "%%MatrixMarket matrix coordinate real general\n%% large\n";
    text += std::to_string(m) + " " + std::to_string(n) + " " + std::to_string(nz) + "\n";
    char line[96];
    for (int k = 0; k < nz; ++k) {
        ri[k] = static_cast<int>(rng() % m);
        ci[k] = static_cast<int>(rng() % n);
        vi[k] = static_cast<double>(static_cast<int>(rng() % 2000001) - 1000000) / 1024.0;
        std::snprintf(line, sizeof line, "%d %d %.17g\n", ri[k] + 1, ci[k] + 1, vi[k]);
        text += line;
    }
    const std::string p = write_file("large.mtx", text);
    std::vector<int> rp(m + 1, 0);
    for (int k = 0; k < nz; ++k) ++rp[ri[k] + 1];
    for (int i = 0; i < m; ++i) rp[i + 1] += rp[i];
    std::vector<int> fill(rp.begin(), rp.end() - 1), ec(nz);
    std::vector<double> ev(nz);
    for (int k = 0; k < nz; ++k) {
        const int d = fill[ri[k]]++;
        ec[d] = ci[k];
        ev[d] = vi[k];
    }
    {
        Csr c;
        CHECK(read(p, c) == HHP_OK);
        CHECK(c.m == m && c.n == n && c.nnz == nz && well_formed(c));
        bool same = true;
        for (int i = 0; i <= m && same; ++i) same = c.rowptr[i] == rp[i];
        for (int k = 0; k < nz && same; ++k) same = c.col[k] == ec[k] && c.val[k] == ev[k];
        CHECK(same);
        // the binary CSR file reads back to the same arrays
        const std::string b = g_dir + "/large.csr";
        CHECK(hhp_csr_file_write(b.c_str(), c.m, c.n, c.nnz, c.rowptr, c.col, c.val) == HHP_OK);
        Csr d;
        CHECK(read(b, d) == HHP_OK);
        CHECK(d.m == m && d.n == n && d.nnz == nz);
        same = true;
        for (int i = 0; i <= m && same; ++i) same = d.rowptr[i] == c.rowptr[i];
        for (int k = 0; k < nz && same; ++k) same = d.col[k] == c.col[k] && d.val[k] == c.val[k];
        CHECK(same);
        // truncated and corrupted binary files are errors
        FILE *f = std::fopen(b.c_str(), "rb");
        std::string raw;
        if (f) {
            char buf[1 << 16];
            size_t got;
            while ((got = std::fread(buf, 1, sizeof buf, f)) > 0) raw.append(buf, got);
            std::fclose(f);
        }
        Csr e;
        CHECK(read(write_file("trunc.csr", raw.substr(0, raw.size() - 8)), e) != HHP_OK);
        std::string bad = raw;
        const size_t col0 = 8 + 3 * 8 + 4 * (static_cast<size_t>(m) + 1);
        bad[col0] = '\x7f';
        bad[col0 + 3] = '\x7f';
        Csr g;
        CHECK(read(write_file("corrupt.csr", bad), g) != HHP_OK);
    }
    // a malformed entry deep inside the file, and a short file, are errors
    std::string broken = text;
    const size_t ls = broken.find('\n', broken.size() / 2) + 1, le = broken.find('\n', ls);
    broken.replace(ls, le - ls, "1 x 2.0");
    Csr c1;
    CHECK(read(write_file("broken.mtx", broken), c1) == HHP_ERR_FORMAT);
    Csr c2;
    CHECK(read(write_file("short.mtx", text.substr(0, text.size() / 3)), c2) == HHP_ERR_FORMAT);
}

void vector_files() {
    const double v[5] = {1.0, -2.5, 1.0 / 3.0, 1e-300, 12345.678901234567};
    const std::string p = g_dir + "/v.txt";
    CHECK(hhp_vector_write(p.c_str(), 5, v, 1) == HHP_OK);
    double r[6] = {0, 0, 0, 0, 0, 0};
    CHECK(hhp_vector_read(p.c_str(), 5, r) == HHP_OK);
    CHECK(std::memcmp(r, v, sizeof v) == 0);
    CHECK(hhp_vector_read(p.c_str(), 6, r) == HHP_ERR_IO);
    CHECK(hhp_vector_write(p.c_str(), 5, v, 0) == HHP_OK);
    CHECK(hhp_vector_read(p.c_str(), 5, r) == HHP_OK && r[2] == 0.333333);
    CHECK(hhp_vector_read((g_dir + "/none.txt").c_str(), 1, r) == HHP_ERR_IO);
    CHECK(hhp_vector_read(p.c_str(), 1, nullptr) == HHP_ERR_ARG);
}

std::vector<int> rowptr_of(const std::vector<int> &lens) {
    std::vector<int> rp(lens.size() + 1, 0);
    for (size_t i = 0; i < lens.size(); ++i) rp[i + 1] = rp[i] + lens[i];
    return rp;
}

void work_plan() {
    std::mt19937 rng(3);
    std::vector<std::vector<int>> cases;
    cases.push_back({});                          // no rows
    cases.push_back({0, 0, 0});                   // empty rows only
    cases.push_back(std::vector<int>(1000, 17));  // uniform
    {
        std::vector<int> l(20000);
        for (auto &x : l) x = static_cast<int>(rng() % 3 == 0 ? rng() % 600 : rng() % 9);
        l[5] = 70000;  // one very long row
        cases.push_back(l);
    }
    {
        // large enough for the plan builder's threaded passes (row classification, length-sorted
        // windows, slice widths and positions)
        std::vector<int> l(1200000);
        for (auto &x : l) x = static_cast<int>(rng() % 5 == 0 ? rng() % 300 : 1 + rng() % 6);
        for (int i = 0; i < 40; ++i) l[static_cast<size_t>(i) * 29989] = 3000 + i;
        cases.push_back(l);
    }
    for (const auto &lens : cases) {
        const std::vector<int> rp = rowptr_of(lens);
        const int m = static_cast<int>(lens.size()), nnz = rp.back();
        for (int rpl : {1, 2, 4})
            for (int cap : {32, 2048}) {
                int ns = -1, nl = -1, nc = -1, so = -1;
                double pad = 0.0;
                CHECK(hhp_plan_stats(m, nnz, rp.data(), rpl, cap, &ns, &nl, &nc, &so, &pad) == HHP_OK);
                int ns2 = -1, nc2 = -1;
                CHECK(hhp_plan_dump(m, nnz, rp.data(), rpl, cap, 0, nullptr, nullptr, &ns2, &nc2) != HHP_OK);
                CHECK(ns2 == ns && nc2 == nc);
                const size_t pos = static_cast<size_t>(ns) * 32 * rpl;
                std::vector<int> rows(pos + 1), chunks(4 * static_cast<size_t>(nc) + 1);
                CHECK(hhp_plan_dump(m, nnz, rp.data(), rpl, cap, static_cast<int>(pos + 4 * nc), rows.data(),
                                    chunks.data(), &ns2, &nc2) == HHP_OK);
                std::vector<int> seen(static_cast<size_t>(m), 0);
                for (size_t q = 0; q < pos; ++q)
                    if (rows[q] >= 0) ++seen[static_cast<size_t>(rows[q])];
                int prev = -1;
                for (int k = 0; k < nc; ++k) {
                    const int r = chunks[4 * k];
                    CHECK(chunks[4 * k + 2] < chunks[4 * k + 3] && chunks[4 * k + 3] - chunks[4 * k + 2] <= cap);
                    if (r != prev) ++seen[static_cast<size_t>(r)];
                    prev = r;
                }
                for (int i = 0; i < m; ++i) CHECK(seen[static_cast<size_t>(i)] == 1);
            }
    }
    int ns, nl, nc, so;
    double pad;
    const int bad_rp[3] = {0, 2, 1};
    CHECK(hhp_plan_stats(2, 1, bad_rp, 2, 2048, &ns, &nl, &nc, &so, &pad) != HHP_OK);
    CHECK(hhp_plan_stats(2, 1, bad_rp, 3, 2048, &ns, &nl, &nc, &so, &pad) == HHP_ERR_ARG);
}

void rcm() {
    std::mt19937 rng(5);
    for (int m : {0, 1, 2, 37, 5000}) {
        std::vector<int> lens(static_cast<size_t>(m));
        for (auto &x : lens) x = static_cast<int>(rng() % 6);
        const std::vector<int> rp = rowptr_of(lens);
        std::vector<int> col(static_cast<size_t>(rp.back()) + 1);
        for (int k = 0; k < rp.back(); ++k) col[static_cast<size_t>(k)] = static_cast<int>(rng() % static_cast<unsigned>(m));
        std::vector<int> perm(static_cast<size_t>(m) + 1, -1);
        CHECK(hhp_reorder_rcm(m, rp.data(), col.data(), perm.data()) == HHP_OK);
        std::vector<int> seen(static_cast<size_t>(m), 0);
        for (int i = 0; i < m; ++i)
            if (perm[static_cast<size_t>(i)] >= 0 && perm[static_cast<size_t>(i)] < m) ++seen[static_cast<size_t>(perm[static_cast<size_t>(i)])];
        for (int i = 0; i < m; ++i) CHECK(seen[static_cast<size_t>(i)] == 1);
    }
    const int rp[3] = {0, 1, 2}, col[2] = {0, 5};
    int perm[2];
    CHECK(hhp_reorder_rcm(2, rp, col, perm) == HHP_ERR_ARG);
    CHECK(hhp_reorder_rcm(-1, rp, col, perm) == HHP_ERR_ARG);
}

// 5-point stencil of an nx x nx grid, columns ascending in every row.
void stencil5(int nx, std::vector<int> &rp, std::vector<int> &col) {
    const int m = nx * nx;
    rp.assign(1, 0);
    col.clear();
    for (int i = 0; i < m; ++i) {
        const int x = i % nx, y = i / nx;
        if (y > 0) col.push_back(i - nx);
        if (x > 0) col.push_back(i - 1);
        col.push_back(i);
        if (x + 1 < nx) col.push_back(i + 1);
        if (y + 1 < nx) col.push_back(i + nx);
        rp.push_back(static_cast<int>(col.size()));
    }
}

void uniform() {
    int doff[hhp::kMaxDiag] = {};
    int K = -1;
    std::vector<int> mask, rp, col;
    // 160,000 rows: the threaded pass (one offset set per range) runs with several ranges
    stencil5(400, rp, col);
    const int m = static_cast<int>(rp.size()) - 1;
    CHECK(hhp::uniform_diagonals(m, rp.data(), col.data(), hhp::kMaxDiag, 0.10, doff, K, mask));
    CHECK(K == 5 && doff[0] == -400 && doff[1] == -1 && doff[2] == 0 && doff[3] == 1 && doff[4] == 400);
    CHECK(mask.size() == static_cast<size_t>(m));
    for (int i = 0; i < m && K == 5; ++i) {
        int want = 0;
        for (int p = rp[static_cast<size_t>(i)]; p < rp[static_cast<size_t>(i) + 1]; ++p)
            for (int k = 0; k < K; ++k)
                if (col[static_cast<size_t>(p)] - i == doff[k]) want |= 1 << k;
        CHECK(mask[static_cast<size_t>(i)] == want);
    }
    // refusals: a row whose columns do not ascend, more offsets than allowed, too much padding,
    // no rows
    std::vector<int> c2 = col;
    std::swap(c2[100], c2[101]);
    CHECK(!hhp::uniform_diagonals(m, rp.data(), c2.data(), hhp::kMaxDiag, 0.10, doff, K, mask));
    CHECK(!hhp::uniform_diagonals(m, rp.data(), col.data(), 4, 0.10, doff, K, mask));
    {
        // every row has its diagonal, one row in 50 also an entry 7 to the right: 2 offsets for
        // 1.02 entries per row pads by ~96 %
        std::vector<int> r3(1, 0), c3;
        for (int i = 0; i < 200000; ++i) {
            c3.push_back(i);
            if (i % 50 == 0 && i + 7 < 200000) c3.push_back(i + 7);
            r3.push_back(static_cast<int>(c3.size()));
        }
        CHECK(!hhp::uniform_diagonals(200000, r3.data(), c3.data(), hhp::kMaxDiag, 0.10, doff, K, mask));
        CHECK(hhp::uniform_diagonals(200000, r3.data(), c3.data(), hhp::kMaxDiag, 1.0, doff, K, mask));
        CHECK(K == 2 && doff[0] == 0 && doff[1] == 7);
    }
    CHECK(!hhp::uniform_diagonals(0, rp.data(), col.data(), hhp::kMaxDiag, 0.10, doff, K, mask));
}

void color() {
    std::mt19937 rng(9);
    std::vector<int> rp, col;
    stencil5(300, rp, col);
    const int m = static_cast<int>(rp.size()) - 1;
    std::vector<int> perm(static_cast<size_t>(m), -1);
    int nc = -1;
    CHECK(hhp_reorder_color(m, rp.data(), col.data(), perm.data(), &nc) == HHP_OK);
    CHECK(nc == 2);  // the 5-point stencil is bipartite: red-black
    for (int m2 : {0, 1, 37, 20000}) {
        std::vector<int> lens(static_cast<size_t>(m2));
        for (auto &x : lens) x = static_cast<int>(rng() % 7);
        const std::vector<int> r2 = rowptr_of(lens);
        std::vector<int> c2(static_cast<size_t>(r2.back()) + 1);
        for (int k = 0; k < r2.back(); ++k) c2[static_cast<size_t>(k)] = static_cast<int>(rng() % static_cast<unsigned>(m2));
        std::vector<int> p2(static_cast<size_t>(m2) + 1, -1);
        int n2 = -1;
        CHECK(hhp_reorder_color(m2, r2.data(), c2.data(), p2.data(), &n2) == HHP_OK);
        std::vector<int> seen(static_cast<size_t>(m2), 0);
        for (int i = 0; i < m2; ++i)
            if (p2[static_cast<size_t>(i)] >= 0 && p2[static_cast<size_t>(i)] < m2) ++seen[static_cast<size_t>(p2[static_cast<size_t>(i)])];
        for (int i = 0; i < m2; ++i) CHECK(seen[static_cast<size_t>(i)] == 1);
        CHECK(m2 == 0 ? n2 == 0 : n2 >= 1);
    }
    const int brp[3] = {0, 1, 2}, bcol[2] = {0, 5};
    int bperm[2], bn = 0;
    CHECK(hhp_reorder_color(2, brp, bcol, bperm, &bn) == HHP_ERR_ARG);
}

}  // namespace

int main(int argc, char **argv) {
    if (argc < 2) {
        std::fprintf(stderr, "usage: sanitize_host <scratch dir>\n");
        return 2;
    }
    g_dir = argv[1];
    small_matrix_market();
    large_matrix_market();
    vector_files();
    work_plan();
    uniform();
    rcm();
    color();
    if (g_fail) {
        std::fprintf(stderr, "%d checks failed\n", g_fail);
        return 1;
    }
    std::printf("sanitize_host: all checks passed\n");
    return 0;
}
