// hhp_io.cpp -- Matrix Market and vector text files, host side.
//
// Matrix Market: same acceptance and ordering as the reference's readMatrixMarketFromFile
// (src/util/hhp_wrap_bora.c:13-104) with the banner/size rules of mm_read_banner and
// mm_read_mtx_crd_size (src/dependencies/mmio/mmio.c:96-217):
//   banner "%%MatrixMarket matrix coordinate <real|integer> general" (case-insensitive tokens);
//   complex, array, symmetric (rejected by the reference) and pattern / skew-symmetric /
//   hermitian files (which the reference would misread) are rejected with HHP_ERR_FORMAT;
//   '%' comment lines, then "M N nz", then nz triplets "i j v", 1-based;
//   rows in order, entries of a row in file order, duplicates kept (SpMV sums them).
// Unlike the reference (fscanf, unchecked), short files and out-of-range indices are errors.
// Parsing maps the whole file (reads it where it cannot be mapped) and converts with
// std::from_chars; large files are parsed by one thread per core on line-aligned chunks, joined
// in file order (so the CSR is identical to the serial parse), and any irregularity (a malformed
// entry, a count mismatch) re-parses serially for the exact error message.
//
// Binary CSR files ("HHPCSR01" magic, then int64 m, n, nnz, then rowptr[m+1] and col[nnz] as
// int32 and val[nnz] as FP64, little-endian) skip text parsing altogether: hhp_csr_file_write
// stores a matrix once, and every reader that takes a Matrix Market path accepts them.
#include <algorithm>
#include <cctype>
#include <charconv>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <system_error>
#include <thread>
#include <vector>

#include <fcntl.h>
#include <sys/mman.h>
#include <sys/stat.h>
#include <unistd.h>

#include "hhp_internal.h"

namespace hhp {

namespace {

bool read_file(const char *path, std::string &buf) {
    FILE *f = std::fopen(path, "rb");
    if (!f) return false;
    std::fseek(f, 0, SEEK_END);
    const long sz = std::ftell(f);
    std::fseek(f, 0, SEEK_SET);
    if (sz < 0) {
        std::fclose(f);
        return false;
    }
    buf.resize(static_cast<size_t>(sz));
    const size_t got = sz > 0 ? std::fread(&buf[0], 1, static_cast<size_t>(sz), f) : 0;
    std::fclose(f);
    return got == static_cast<size_t>(sz);
}

// A read-only view of a whole file: mapped from the page cache (no copy, no zero-fill of a
// fresh buffer), or read into memory where mapping is not possible.
struct FileView {
    const char *data = nullptr;
    size_t size = 0;
    void *map = nullptr;
    std::string copy;
    FileView() = default;
    FileView(const FileView &) = delete;
    FileView &operator=(const FileView &) = delete;
    ~FileView() {
        if (map) munmap(map, size);
    }
    bool open(const char *path) {
        const int fd = ::open(path, O_RDONLY);
        if (fd >= 0) {
            struct stat st;
            if (fstat(fd, &st) == 0 && st.st_size > 0) {
                void *m = mmap(nullptr, static_cast<size_t>(st.st_size), PROT_READ, MAP_PRIVATE, fd, 0);
                if (m != MAP_FAILED) {
                    map = m;
                    data = static_cast<const char *>(m);
                    size = static_cast<size_t>(st.st_size);
                    ::close(fd);
                    return true;
                }
            }
            ::close(fd);
        }
        if (!read_file(path, copy)) return false;
        data = copy.data();
        size = copy.size();
        return true;
    }
};

struct Cursor {
    const char *p, *e;
    void skip_ws() {
        while (p < e && std::isspace(static_cast<unsigned char>(*p))) ++p;
    }
    template <typename T>
    bool num(T &out) {
        skip_ws();
        if (p >= e) return false;
        const char *q = p;
        if (*q == '+') ++q;  // from_chars rejects a leading '+', scanf accepts it
        auto r = std::from_chars(q, e, out);
        if (r.ec != std::errc()) return false;
        p = r.ptr;
        return true;
    }
};

std::string lower(std::string s) {
    for (char &c : s) c = static_cast<char>(std::tolower(static_cast<unsigned char>(c)));
    return s;
}

}  // namespace

namespace {

constexpr char kCsrMagic[8] = {'H', 'H', 'P', 'C', 'S', 'R', '0', '1'};

// One thread's entries of a line-aligned chunk, in file order.
struct EntryChunk {
    std::vector<int> ri, ci;
    std::vector<double> vv;
    bool ok = true;        // every triplet in the chunk parsed and in range
    bool sorted = true;    // rows non-decreasing inside the chunk
};

void parse_chunk(const char *p, const char *e, long long M, long long N, EntryChunk &out) {
    const size_t guess = static_cast<size_t>(e - p) / 24 + 16;
    out.ri.reserve(guess);
    out.ci.reserve(guess);
    out.vv.reserve(guess);
    Cursor c{p, e};
    int last = -1;
    for (;;) {
        c.skip_ws();
        if (c.p >= c.e) return;
        long long i = 0, j = 0;
        double v = 0.0;
        if (!c.num(i) || !c.num(j) || !c.num(v) || i < 1 || i > M || j < 1 || j > N) {
            out.ok = false;
            return;
        }
        const int r = static_cast<int>(i - 1);
        if (r < last) out.sorted = false;
        last = r;
        out.ri.push_back(r);
        out.ci.push_back(static_cast<int>(j - 1));
        out.vv.push_back(v);
    }
}

// Parallel parse of the entry section [p, e) into CSR; false if the serial path must run (a
// malformed or out-of-range entry, or a count other than nnz).
// fn(t) for t in [0, T) on T threads; a share whose thread cannot be created runs on this one.
template <typename Fn>
void run_threads(int T, Fn fn) {
    std::vector<std::thread> th;
    th.reserve(static_cast<size_t>(T));
    for (int t = 0; t < T; ++t) {
        try {
            th.emplace_back(fn, t);
        } catch (const std::system_error &) {
            fn(t);
        }
    }
    for (auto &x : th) x.join();
}

bool parse_entries_parallel(const char *p, const char *e, long long M, long long N, int nnz, int m,
                            std::vector<int> &rowptr, std::vector<int> &col, std::vector<double> &val) {
    const size_t bytes = static_cast<size_t>(e - p);
    const unsigned hw = std::max(1u, std::thread::hardware_concurrency());
    const int T = static_cast<int>(std::min<size_t>(std::min(hw, 64u), bytes / (4u << 20)));
    if (T < 2) return false;
    std::vector<const char *> cut(static_cast<size_t>(T) + 1);
    cut[0] = p;
    cut[static_cast<size_t>(T)] = e;
    for (int t = 1; t < T; ++t) {
        const char *q = p + bytes * static_cast<size_t>(t) / static_cast<size_t>(T);
        const char *nl = static_cast<const char *>(std::memchr(q, '\n', static_cast<size_t>(e - q)));
        cut[static_cast<size_t>(t)] = nl ? nl + 1 : e;
    }
    std::vector<EntryChunk> ch(static_cast<size_t>(T));
    run_threads(T, [&](int t) {
        parse_chunk(std::max(cut[static_cast<size_t>(t)], cut[0]),
                    std::max(cut[static_cast<size_t>(t) + 1], cut[static_cast<size_t>(t)]), M, N,
                    ch[static_cast<size_t>(t)]);
    });
    long long total = 0;
    bool sorted = true;
    int prev_last = -1;
    for (const auto &c : ch) {
        if (!c.ok) return false;
        total += static_cast<long long>(c.ri.size());
        if (!c.sorted || (!c.ri.empty() && c.ri.front() < prev_last)) sorted = false;
        if (!c.ri.empty()) prev_last = c.ri.back();
    }
    if (total != nnz) return false;
    rowptr.assign(static_cast<size_t>(m) + 1, 0);
    col.resize(static_cast<size_t>(nnz));
    val.resize(static_cast<size_t>(nnz));
    if (sorted) {
        // row counts: each chunk's rows form a range that meets its neighbours' only at the ends,
        // so the chunks count their own rows in parallel and only boundary rows are merged
        std::vector<std::vector<int>> edge(static_cast<size_t>(T));  // {first row, its count, last row, its count}
        run_threads(T, [&](int t) {
                const EntryChunk &c = ch[static_cast<size_t>(t)];
                if (c.ri.empty()) return;
                const int first = c.ri.front(), last = c.ri.back();
                int nf = 0, nl = 0;
                for (int r : c.ri) {
                    if (r == first) ++nf;
                    else if (r == last) ++nl;
                    else rowptr[static_cast<size_t>(r) + 1]++;  // interior rows belong to this chunk alone
                }
                edge[static_cast<size_t>(t)] = {first, nf, last, nl};
            });
        for (const auto &eg : edge) {
            if (eg.empty()) continue;
            rowptr[static_cast<size_t>(eg[0]) + 1] += eg[1];
            if (eg[2] != eg[0]) rowptr[static_cast<size_t>(eg[2]) + 1] += eg[3];
        }
        for (int r = 0; r < m; ++r) rowptr[static_cast<size_t>(r) + 1] += rowptr[static_cast<size_t>(r)];
        // rows in file order already: the CSR is the chunks' concatenation
        std::vector<size_t> off(static_cast<size_t>(T) + 1, 0);
        for (int t = 0; t < T; ++t) off[static_cast<size_t>(t) + 1] = off[static_cast<size_t>(t)] + ch[static_cast<size_t>(t)].ri.size();
        run_threads(T, [&](int t) {
                const EntryChunk &c = ch[static_cast<size_t>(t)];
                if (c.ci.empty()) return;
                std::memcpy(col.data() + off[static_cast<size_t>(t)], c.ci.data(), sizeof(int) * c.ci.size());
                std::memcpy(val.data() + off[static_cast<size_t>(t)], c.vv.data(), sizeof(double) * c.vv.size());
            });
    } else {
        // stable counting sort by row, chunks in file order: entries of a row keep file order
        for (const auto &c : ch)
            for (int r : c.ri) rowptr[static_cast<size_t>(r) + 1]++;
        for (int r = 0; r < m; ++r) rowptr[static_cast<size_t>(r) + 1] += rowptr[static_cast<size_t>(r)];
        std::vector<int> fill(rowptr.begin(), rowptr.end() - 1);
        for (const auto &c : ch)
            for (size_t k = 0; k < c.ri.size(); ++k) {
                const int d = fill[static_cast<size_t>(c.ri[k])]++;
                col[static_cast<size_t>(d)] = c.ci[k];
                val[static_cast<size_t>(d)] = c.vv[k];
            }
    }
    return true;
}

// Binary CSR file (see the file comment); false if `buf` does not start with the magic.
bool is_csr_file(const FileView &buf) {
    return buf.size >= sizeof(kCsrMagic) && std::memcmp(buf.data, kCsrMagic, sizeof(kCsrMagic)) == 0;
}

hhp_status parse_csr_file(const char *path, const FileView &buf, int &m, int &n, int &nnz,
                          std::vector<int> &rowptr, std::vector<int> &col, std::vector<double> &val) {
    long long h[3];
    if (buf.size < sizeof(kCsrMagic) + sizeof(h)) {
        set_error("'%s': truncated binary CSR header", path);
        return HHP_ERR_FORMAT;
    }
    std::memcpy(h, buf.data + sizeof(kCsrMagic), sizeof(h));
    if (h[0] < 0 || h[1] < 0 || h[2] < 0 || h[0] > 2147483646LL || h[1] > 2147483646LL || h[2] > 2147483646LL) {
        set_error("'%s': binary CSR sizes out of range", path);
        return HHP_ERR_FORMAT;
    }
    const size_t need = sizeof(kCsrMagic) + sizeof(h) + sizeof(int) * static_cast<size_t>(h[0] + 1) +
                        (sizeof(int) + sizeof(double)) * static_cast<size_t>(h[2]);
    if (buf.size != need) {
        set_error("'%s': binary CSR file has %zu bytes, expected %zu", path, buf.size, need);
        return HHP_ERR_FORMAT;
    }
    m = static_cast<int>(h[0]);
    n = static_cast<int>(h[1]);
    nnz = static_cast<int>(h[2]);
    const char *q = buf.data + sizeof(kCsrMagic) + sizeof(h);
    rowptr.resize(static_cast<size_t>(m) + 1);
    col.resize(static_cast<size_t>(nnz));
    val.resize(static_cast<size_t>(nnz));
    std::memcpy(rowptr.data(), q, sizeof(int) * rowptr.size());
    q += sizeof(int) * rowptr.size();
    if (nnz) std::memcpy(col.data(), q, sizeof(int) * col.size());
    q += sizeof(int) * col.size();
    if (nnz) std::memcpy(val.data(), q, sizeof(double) * val.size());
    // the same validity rules as a Matrix Market file: monotone row pointers, columns in range
    if (rowptr[0] != 0 || rowptr[static_cast<size_t>(m)] != nnz) {
        set_error("'%s': binary CSR row pointers do not span 0..nnz", path);
        return HHP_ERR_FORMAT;
    }
    for (int r = 0; r < m; ++r)
        if (rowptr[static_cast<size_t>(r) + 1] < rowptr[static_cast<size_t>(r)]) {
            set_error("'%s': binary CSR row pointers decrease at row %d", path, r);
            return HHP_ERR_FORMAT;
        }
    for (int k = 0; k < nnz; ++k)
        if (col[static_cast<size_t>(k)] < 0 || col[static_cast<size_t>(k)] >= n) {
            set_error("'%s': binary CSR column index %d out of range at entry %d", path, col[static_cast<size_t>(k)], k);
            return HHP_ERR_FORMAT;
        }
    return HHP_OK;
}

}  // namespace

// Parses a Matrix Market (or binary CSR) file into host CSR arrays.
hhp_status read_mtx(const char *path, int &m, int &n, int &nnz, std::vector<int> &rowptr, std::vector<int> &col,
                    std::vector<double> &val) {
    FileView buf;
    if (!path || !buf.open(path)) {
        set_error("cannot read matrix file '%s'", path ? path : "(null)");
        return HHP_ERR_IO;
    }
    if (is_csr_file(buf)) return parse_csr_file(path, buf, m, n, nnz, rowptr, col, val);
    const char *p = buf.data, *e = buf.data + buf.size;
    const char *eol = static_cast<const char *>(std::memchr(p, '\n', static_cast<size_t>(e - p)));
    std::string first(p, eol ? eol : e);
    char t[5][64];
    if (std::sscanf(first.c_str(), "%63s %63s %63s %63s %63s", t[0], t[1], t[2], t[3], t[4]) != 5 ||
        std::strncmp(t[0], "%%MatrixMarket", 14) != 0) {
        set_error("'%s': missing or malformed Matrix Market banner", path);
        return HHP_ERR_FORMAT;
    }
    const std::string obj = lower(t[1]), fmt = lower(t[2]), field = lower(t[3]), sym = lower(t[4]);
    if (obj != "matrix" || fmt != "coordinate" || (field != "real" && field != "integer") || sym != "general") {
        set_error("'%s': unsupported Matrix Market type [%s %s %s %s]", path, t[1], t[2], t[3], t[4]);
        return HHP_ERR_FORMAT;
    }
    p = eol ? eol + 1 : e;
    // comment lines
    while (p < e) {
        const char *q = p;
        while (q < e && (*q == ' ' || *q == '\t' || *q == '\r')) ++q;
        if (q < e && *q == '%') {
            const char *nl = static_cast<const char *>(std::memchr(q, '\n', static_cast<size_t>(e - q)));
            p = nl ? nl + 1 : e;
            continue;
        }
        break;
    }
    Cursor c{p, e};
    long long M = 0, N = 0, NZ = 0;
    if (!c.num(M) || !c.num(N) || !c.num(NZ) || M < 0 || N < 0 || NZ < 0 || M > 2147483646LL ||
        N > 2147483646LL || NZ > 2147483646LL) {
        set_error("'%s': malformed size line", path);
        return HHP_ERR_FORMAT;
    }
    // the rest of the size line is ignored, as sscanf on that line does in mm_read_mtx_crd_size
    while (c.p < c.e && *c.p != '\n') ++c.p;
    m = static_cast<int>(M);
    n = static_cast<int>(N);
    nnz = static_cast<int>(NZ);
    if (parse_entries_parallel(c.p, c.e, M, N, nnz, m, rowptr, col, val)) return HHP_OK;
    std::vector<int> ri(static_cast<size_t>(nnz)), ci(static_cast<size_t>(nnz));
    std::vector<double> vv(static_cast<size_t>(nnz));
    rowptr.assign(static_cast<size_t>(m) + 1, 0);
    for (int k = 0; k < nnz; ++k) {
        long long i = 0, j = 0;
        double v = 0.0;
        if (!c.num(i) || !c.num(j) || !c.num(v)) {
            set_error("'%s': entry %d of %d missing or malformed", path, k + 1, nnz);
            return HHP_ERR_FORMAT;
        }
        if (i < 1 || i > M || j < 1 || j > N) {
            set_error("'%s': entry %d (%lld, %lld) outside %lld x %lld", path, k + 1, i, j, M, N);
            return HHP_ERR_FORMAT;
        }
        ri[static_cast<size_t>(k)] = static_cast<int>(i - 1);
        ci[static_cast<size_t>(k)] = static_cast<int>(j - 1);
        vv[static_cast<size_t>(k)] = v;
        rowptr[static_cast<size_t>(i)]++;
    }
    for (int r = 0; r < m; ++r) rowptr[static_cast<size_t>(r) + 1] += rowptr[static_cast<size_t>(r)];
    col.resize(static_cast<size_t>(nnz));
    val.resize(static_cast<size_t>(nnz));
    std::vector<int> fill(rowptr.begin(), rowptr.end() - 1);
    for (int k = 0; k < nnz; ++k) {
        const int d = fill[static_cast<size_t>(ri[static_cast<size_t>(k)])]++;
        col[static_cast<size_t>(d)] = ci[static_cast<size_t>(k)];
        val[static_cast<size_t>(d)] = vv[static_cast<size_t>(k)];
    }
    return HHP_OK;
}

}  // namespace hhp

extern "C" hhp_status hhp_vector_read(const char *path, int size, double *out) {
    HHP_API_BEGIN
    if (!path || size < 0 || (size > 0 && !out)) {
        hhp::set_error("hhp_vector_read: invalid arguments");
        return HHP_ERR_ARG;
    }
    std::string buf;
    if (!hhp::read_file(path, buf)) {
        hhp::set_error("cannot read vector file '%s'", path);
        return HHP_ERR_IO;
    }
    hhp::Cursor c{buf.data(), buf.data() + buf.size()};
    for (int i = 0; i < size; ++i) {
        if (!c.num(out[i])) {
            hhp::set_error("'%s': expected %d values, found %d", path, size, i);
            return HHP_ERR_IO;
        }
    }
    return HHP_OK;
    HHP_API_END
}

extern "C" hhp_status hhp_vector_write(const char *path, int size, const double *v, int exact) {
    HHP_API_BEGIN
    if (!path || size < 0 || (size > 0 && !v)) {
        hhp::set_error("hhp_vector_write: invalid arguments");
        return HHP_ERR_ARG;
    }
    FILE *f = std::fopen(path, "w");
    if (!f) {
        hhp::set_error("cannot write vector file '%s'", path);
        return HHP_ERR_IO;
    }
    for (int i = 0; i < size; ++i) {
        if (std::fprintf(f, exact ? "%.17g\n" : "%lf\n", v[i]) < 0) {
            std::fclose(f);
            hhp::set_error("write to '%s' failed", path);
            return HHP_ERR_IO;
        }
    }
    if (std::fclose(f) != 0) {
        hhp::set_error("closing '%s' failed", path);
        return HHP_ERR_IO;
    }
    return HHP_OK;
    HHP_API_END
}

extern "C" hhp_status hhp_mtx_read(const char *path, int *m, int *n, int *nnz, int **rowptr, int **col,
                                   double **val) {
    HHP_API_BEGIN
    if (!m || !n || !nnz || !rowptr || !col || !val) {
        hhp::set_error("hhp_mtx_read: null output pointer");
        return HHP_ERR_ARG;
    }
    std::vector<int> rp, c;
    std::vector<double> v;
    int mm = 0, nn = 0, nz = 0;
    const hhp_status st = hhp::read_mtx(path, mm, nn, nz, rp, c, v);
    if (st != HHP_OK) return st;
    int *a = static_cast<int *>(std::malloc(sizeof(int) * rp.size()));
    int *b = static_cast<int *>(std::malloc(sizeof(int) * (c.size() + 1)));
    double *d = static_cast<double *>(std::malloc(sizeof(double) * (v.size() + 1)));
    if (!a || !b || !d) {
        std::free(a);
        std::free(b);
        std::free(d);
        hhp::set_error("hhp_mtx_read: out of host memory");
        return HHP_ERR_OOM;
    }
    std::memcpy(a, rp.data(), sizeof(int) * rp.size());
    if (!c.empty()) std::memcpy(b, c.data(), sizeof(int) * c.size());
    if (!v.empty()) std::memcpy(d, v.data(), sizeof(double) * v.size());
    *m = mm;
    *n = nn;
    *nnz = nz;
    *rowptr = a;
    *col = b;
    *val = d;
    return HHP_OK;
    HHP_API_END
}

extern "C" void hhp_free(void *p) { std::free(p); }

extern "C" hhp_status hhp_csr_file_write(const char *path, int m, int n, int nnz, const int *rowptr, const int *col,
                                         const double *val) {
    HHP_API_BEGIN
    if (!path || m < 0 || n < 0 || nnz < 0 || !rowptr || (nnz > 0 && (!col || !val))) {
        hhp::set_error("hhp_csr_file_write: invalid arguments");
        return HHP_ERR_ARG;
    }
    if (rowptr[0] != 0 || rowptr[m] != nnz) {
        hhp::set_error("hhp_csr_file_write: rowptr[0] must be 0 and rowptr[m] must equal nnz");
        return HHP_ERR_ARG;
    }
    FILE *f = std::fopen(path, "wb");
    if (!f) {
        hhp::set_error("cannot write '%s'", path);
        return HHP_ERR_IO;
    }
    const long long h[3] = {m, n, nnz};
    bool ok = std::fwrite(hhp::kCsrMagic, 1, sizeof(hhp::kCsrMagic), f) == sizeof(hhp::kCsrMagic) &&
              std::fwrite(h, sizeof(h), 1, f) == 1 &&
              std::fwrite(rowptr, sizeof(int), static_cast<size_t>(m) + 1, f) == static_cast<size_t>(m) + 1;
    if (ok && nnz > 0)
        ok = std::fwrite(col, sizeof(int), static_cast<size_t>(nnz), f) == static_cast<size_t>(nnz) &&
             std::fwrite(val, sizeof(double), static_cast<size_t>(nnz), f) == static_cast<size_t>(nnz);
    if (std::fclose(f) != 0) ok = false;
    if (!ok) {
        hhp::set_error("write to '%s' failed", path);
        return HHP_ERR_IO;
    }
    return HHP_OK;
    HHP_API_END
}
