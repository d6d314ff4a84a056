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
// Parsing reads the whole file and converts with std::from_chars.
#include <algorithm>
#include <cctype>
#include <charconv>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

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

// Parses a Matrix Market file into host CSR arrays.
hhp_status read_mtx(const char *path, int &m, int &n, int &nnz, std::vector<int> &rowptr, std::vector<int> &col,
                    std::vector<double> &val) {
    std::string buf;
    if (!path || !read_file(path, buf)) {
        set_error("cannot read matrix file '%s'", path ? path : "(null)");
        return HHP_ERR_IO;
    }
    const char *p = buf.data(), *e = buf.data() + buf.size();
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
}

extern "C" hhp_status hhp_vector_write(const char *path, int size, const double *v, int exact) {
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
}

extern "C" hhp_status hhp_mtx_read(const char *path, int *m, int *n, int *nnz, int **rowptr, int **col,
                                   double **val) {
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
}

extern "C" void hhp_free(void *p) { std::free(p); }
