/*
 * hhp_oracle.c -- CPU oracle for the BiCGStab / CSR-SpMV path (TEST INFRASTRUCTURE ONLY).
 *
 * A plain-C restatement of HetHypPar's CPU path, used by the tests, the smoke check and the
 * benchmark's CPU-baseline leg, to compare against. The product never links or calls this file.
 * Compile with -ffp-contract=off (the build does): every multiply and add then rounds on its
 * own, in the order the reference's loops use, so results match the reference bit for bit on
 * the golden vectors in tests/golden/ (made from the reference's own compiled functions).
 */
#include "hhp_oracle.h"

#include <ctype.h>
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

void orc_free(void *p) { free(p); }

/* ---------------------------------------------------------------------------------------------
 * Matrix Market reader.
 * Banner and size rules: mm_read_banner (src/dependencies/mmio/mmio.c:96-179) -- five tokens,
 * the first must start with "%%MatrixMarket", the rest are compared case-insensitively;
 * mm_read_mtx_crd_size (mmio.c:189-217) -- skip '%' lines, then "M N nz".
 * Acceptance: readMatrixMarketFromFile (src/util/hhp_wrap_bora.c:36-41) rejects complex,
 * non-matrix, non-coordinate and symmetric files. The reference would go on to misread pattern
 * files (no value column) and to treat skew/hermitian files as general; the oracle rejects them.
 * CSR build: count per row, prefix sum, then fill from the last entry backwards with a
 * pre-decrement (hhp_wrap_bora.c:61-85), which keeps every row's entries in file order.
 * ------------------------------------------------------------------------------------------- */
static void lower(char *s) { for (; *s; ++s) *s = (char)tolower((unsigned char)*s); }

int orc_read_mtx(const char *path, int *m_out, int *n_out, int *nnz_out, int **rowptr_out, int **col_out,
                 double **val_out) {
    FILE *f = fopen(path, "r");
    if (!f) return ORC_ERR_IO;
    char line[1100], banner[64], mtx[64], crd[64], dtype[64], storage[64];
    if (!fgets(line, sizeof line, f)) { fclose(f); return ORC_ERR_FORMAT; }
    if (sscanf(line, "%63s %63s %63s %63s %63s", banner, mtx, crd, dtype, storage) != 5) {
        fclose(f);
        return ORC_ERR_FORMAT;
    }
    lower(mtx); lower(crd); lower(dtype); lower(storage);
    if (strncmp(banner, "%%MatrixMarket", 14) != 0 || strcmp(mtx, "matrix") != 0 ||
        strcmp(crd, "coordinate") != 0 || (strcmp(dtype, "real") != 0 && strcmp(dtype, "integer") != 0) ||
        strcmp(storage, "general") != 0) {
        fclose(f);
        return ORC_ERR_FORMAT;
    }
    int M = 0, N = 0, NZ = 0;
    do {
        if (!fgets(line, sizeof line, f)) { fclose(f); return ORC_ERR_FORMAT; }
    } while (line[0] == '%');
    if (sscanf(line, "%d %d %d", &M, &N, &NZ) != 3) {
        int got;
        do {
            got = fscanf(f, "%d %d %d", &M, &N, &NZ);
            if (got == EOF) { fclose(f); return ORC_ERR_FORMAT; }
        } while (got != 3);
    }
    if (M < 0 || N < 0 || NZ < 0) { fclose(f); return ORC_ERR_FORMAT; }
    int *ri = (int *)malloc(sizeof(int) * ((size_t)NZ + 1));
    int *ci = (int *)malloc(sizeof(int) * ((size_t)NZ + 1));
    double *vv = (double *)malloc(sizeof(double) * ((size_t)NZ + 1));
    int *rowptr = (int *)calloc((size_t)M + 1, sizeof(int));
    int *col = (int *)malloc(sizeof(int) * ((size_t)NZ + 1));
    double *val = (double *)malloc(sizeof(double) * ((size_t)NZ + 1));
    if (!ri || !ci || !vv || !rowptr || !col || !val) {
        free(ri); free(ci); free(vv); free(rowptr); free(col); free(val);
        fclose(f);
        return ORC_ERR_IO;
    }
    for (int i = 0; i < NZ; ++i) {
        if (fscanf(f, "%d %d %lf", &ri[i], &ci[i], &vv[i]) != 3 || ri[i] < 1 || ri[i] > M || ci[i] < 1 ||
            ci[i] > N) {
            free(ri); free(ci); free(vv); free(rowptr); free(col); free(val);
            fclose(f);
            return ORC_ERR_FORMAT;
        }
        ri[i]--;
        ci[i]--;
        rowptr[ri[i]]++;
    }
    fclose(f);
    for (int i = 1; i <= M; ++i) rowptr[i] += rowptr[i - 1];
    for (int i = NZ - 1; i >= 0; --i) {
        int off = --rowptr[ri[i]];
        col[off] = ci[i];
        val[off] = vv[i];
    }
    free(ri); free(ci); free(vv);
    *m_out = M; *n_out = N; *nnz_out = NZ;
    *rowptr_out = rowptr; *col_out = col; *val_out = val;
    return ORC_OK;
}

/* vector_read (src/util/hhp_cpu.c:411-428): fscanf("%lf") until `size` values or a failure.
 * Unlike the reference (which post-increments the index even on a failed read) this returns the
 * exact count, so a short file is detectable. */
int orc_vector_read(const char *path, int size, double *out) {
    FILE *f = fopen(path, "r");
    if (!f) return -1;
    int i = 0;
    while (i < size && fscanf(f, "%lf", &out[i]) == 1) ++i;
    fclose(f);
    return i;
}

int orc_vector_write(const char *path, int size, const double *v, int exact) {
    FILE *f = fopen(path, "w");
    if (!f) return ORC_ERR_IO;
    for (int i = 0; i < size; ++i) {
        if (fprintf(f, exact ? "%.17g\n" : "%lf\n", v[i]) < 0) { fclose(f); return ORC_ERR_IO; }
    }
    fclose(f);
    return ORC_OK;
}

/* ---------------------------------------------------------------------------------------------
 * SpMV and BLAS-1
 * ------------------------------------------------------------------------------------------- */
void orc_spmv(int m, const int *rowptr, const int *col, const double *val, const double *x, double *y) {
    for (int i = 0; i < m; ++i) {
        double res = 0.0;
        for (int j = rowptr[i]; j < rowptr[i + 1]; ++j) res += val[j] * x[col[j]];
        y[i] = res;
    }
}

void orc_spmv_fma(int m, const int *rowptr, const int *col, const double *val, const double *x, double *y) {
    for (int i = 0; i < m; ++i) {
        double res = 0.0;
        for (int j = rowptr[i]; j < rowptr[i + 1]; ++j) res = fma(val[j], x[col[j]], res);
        y[i] = res;
    }
}

void orc_spmv_omp(int m, const int *rowptr, const int *col, const double *val, const double *x, double *y,
                  int nthreads) {
#ifdef _OPENMP
#pragma omp parallel for schedule(guided) num_threads(nthreads > 0 ? nthreads : omp_get_max_threads())
#endif
    for (int i = 0; i < m; ++i) {
        double res = 0.0;
        for (int j = rowptr[i]; j < rowptr[i + 1]; ++j) res += val[j] * x[col[j]];
        y[i] = res;
    }
    (void)nthreads;
}

void orc_spmv_t(int m, int n, const int *rowptr, const int *col, const double *val, const double *x, double *y) {
    for (int j = 0; j < n; ++j) y[j] = 0.0;
    for (int i = 0; i < m; ++i)
        for (int k = rowptr[i]; k < rowptr[i + 1]; ++k) y[col[k]] += val[k] * x[i];
}

double orc_dot(int n, const double *a, const double *b) {
    double res = 0.0;
    for (int i = 0; i < n; ++i) res += a[i] * b[i];
    return res;
}

/* ---------------------------------------------------------------------------------------------
 * BiCGStab, the loop of src/entry/bicgstab_cpu.c:176-255.
 * Each element update below performs the same roundings, in the same order, as the chain of
 * vector_scale_seq / vector_sub_seq / vector_add_seq calls it replaces (the calls are
 * element-wise, so running them element by element changes nothing):
 *   P: V*=omega; P-=V; P*=beta; P+=R        (bicgstab_cpu.c:210-213)
 *   S: S=V*alpha; S=R-S                     (:222-223)
 *   X: Y=P*alpha; X+=Y; Y=S*omega; X+=Y     (:232-235)
 *   R: R=T*omega; R=S-R                     (:238-239)
 * The unused tol=S.S (:242) is skipped; it changes no state.
 * ------------------------------------------------------------------------------------------- */
typedef struct {
    double *R, *R0, *P, *V, *S, *T, *Y;
} orc_ws;

static int ws_alloc(orc_ws *w, int m) {
    double *blk = (double *)calloc((size_t)7 * (size_t)(m > 0 ? m : 1), sizeof(double));
    if (!blk) return ORC_ERR_IO;
    size_t s = (size_t)(m > 0 ? m : 1);
    w->R = blk; w->R0 = blk + s; w->P = blk + 2 * s; w->V = blk + 3 * s;
    w->S = blk + 4 * s; w->T = blk + 5 * s; w->Y = blk + 6 * s;
    return ORC_OK;
}
static void ws_free(orc_ws *w) { free(w->R); }

static double true_relres(int m, const int *rowptr, const int *col, const double *val, const double *b,
                          const double *x, double *Y) {
    orc_spmv(m, rowptr, col, val, x, Y);
    for (int i = 0; i < m; ++i) Y[i] = b[i] - Y[i];
    double sy = orc_dot(m, Y, Y), sb = orc_dot(m, b, b);
    return sqrt(sy / sb);
}

typedef struct {
    double rho, alpha, omega, rr0;
} orc_scalars;

static void bicg_init(int m, const int *rowptr, const int *col, const double *val, const double *b,
                      const double *x, orc_ws *w, orc_scalars *s) {
    s->rho = 1.0; s->alpha = 1.0; s->omega = 1.0;
    orc_spmv(m, rowptr, col, val, x, w->Y);
    for (int i = 0; i < m; ++i) {
        w->R[i] = b[i] - w->Y[i];
        w->R0[i] = w->R[i];
        w->P[i] = 0.0;
        w->V[i] = 0.0;
        w->Y[i] = 0.0;
    }
    s->rr0 = orc_dot(m, w->R0, w->R0);
}

static void bicg_iter(int m, const int *rowptr, const int *col, const double *val, double *x, orc_ws *w,
                      orc_scalars *s) {
    double temp_rho = orc_dot(m, w->R, w->R0);
    double beta = (temp_rho / s->rho) * (s->alpha / s->omega);
    s->rho = temp_rho;
    for (int i = 0; i < m; ++i) {
        double v = w->V[i] * s->omega;
        double p = w->P[i] - v;
        p = p * beta;
        w->P[i] = p + w->R[i];
    }
    orc_spmv(m, rowptr, col, val, w->P, w->V);
    s->alpha = s->rho / orc_dot(m, w->R0, w->V);
    for (int i = 0; i < m; ++i) {
        double t = w->V[i] * s->alpha;
        w->S[i] = w->R[i] - t;
    }
    orc_spmv(m, rowptr, col, val, w->S, w->T);
    s->omega = orc_dot(m, w->T, w->S) / orc_dot(m, w->T, w->T);
    for (int i = 0; i < m; ++i) {
        double y = w->P[i] * s->alpha;
        double xi = x[i] + y;
        y = w->S[i] * s->omega;
        x[i] = xi + y;
        double r = w->T[i] * s->omega;
        w->R[i] = w->S[i] - r;
    }
}

int orc_bicgstab_fixed(int m, const int *rowptr, const int *col, const double *val, const double *b, double *x,
                       int niters, double *relres, double *hist_true, double *hist_rec) {
    if (m <= 0 || niters < 0) return ORC_ERR_ARG;
    orc_ws w;
    if (ws_alloc(&w, m)) return ORC_ERR_IO;
    orc_scalars s;
    bicg_init(m, rowptr, col, val, b, x, &w, &s);
    double *scratch = NULL;
    if (hist_true) scratch = (double *)malloc(sizeof(double) * (size_t)m);
    for (int it = 0; it < niters; ++it) {
        bicg_iter(m, rowptr, col, val, x, &w, &s);
        if (hist_true) hist_true[it] = true_relres(m, rowptr, col, val, b, x, scratch);
        if (hist_rec) hist_rec[it] = sqrt(orc_dot(m, w.R, w.R) / s.rr0);
    }
    free(scratch);
    if (relres) *relres = true_relres(m, rowptr, col, val, b, x, w.Y);
    ws_free(&w);
    return ORC_OK;
}

int orc_bicgstab_iters_to_tol(int m, const int *rowptr, const int *col, const double *val, const double *b,
                              double *x, double rtol, int maxit, double *relres) {
    if (m <= 0 || maxit < 0) return -1;
    orc_ws w;
    if (ws_alloc(&w, m)) return -1;
    orc_scalars s;
    bicg_init(m, rowptr, col, val, b, x, &w, &s);
    double *scratch = (double *)malloc(sizeof(double) * (size_t)m);
    int found = -1;
    double rr = true_relres(m, rowptr, col, val, b, x, scratch);
    if (rr <= rtol) found = 0;
    for (int it = 1; found < 0 && it <= maxit; ++it) {
        bicg_iter(m, rowptr, col, val, x, &w, &s);
        rr = true_relres(m, rowptr, col, val, b, x, scratch);
        if (rr <= rtol) found = it;
    }
    if (relres) *relres = rr;
    free(scratch);
    ws_free(&w);
    return found;
}

/* ---------------------------------------------------------------------------------------------
 * The MPI-rank decomposition of src/entry/bicgstab_mpi.c:256-300 with ranks as threads.
 * ------------------------------------------------------------------------------------------- */
int orc_bicgstab_fixed_mt(int m, const int *rowptr, const int *col, const double *val, const double *b, double *x,
                          int niters, int nthreads, double *relres) {
    if (m <= 0 || niters < 0) return ORC_ERR_ARG;
#ifndef _OPENMP
    nthreads = 1;
#endif
    if (nthreads < 1) nthreads = 1;
    orc_ws w;
    if (ws_alloc(&w, m)) return ORC_ERR_IO;
    double *part = (double *)calloc((size_t)nthreads * 8, sizeof(double));
    double result = 0.0;
#ifdef _OPENMP
#pragma omp parallel num_threads(nthreads)
#endif
    {
#ifdef _OPENMP
        int t = omp_get_thread_num();
        int nt = omp_get_num_threads();
#else
        int t = 0, nt = 1;
#endif
        int lo = (int)((long long)m * t / nt), hi = (int)((long long)m * (t + 1) / nt);
        int cnt = hi - lo;
        double rho = 1.0, alpha = 1.0, omega = 1.0;
        orc_spmv(cnt, rowptr + lo, col, val, x, w.Y + lo);
        for (int i = lo; i < hi; ++i) {
            w.R[i] = b[i] - w.Y[i];
            w.R0[i] = w.R[i];
            w.P[i] = 0.0;
            w.V[i] = 0.0;
        }
#ifdef _OPENMP
#pragma omp barrier
#endif
        for (int it = 0; it < niters; ++it) {
            part[t * 8 + 0] = orc_dot(cnt, w.R + lo, w.R0 + lo);
#ifdef _OPENMP
#pragma omp barrier
#endif
            double temp_rho = 0.0;
            for (int q = 0; q < nt; ++q) temp_rho += part[q * 8 + 0];
            double beta = (temp_rho / rho) * (alpha / omega);
            rho = temp_rho;
            for (int i = lo; i < hi; ++i) {
                double v = w.V[i] * omega;
                double p = w.P[i] - v;
                p = p * beta;
                w.P[i] = p + w.R[i];
            }
#ifdef _OPENMP
#pragma omp barrier
#endif
            orc_spmv(cnt, rowptr + lo, col, val, w.P, w.V + lo);
            part[t * 8 + 1] = orc_dot(cnt, w.R0 + lo, w.V + lo);
#ifdef _OPENMP
#pragma omp barrier
#endif
            double rv = 0.0;
            for (int q = 0; q < nt; ++q) rv += part[q * 8 + 1];
            alpha = rho / rv;
            for (int i = lo; i < hi; ++i) {
                double tt = w.V[i] * alpha;
                w.S[i] = w.R[i] - tt;
            }
#ifdef _OPENMP
#pragma omp barrier
#endif
            orc_spmv(cnt, rowptr + lo, col, val, w.S, w.T + lo);
            part[t * 8 + 2] = orc_dot(cnt, w.T + lo, w.S + lo);
            part[t * 8 + 3] = orc_dot(cnt, w.T + lo, w.T + lo);
#ifdef _OPENMP
#pragma omp barrier
#endif
            double ts = 0.0, tt2 = 0.0;
            for (int q = 0; q < nt; ++q) { ts += part[q * 8 + 2]; tt2 += part[q * 8 + 3]; }
            omega = ts / tt2;
            for (int i = lo; i < hi; ++i) {
                double y = w.P[i] * alpha;
                double xi = x[i] + y;
                y = w.S[i] * omega;
                x[i] = xi + y;
                double r = w.T[i] * omega;
                w.R[i] = w.S[i] - r;
            }
            /* part[.,0] of the next iteration is written only after every thread has passed the
             * barrier above, which follows every read of part[.,0] in this iteration. */
        }
#ifdef _OPENMP
#pragma omp barrier
#endif
        orc_spmv(cnt, rowptr + lo, col, val, x, w.Y + lo);
        for (int i = lo; i < hi; ++i) w.Y[i] = b[i] - w.Y[i];
        part[t * 8 + 4] = orc_dot(cnt, w.Y + lo, w.Y + lo);
        part[t * 8 + 5] = orc_dot(cnt, b + lo, b + lo);
#ifdef _OPENMP
#pragma omp barrier
#pragma omp single
#endif
        {
            double sy = 0.0, sb = 0.0;
            for (int q = 0; q < nt; ++q) { sy += part[q * 8 + 4]; sb += part[q * 8 + 5]; }
            result = sqrt(sy / sb);
        }
    }
    if (relres) *relres = result;
    free(part);
    ws_free(&w);
    return ORC_OK;
}

/* ---------------------------------------------------------------------------------------------
 * Transpose and permutation
 * ------------------------------------------------------------------------------------------- */
void orc_csr_to_csc(int m, int n, int nnz, const int *rowptr, const int *col, const double *val, int *colptr,
                    int *rowidx, double *tval) {
    for (int j = 0; j <= n; ++j) colptr[j] = 0;
    for (int k = 0; k < nnz; ++k) colptr[col[k] + 1]++;
    for (int j = 1; j <= n; ++j) colptr[j] += colptr[j - 1];
    int *fill = (int *)calloc((size_t)(n > 0 ? n : 1), sizeof(int));
    for (int i = 0; i < m; ++i) {
        for (int k = rowptr[i]; k < rowptr[i + 1]; ++k) {
            int c = col[k];
            int dest = colptr[c] + fill[c]++;
            rowidx[dest] = i;
            tval[dest] = val[k];
        }
    }
    free(fill);
}

void orc_csr_permute(int m, int nnz, const int *rowptr, const int *col, const double *val, const int *perm,
                     const int *perm_inv, int *orowptr, int *ocol, double *oval) {
    (void)nnz;
    orowptr[0] = 0;
    for (int i = 0; i < m; ++i) orowptr[i + 1] = orowptr[i] + (rowptr[perm[i] + 1] - rowptr[perm[i]]);
    for (int i = 0; i < m; ++i) {
        int old = perm[i], s = rowptr[old], cnt = rowptr[old + 1] - s, d = orowptr[i];
        for (int k = 0; k < cnt; ++k) {
            ocol[d + k] = perm_inv[col[s + k]];
            oval[d + k] = val[s + k];
        }
    }
}

/* ---------------------------------------------------------------------------------------------
 * ILU(0): IKJ factorization (Saad, Algorithm 10.4), the two triangular solves, the
 * preconditioned loop of src/entry/bicgstab_gpu.c:155-290 with steps 9 and 14 enabled, and the
 * greedy multicolouring.
 * ------------------------------------------------------------------------------------------- */
static int diag_positions(int m, const int *rowptr, const int *col, int *dpos) {
    for (int i = 0; i < m; ++i) {
        dpos[i] = -1;
        for (int p = rowptr[i]; p < rowptr[i + 1]; ++p) {
            if (col[p] < 0 || col[p] >= m) return ORC_ERR_ARG;
            if (p > rowptr[i] && col[p] <= col[p - 1]) return ORC_ERR_ARG;
            if (col[p] == i) dpos[i] = p;
        }
        if (dpos[i] < 0) return ORC_ERR_ARG;
    }
    return ORC_OK;
}

int orc_ilu0(int m, const int *rowptr, const int *col, const double *val, double *lu, int *bad_row) {
    if (m <= 0) return ORC_ERR_ARG;
    int *dpos = (int *)malloc(sizeof(int) * (size_t)m);
    if (!dpos) return ORC_ERR_IO;
    int rc = diag_positions(m, rowptr, col, dpos);
    if (rc != ORC_OK) {
        free(dpos);
        return rc;
    }
    memcpy(lu, val, sizeof(double) * (size_t)rowptr[m]);
    if (bad_row) *bad_row = -1;
    for (int i = 0; i < m && rc == ORC_OK; ++i) {
        const int end = rowptr[i + 1];
        for (int p = rowptr[i]; p < dpos[i]; ++p) {
            const int k = col[p];
            const double l = lu[p] / lu[dpos[k]];
            lu[p] = l;
            const int kb = dpos[k] + 1, ke = rowptr[k + 1];
            for (int q = p + 1; q < end; ++q) {
                int lo = kb, hi = ke;
                const int j = col[q];
                while (lo < hi) {
                    int mid = lo + (hi - lo) / 2;
                    if (col[mid] < j) lo = mid + 1;
                    else hi = mid;
                }
                if (lo < ke && col[lo] == j) lu[q] = fma(-l, lu[lo], lu[q]);
            }
        }
        const double u = lu[dpos[i]];
        if (u == 0.0 || !isfinite(u)) {
            if (bad_row) *bad_row = i;
            rc = ORC_ERR_FORMAT;
        }
    }
    free(dpos);
    return rc;
}

/* the butterfly of the GPU's warp-wide rows: at each distance every slot adds its partner */
static double butterfly32(double *a) {
    double b[32];
    for (int off = 16; off >= 1; off >>= 1) {
        for (int l = 0; l < 32; ++l) b[l] = a[l] + a[l ^ off];
        memcpy(a, b, sizeof(b));
    }
    return a[0];
}

static double tri_row(const int *col, const double *lu, int b, int e, const double *z, double rhs) {
    if (e - b <= ORC_ILU_LONG) {
        double acc = rhs;
        for (int p = b; p < e; ++p) acc = fma(-lu[p], z[col[p]], acc);
        return acc;
    }
    if (e - b <= ORC_ILU_BIG) {
        double a[32] = {0};
        for (int p = b; p < e; ++p) a[(p - b) & 31] = fma(lu[p], z[col[p]], a[(p - b) & 31]);
        return rhs - butterfly32(a);
    }
    /* ORC_ILU_BLOCK partial sums, a butterfly over each group of 32, the group sums in order */
    static double a[ORC_ILU_BLOCK];
    memset(a, 0, sizeof(a));
    for (int p = b; p < e; ++p) a[(p - b) % ORC_ILU_BLOCK] = fma(lu[p], z[col[p]], a[(p - b) % ORC_ILU_BLOCK]);
    double tot = 0.0;
    for (int w = 0; w < ORC_ILU_BLOCK / 32; ++w) tot += butterfly32(a + 32 * w);
    return rhs - tot;
}

void orc_ilu0_apply(int m, const int *rowptr, const int *col, const double *lu, const double *r, double *z) {
    int *dpos = (int *)malloc(sizeof(int) * (size_t)(m > 0 ? m : 1));
    if (!dpos || diag_positions(m, rowptr, col, dpos) != ORC_OK) {
        free(dpos);
        for (int i = 0; i < m; ++i) z[i] = NAN;
        return;
    }
    for (int i = 0; i < m; ++i) z[i] = tri_row(col, lu, rowptr[i], dpos[i], z, r[i]);
    for (int i = m - 1; i >= 0; --i) {
        const double dinv = 1.0 / lu[dpos[i]];
        z[i] = tri_row(col, lu, dpos[i] + 1, rowptr[i + 1], z, z[i]) * dinv;
    }
    free(dpos);
}

int orc_bicgstab_ilu0_iters_to_tol(int m, const int *rowptr, const int *col, const double *val, const double *b,
                                   double *x, double rtol, int maxit, double *relres) {
    if (m <= 0 || maxit < 0) return -1;
    const size_t nz = (size_t)rowptr[m];
    double *lu = (double *)malloc(sizeof(double) * (nz ? nz : 1));
    double *blk = (double *)calloc((size_t)9 * (size_t)m, sizeof(double));
    if (!lu || !blk) {
        free(lu);
        free(blk);
        return -2;
    }
    if (orc_ilu0(m, rowptr, col, val, lu, NULL) != ORC_OK) {
        free(lu);
        free(blk);
        return -2;
    }
    double *R = blk, *R0 = blk + m, *P = blk + 2 * (size_t)m, *V = blk + 3 * (size_t)m, *S = blk + 4 * (size_t)m,
           *T = blk + 5 * (size_t)m, *PH = blk + 6 * (size_t)m, *SH = blk + 7 * (size_t)m, *Y = blk + 8 * (size_t)m;
    orc_spmv(m, rowptr, col, val, x, Y);
    for (int i = 0; i < m; ++i) R[i] = R0[i] = b[i] - Y[i];
    double delta = orc_dot(m, R0, R), delta_prev = delta, alpha = 1.0, omega = 1.0;
    double rr = true_relres(m, rowptr, col, val, b, x, Y);
    int found = rr <= rtol ? 0 : -1;
    for (int it = 1; found < 0 && it <= maxit; ++it) {
        if (it == 1) {
            memcpy(P, R, sizeof(double) * (size_t)m);
        } else {
            delta = orc_dot(m, R0, R);
            const double beta = (delta / delta_prev) * (alpha / omega);
            delta_prev = delta;
            for (int i = 0; i < m; ++i) P[i] = R[i] + beta * (P[i] - omega * V[i]);
        }
        orc_ilu0_apply(m, rowptr, col, lu, P, PH);
        orc_spmv(m, rowptr, col, val, PH, V);
        alpha = delta / orc_dot(m, R0, V);
        for (int i = 0; i < m; ++i) {
            x[i] += alpha * PH[i];
            S[i] = R[i] - alpha * V[i];
        }
        orc_ilu0_apply(m, rowptr, col, lu, S, SH);
        orc_spmv(m, rowptr, col, val, SH, T);
        omega = orc_dot(m, T, S) / orc_dot(m, T, T);
        for (int i = 0; i < m; ++i) {
            x[i] += omega * SH[i];
            R[i] = S[i] - omega * T[i];
        }
        rr = true_relres(m, rowptr, col, val, b, x, Y);
        if (rr <= rtol) found = it;
    }
    if (relres) *relres = rr;
    free(lu);
    free(blk);
    return found;
}

int orc_color(int m, const int *rowptr, const int *col, int *color) {
    /* adjacency of A + A^T without the diagonal: the rows of A and the rows of A^T */
    int *tptr = (int *)calloc((size_t)m + 1, sizeof(int));
    int *tcol = (int *)malloc(sizeof(int) * (size_t)(rowptr[m] > 0 ? rowptr[m] : 1));
    int *mark = (int *)malloc(sizeof(int) * (size_t)m + sizeof(int));
    if (!tptr || !tcol || !mark) {
        free(tptr);
        free(tcol);
        free(mark);
        return -1;
    }
    for (int p = 0; p < rowptr[m]; ++p) tptr[col[p] + 1]++;
    for (int j = 0; j < m; ++j) tptr[j + 1] += tptr[j];
    int *fill = (int *)calloc((size_t)m + 1, sizeof(int));
    for (int i = 0; i < m; ++i)
        for (int p = rowptr[i]; p < rowptr[i + 1]; ++p) tcol[tptr[col[p]] + fill[col[p]]++] = i;
    free(fill);
    int ncol = 0;
    for (int i = 0; i < m; ++i) mark[i] = -1;
    for (int i = 0; i < m; ++i) {
        /* mark[c] == i: colour c is taken by a neighbour of i */
        for (int p = rowptr[i]; p < rowptr[i + 1]; ++p)
            if (col[p] != i && col[p] < i) mark[color[col[p]]] = i;
        for (int p = tptr[i]; p < tptr[i + 1]; ++p)
            if (tcol[p] != i && tcol[p] < i) mark[color[tcol[p]]] = i;
        int c = 0;
        while (mark[c] == i) ++c;
        color[i] = c;
        if (c + 1 > ncol) ncol = c + 1;
    }
    free(tptr);
    free(tcol);
    free(mark);
    return ncol;
}
