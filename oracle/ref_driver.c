/*
 * ref_driver.c -- in-process access to the reference's own CPU functions (TEST INFRASTRUCTURE).
 *
 * Linked with the reference's unmodified sources (src/util/hhp_cpu.c, hhp_matrix.c,
 * hhp_wrap_bora.c, hhp_dp_helpers.c, mmio, bora matrix.c) into oracle/_ref/libhhpref.so by
 * oracle/Makefile. tests/golden/make_golden.py calls these wrappers through ctypes to record the
 * reference's results at full double precision (its executables print only %E and %lf).
 * Every numerical step below is a call into the reference; this file only marshals arrays.
 */
#include <math.h>
#include <stdlib.h>
#include <string.h>

#include "hhp_common.h"
#include "hhp_cpu.h"
#include "hhp_dp_helpers.h"
#include "hhp_matrix.h"

#define EXPORT __attribute__((visibility("default")))

static CSR make_csr(int m, int n, int nnz, int *I, int *J, double *val) {
    CSR a;
    a.I = I; a.J = J; a.val = val; a.nnz = nnz; a.m = m; a.n = n;
    return a;
}

/* buReadSparseMatrix (src/util/hhp_matrix.c:116). Arrays belong to the reference's allocator;
 * release them with refd_free. */
EXPORT int refd_read(char *path, int *m, int *n, int *nnz, int **I, int **J, double **val) {
    CSR a = buReadSparseMatrix(path);
    *m = a.m; *n = a.n; *nnz = a.nnz; *I = a.I; *J = a.J; *val = a.val;
    return 0;
}

EXPORT void refd_free(void *p) { free(p); }

/* CSR_spmxv_seq (src/util/hhp_cpu.c:445). */
EXPORT void refd_spmv(int m, int n, int nnz, int *I, int *J, double *val, double *x, double *y) {
    CSR a = make_csr(m, n, nnz, I, J, val);
    Vector X = {x, (unsigned)n}, Y = {y, (unsigned)m};
    CSR_spmxv_seq(a, X, Y);
}

/* vector_dot_seq (src/util/hhp_cpu.c:84). */
EXPORT double refd_dot(int n, double *a, double *b) {
    Vector A = {a, (unsigned)n}, B = {b, (unsigned)n};
    return vector_dot_seq(A, B);
}

/* The body of src/entry/bicgstab_cpu.c:172-255, call for call, on caller arrays.
 * x: in X_init, out X after niters iterations; returns the true relative residual. */
EXPORT double refd_bicgstab(int m, int n, int nnz, int *I, int *J, double *val, double *b, double *x, int niters) {
    CSR A = make_csr(m, n, nnz, I, J, val);
    Vector X = {x, (unsigned)n};
    Vector B = {b, (unsigned)m};
    Vector Y = vector_init_const(A.m, 0);
    double rho = 1.0, alpha = 1.0, omega = 1.0;
    Vector V = vector_init_const(Y.nvals, 0);
    Vector P = vector_init_const(Y.nvals, 0);
    Vector R = vector_init_clone(B);
    CSR_spmxv_seq(A, X, Y);
    vector_sub_seq(R, Y, R);
    vector_zero(Y);
    Vector R_0 = vector_init_clone(R);
    Vector S = vector_init(Y.nvals);
    Vector T = vector_init(Y.nvals);
    for (int i = 0; i < niters; i++) {
        double temp_rho = vector_dot_seq(R, R_0);
        double beta = (temp_rho / rho) * (alpha / omega);
        rho = temp_rho;
        vector_scale_seq(V, omega, V);
        vector_sub_seq(P, V, P);
        vector_scale_seq(P, beta, P);
        vector_add_seq(P, R, P);
        CSR_spmxv_seq(A, P, V);
        alpha = rho / vector_dot_seq(R_0, V);
        vector_scale_seq(V, alpha, S);
        vector_sub_seq(R, S, S);
        CSR_spmxv_seq(A, S, T);
        omega = vector_dot_seq(T, S) / vector_dot_seq(T, T);
        vector_scale_seq(P, alpha, Y);
        vector_add_seq(X, Y, X);
        vector_scale_seq(S, omega, Y);
        vector_add_seq(X, Y, X);
        vector_scale_seq(T, omega, R);
        vector_sub_seq(S, R, R);
    }
    CSR_spmxv_seq(A, X, Y);
    vector_sub_seq(B, Y, Y);
    double sy = vector_dot_seq(Y, Y);
    double sb = vector_dot_seq(B, B);
    vector_destroy(&Y); vector_destroy(&P); vector_destroy(&S); vector_destroy(&V);
    vector_destroy(&R); vector_destroy(&R_0); vector_destroy(&T);
    return sqrt(sy / sb);
}

/* CSR_to_CSC (src/util/hhp_matrix.c:1476); outputs copied into caller arrays. */
EXPORT void refd_csr_to_csc(int m, int n, int nnz, int *I, int *J, double *val, int *colptr, int *rowidx, double *tval) {
    CSR a = make_csr(m, n, nnz, I, J, val);
    CSC c = CSR_to_CSC(a);
    memcpy(colptr, c.I, sizeof(int) * ((size_t)n + 1));
    memcpy(rowidx, c.J, sizeof(int) * (size_t)nnz);
    memcpy(tval, c.val, sizeof(double) * (size_t)nnz);
    free(c.I); free(c.J); free(c.val);
}

/* csr_permute (src/util/hhp_dp_helpers.c:18). */
EXPORT void refd_csr_permute(int m, int n, int nnz, int *I, int *J, double *val, int *perm, int *perm_inv, int *oI, int *oJ,
                      double *oval) {
    CSR a = make_csr(m, n, nnz, I, J, val);
    CSR o = csr_permute(a, perm, perm_inv);
    memcpy(oI, o.I, sizeof(int) * ((size_t)m + 1));
    memcpy(oJ, o.J, sizeof(int) * (size_t)nnz);
    memcpy(oval, o.val, sizeof(double) * (size_t)nnz);
    free(o.I); free(o.J); free(o.val);
}
