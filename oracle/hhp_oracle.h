/*
 * hhp_oracle.h -- CPU oracle for the BiCGStab / CSR-SpMV path (TEST INFRASTRUCTURE).
 *
 * This is a plain-C restatement of HetHypPar's CPU path. It exists only to check the CUDA
 * library: tests, the smoke check and the benchmark's CPU-baseline leg may call it; the
 * product (libhhp_gpu.so and everything in hethyppar_gb300/) never links, loads or calls it.
 *
 * Each function names the reference file:line it follows (paths inside the HetHypPar tree).
 * The oracle is pinned against the reference itself: the reference's own functions, compiled
 * from its sources into oracle/_ref, produce the golden vectors under tests/golden/, and the
 * CPU test-suite checks this restatement against them bit for bit.
 *
 * Arithmetic: the file is compiled with -ffp-contract=off, so every multiply and add rounds
 * separately, in the reference's order. That is what the reference computes on x86-64 (no FMA
 * instruction is available to gcc there by default). orc_spmv_fma() is the one exception: it
 * sums each row in the same order with a fused multiply-add, which is the order the GPU
 * kernels use for rows they sum sequentially.
 */
#ifndef HHP_ORACLE_H
#define HHP_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Status codes (same meaning as the library's hhp_status values). */
#define ORC_OK 0
#define ORC_ERR_ARG 1
#define ORC_ERR_IO 2
#define ORC_ERR_FORMAT 8

/* Matrix Market coordinate file -> 0-based CSR, rows in order, entries of a row in FILE order,
 * duplicates kept. Follows readMatrixMarketFromFile (src/util/hhp_wrap_bora.c:13-104) and the
 * banner/size rules of mm_read_banner / mm_read_mtx_crd_size (src/dependencies/mmio/mmio.c:96,189).
 * Arrays are malloc'ed; free them with orc_free. Returns ORC_ERR_FORMAT for banners the reference
 * rejects (complex, array, symmetric) and for the pattern/skew/hermitian kinds it would misread. */
int orc_read_mtx(const char *path, int *m, int *n, int *nnz, int **rowptr, int **col, double **val);
void orc_free(void *p);

/* Header-less whitespace-separated doubles; reads at most `size` values into out.
 * Follows vector_read (src/util/hhp_cpu.c:411-428). Returns the number of values read. */
int orc_vector_read(const char *path, int size, double *out);
/* Writes one value per line: "%lf" like vector_write (src/util/hhp_cpu.c:430-442) when exact==0,
 * "%.17g" (round-trip exact) when exact!=0. Returns ORC_OK or ORC_ERR_IO. */
int orc_vector_write(const char *path, int size, const double *v, int exact);

/* y = A x, each row summed in CSR order, multiply then add: CSR_spmxv_seq (src/util/hhp_cpu.c:445-455). */
void orc_spmv(int m, const int *rowptr, const int *col, const double *val, const double *x, double *y);
/* Same order, each step a fused multiply-add (the GPU's order for sequentially summed rows). */
void orc_spmv_fma(int m, const int *rowptr, const int *col, const double *val, const double *x, double *y);
/* Row-parallel variant, CSR_spmxv_omp (src/util/hhp_cpu.c:459-468); per-row result identical to orc_spmv. */
void orc_spmv_omp(int m, const int *rowptr, const int *col, const double *val, const double *x, double *y,
                  int nthreads);
/* y = A^T x via the CSC accumulation of CSC_spmxv_seq_acc (src/util/hhp_cpu.c:483-491) on the
 * CSR arrays (y is overwritten, entries accumulated in CSR order). */
void orc_spmv_t(int m, int n, const int *rowptr, const int *col, const double *val, const double *x, double *y);

/* vector_dot_seq (src/util/hhp_cpu.c:84-90). */
double orc_dot(int n, const double *a, const double *b);

/* BiCGStab exactly as bicgstab_cpu.c:176-255 runs it: rho=alpha=omega=1, V=P=0, R=R0=b-A x,
 * then `niters` iterations of the fixed loop with no stop test, then the true relative residual
 * ||b-Ax||/||b|| (returned in *relres). x is updated in place (in: X_init, out: X).
 * If hist_true != NULL it receives the true relative residual after every iteration (an extra
 * SpMV per iteration that does not touch the solver state). If hist_rec != NULL it receives the
 * recursive ||R||/||R0|| after every iteration. */
int orc_bicgstab_fixed(int m, const int *rowptr, const int *col, const double *val, const double *b,
                       double *x, int niters, double *relres, double *hist_true, double *hist_rec);

/* The reference iteration count to a tolerance: the smallest k for which the fixed-k loop above
 * gives a true relative residual <= rtol (k <= maxit). The reference has no stop test of its own
 * (bicgstab_cpu.c:200), so this is what `bicgstab-cpu -n k` would need. Returns k, or -1 if
 * maxit iterations do not reach rtol. x ends at iteration k (or maxit), *relres is its residual. */
int orc_bicgstab_iters_to_tol(int m, const int *rowptr, const int *col, const double *val,
                              const double *b, double *x, double rtol, int maxit, double *relres);

/* The MPI CPU-rank form of the same loop (src/entry/bicgstab_mpi.c:256-300) with the ranks as
 * threads: each of `nthreads` threads owns a contiguous block of rows, every dot product is the
 * sum of per-block partials in block order (the MPI_Allreduce of MPI_vector_dot,
 * src/util/hhp_cpu.c:192-197), and the SpMV is row-sequential per block. Fixed `niters`
 * iterations; returns the true relative residual in *relres. */
int orc_bicgstab_fixed_mt(int m, const int *rowptr, const int *col, const double *val, const double *b,
                          double *x, int niters, int nthreads, double *relres);

/* CSR -> CSC (= CSR of A^T): count, prefix sum, scatter in row order, as CSR_to_CSC
 * (src/util/hhp_matrix.c:1476-1535). Output arrays are caller-allocated (n+1, nnz, nnz). */
void orc_csr_to_csc(int m, int n, int nnz, const int *rowptr, const int *col, const double *val,
                    int *colptr, int *rowidx, double *tval);

/* out[i,:] = A[perm[i], :] with columns renumbered by perm_inv: csr_permute
 * (src/util/hhp_dp_helpers.c:18-37). Output arrays caller-allocated (m+1, nnz, nnz). */
void orc_csr_permute(int m, int nnz, const int *rowptr, const int *col, const double *val,
                     const int *perm, const int *perm_inv, int *orowptr, int *ocol, double *oval);

/* ---- ILU(0) --------------------------------------------------------------------------------
 * The preconditioner of the SpSV path of gpu_BiCGStab (src/entry/bicgstab_gpu.c:185-201 and
 * 238-254, commented out there; cuSPARSE's csrilu02 and SpSV would supply the factorization and
 * the triangular solves, neither of which is part of the reference's own sources). Restated from
 * the published algorithm: ILU(0) in its IKJ form (Saad, Iterative Methods for Sparse Linear
 * Systems, 2nd ed., Algorithm 10.4), M = L U with L unit lower and U upper on A's pattern.
 * No reference output exists to pin these against; the tests pin them by the defining property
 * of ILU(0), (L U)_ij = a_ij on the pattern, and by the closed form of the 5-point stencil. */

/* Factors A in place of a copy: lu (nnz) receives L's multipliers below the diagonal and U on
 * and above it, in A's CSR order. Row by row, for each k < i with a_ik stored, in ascending k:
 * l_ik = a_ik / u_kk, then a_ij = fma(-l_ik, u_kj, a_ij) for every j > k stored in both rows i
 * and k. Needs square A, every row's columns strictly ascending and every diagonal stored
 * (ORC_ERR_ARG otherwise). A zero or non-finite pivot u_ii returns ORC_ERR_FORMAT with the first
 * such row in *bad_row. */
int orc_ilu0(int m, const int *rowptr, const int *col, const double *val, double *lu, int *bad_row);

/* Rows of one triangle with more than ORC_ILU_LONG stored entries are summed as the GPU's
 * warp-wide path sums them, rows with more than ORC_ILU_BIG as its block-wide path (blocks of
 * ORC_ILU_BLOCK threads) does (below); shorter rows sequentially. */
#define ORC_ILU_LONG 64
#define ORC_ILU_BIG 2048
#define ORC_ILU_BLOCK 1024

/* z = U^-1 L^-1 r. Forward, rows ascending: z_i = r_i - sum_{k<i} l_ik z_k; backward, rows
 * descending: z_i = (z_i - sum_{j>i} u_ij z_j) * d_i with d_i = 1 / u_ii rounded once (the GPU
 * stores these reciprocals). A row whose triangle part has at most
 * ORC_ILU_LONG entries is summed in ascending column order as acc = fma(-v, z, acc) starting from
 * the right-hand value; a longer row accumulates 32 partial sums (entry e into slot e mod 32,
 * acc = fma(v, z, acc) from 0), adds them by a butterfly (at distances 16, 8, 4, 2, 1 every slot
 * adds its partner) and subtracts slot 0 from the right-hand value; a row above ORC_ILU_BIG
 * accumulates ORC_ILU_BLOCK partial sums the same way, reduces each group of 32 by the butterfly
 * and adds the group sums in group order from 0. These are the GPU's orders, so results agree bit
 * for bit. */
void orc_ilu0_apply(int m, const int *rowptr, const int *col, const double *lu, const double *r, double *z);

/* Right-preconditioned BiCGStab with M = ILU(0) of A, the loop of bicgstab_gpu.c:155-290 with
 * its preconditioning steps 9 and 14 in place: p^ = M^-1 p, v = A p^, x += alpha p^,
 * s^ = M^-1 s, t = A s^, x += omega s^. Returns the first iteration whose true relative residual
 * ||b - A x|| / ||b|| is <= rtol (-1 if maxit iterations do not reach it, -2 on an ILU error);
 * x is updated in place and *relres receives its residual. */
int orc_bicgstab_ilu0_iters_to_tol(int m, const int *rowptr, const int *col, const double *val,
                                   const double *b, double *x, double rtol, int maxit, double *relres);

/* Greedy multicolouring of the pattern of A + A^T: rows in ascending order take the smallest
 * colour none of their coloured neighbours has. color[m] receives the colours; returns their
 * number. */
int orc_color(int m, const int *rowptr, const int *col, int *color);

#ifdef __cplusplus
}
#endif
#endif
