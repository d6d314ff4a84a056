/*
 * hhp_gpu.h -- C ABI of libhhp_gpu.so: GB300 (sm_103a) BiCGStab and CSR SpMV.
 *
 * A drop-in for the single-GPU solver path of HetHypPar. Every entry point takes plain pointers
 * and sizes. Each declaration names the reference interface it replaces (paths inside the
 * HetHypPar tree). Functions with a `_dev` suffix take caller-owned DEVICE pointers and run on
 * the context's stream; the others take caller-owned HOST pointers and copy in and out.
 *
 * Conventions
 *  - Every function returns an hhp_status (never exits the process); hhp_status_str() names it,
 *    hhp_last_error() gives a one-line description of the most recent failure on this thread.
 *  - An hhp_ctx owns one CUDA stream on one device; calls on a context are serialised on that
 *    stream. Use one context per host thread.
 *  - An hhp_mat owns its device CSR arrays (int32 indices, FP64 values) and everything derived
 *    from them (the SpMV work plan, an FP32 copy of the values, the transpose), built lazily.
 *  - Sizes are int (the reference's CSR uses int m, n, nnz: src/include/hhp_common.h:43-50).
 */
#ifndef HHP_GPU_H
#define HHP_GPU_H

#ifdef __cplusplus
extern "C" {
#endif

typedef struct hhp_ctx hhp_ctx;
typedef struct hhp_mat hhp_mat;

typedef enum {
    HHP_OK = 0,
    HHP_ERR_ARG = 1,       /* invalid argument (null pointer, bad size, non-square for a solve) */
    HHP_ERR_IO = 2,        /* file could not be opened / read / written, or is short            */
    HHP_ERR_CUDA = 3,      /* a CUDA runtime call failed                                        */
    HHP_ERR_OOM = 4,       /* device or host allocation failed                                  */
    HHP_ERR_BREAKDOWN = 5, /* BiCGStab breakdown: rho, (r0,v) or (t,t) zero or not finite       */
    HHP_ERR_MAXIT = 6,     /* maxit reached before the tolerance                                */
    HHP_ERR_TIMEOUT = 7,   /* a bounded device wait gave up                                     */
    HHP_ERR_FORMAT = 8,    /* Matrix Market banner/size/entry not supported or malformed        */
    HHP_ERR_STATE = 9      /* call not valid in the object's current state                      */
} hhp_status;

/* Per-iteration residual callback: iter is 1-based, rel_res is the recursive ||r_k|| / ||b||.
 * Called on the calling thread after the device loop, in iteration order (every `print_every`-th
 * iteration when print_every > 0). Replaces the "Iteration = %d; Error Norm = %e" lines of
 * gpu_BiCGStab (src/entry/bicgstab_gpu.c:156). */
typedef void (*hhp_iter_cb)(int iter, double rel_res, void *user);

typedef enum { HHP_PREC_FP64 = 0, HHP_PREC_MIXED = 1 } hhp_precision;

/* Preconditioner. JACOBI: right preconditioning with M = diag(A) (the diagonal form of the ILU path
 * left commented out in gpu_BiCGStab, src/entry/bicgstab_gpu.c:185-201, 238-254): BiCGStab runs on
 * A M^-1 (a column-scaled copy of A built once per matrix) and x = M^-1 y; the stop test and the
 * reported residual are those of A x = b. JACOBI_ROW: left preconditioning with the same M (row
 * equilibration, for matrices whose rows differ in scale by orders of magnitude): BiCGStab runs on
 * M^-1 A x = M^-1 b (a row-scaled copy of A), and after each pass the residual of A x = b itself is
 * checked; while it is above rtol the scaled solve continues from x with a tolerance tightened by
 * the shortfall, so the reported residual and the status are those of A x = b (iters counts the
 * scaled solve's iterations, outer_iters its passes; the callback sees the scaled residual). Both
 * need a nonzero diagonal (HHP_ERR_ARG otherwise). ILU0: right preconditioning with M = L U, the
 * ILU(0) factorization of A in its stored order -- the SpSV path itself (steps 9 and 14 of
 * gpu_BiCGStab: p^ = M^-1 p, v = A p^, x += alpha p^; s^ = M^-1 s, t = A s^, x += omega s^). The
 * factors are built on the device on first use (and again after hhp_mat_set_values); each
 * application is two triangular solves walking the dependency levels of L and U, so its cost
 * grows with their number: reorder a stencil-like matrix with hhp_reorder_color first (two levels
 * for the 5- and 7-point stencils) -- the natural order of an N x N grid has 2N - 1. FP64 only
 * (HHP_ERR_ARG with the mixed form); either loop schedule. Rows may store their entries in any
 * column order (each is factored and solved in ascending column order); every diagonal must be
 * stored and no column twice in a row (HHP_ERR_ARG), and the pivots u_ii must be nonzero
 * (HHP_ERR_BREAKDOWN). */
typedef enum {
    HHP_PRECOND_NONE = 0,
    HHP_PRECOND_JACOBI = 1,
    HHP_PRECOND_JACOBI_ROW = 2,
    HHP_PRECOND_ILU0 = 3
} hhp_precond;

/* FP64 iteration schedule. MERGED: the stop tests and beta come from the dot products of the
 * t = A s step (||r_new||^2 = s.s - omega t.s, r0.r_new = r0.s - omega r0.t), so one iteration is
 * 4 kernels (two SpMVs and two fused vector kernels) instead of 5. CLASSIC: the reference's order
 * (src/entry/bicgstab_gpu_dp.c:165-196): rho_new = r.r0 and ||r|| as direct dot products of the
 * new residual. AUTO (0, the default): MERGED for hhp_bicgstab*, CLASSIC for the adjoint solve of
 * hhp_bicgstab_backward* (whose tolerances sit near the rounding floor, where the direct dot
 * products reach a lower true residual). Fixed-iteration runs always use CLASSIC. ILU(0) adds its
 * two applications to either schedule (MERGED: 8 kernels per iteration, CLASSIC: 9). The FP32
 * inner loop of the mixed form follows the same choice (MERGED: its kernel with the x and r
 * updates also takes the reliable-update test). */
typedef enum { HHP_LOOP_AUTO = 0, HHP_LOOP_MERGED = 1, HHP_LOOP_CLASSIC = 2 } hhp_loop;

typedef struct {
    double rtol;        /* stop when ||b - A x|| <= rtol * ||b|| (the relative residual the reference
                           prints, bicgstab_cpu.c:251-255; equal to gpu_BiCGStab's threshold
                           tol * ||r0||, bicgstab_gpu.c:149-150, when x0 = 0)                   */
    int maxit;          /* iteration cap (maxIterations, bicgstab_gpu.c:120); >= 0                */
    int precision;      /* hhp_precision                                                          */
    double inner_rtol;  /* mixed form: the FP32 recurrences run until their residual has dropped by
                           this factor since the last FP64 refinement step x += d,
                           r = b - A x (<= 0: 0.05 for solves, 0.1 for the adjoint entry points,
                           whose tolerances sit near the FP64 rounding floor)                    */
    int max_outer;      /* FP64 form: cap on residual-replacement restarts (<= 0: 50)            */
    int fixed_iters;    /* 1: run exactly maxit iterations with no stop test, like the reference's
                           executables (src/entry/bicgstab_cpu.c:200); FP64 only                  */
    int print_every;    /* callback stride; 0 = no callback                                       */
    hhp_iter_cb cb;
    void *user;
    int precond;        /* hhp_precond (forward solves; the adjoint runs unpreconditioned)        */
    int loop;           /* hhp_loop                                                               */
} hhp_solve_opts;

typedef struct {
    int iters;                 /* BiCGStab iterations (mixed: total inner iterations)            */
    int outer_iters;           /* mixed: FP64 refinement steps; FP64: graph passes (restarts + 1) */
    int half_step;             /* 1 if the last iteration stopped at the ||s|| test              */
    double rel_res_true;       /* ||b - A x|| / ||b||, recomputed in FP64 after the solve         */
    double rel_res_recursive;  /* the solver's own ||r_k|| / ||b||                                */
    double err_vs_target;      /* max_i |x_i - x_target_i| (NaN when no target was given)        */
    double t_solve_s;          /* device time of the solve (CUDA events on the context stream)   */
    hhp_status status;
    int fp64_fallback;         /* mixed: 1 if the FP32 recurrences kept breaking down or diverging
                                  and the solve was finished in FP64 from the last FP64 iterate  */
} hhp_solve_info;

/* ---- errors -------------------------------------------------------------------------------- */
const char *hhp_status_str(hhp_status s);
const char *hhp_last_error(void);

/* ---- context: replaces cudaSetDevice + cusparseCreate/cublasCreate of the entries
 *      (src/entry/bicgstab_gpu_dp.c:97-99) --------------------------------------------------- */
hhp_status hhp_ctx_create(int device, hhp_ctx **out);
/* Destroy every hhp_mat created on the context before destroying the context. */
void hhp_ctx_destroy(hhp_ctx *ctx);
/* The context's cudaStream_t, as an opaque pointer. */
void *hhp_ctx_stream(hhp_ctx *ctx);
hhp_status hhp_ctx_sync(hhp_ctx *ctx);
/* Number of kernels this context has launched (graph launches count their kernel nodes). */
long long hhp_ctx_kernel_launches(const hhp_ctx *ctx);
/* No counterpart in the reference: the device's FP64 fused multiply-add throughput (lane FMAs per
 * second), measured by a short probe kernel on the context's stream (synchronises it). The FP64
 * SpMV and vector kernels are bound by this rate as much as by HBM on GB300; it is the denominator
 * of their FP64 floor. */
hhp_status hhp_ctx_fp64_fma_rate(hhp_ctx *ctx, double *fma_per_s);

/* ---- matrices: replace device_csr_create / device_csr_destroy (src/util/hhp_cuda.c:19-51,
 *      src/include/hhp_cuda.h:46-47) and buReadSparseMatrix (src/util/hhp_matrix.c:116) -------- */
/* Host CSR (0-based, int32), copied to the device. Entries of a row are used in the given order.
 * perm (nullable, length m, a permutation of 0..m-1; needs m == n) reorders the matrix as
 * csr_permute does (src/util/hhp_dp_helpers.c:18-37): row i of the result is row perm[i] of A
 * and column j becomes perm_inv[j]. */
hhp_status hhp_mat_from_csr(hhp_ctx *ctx, int m, int n, int nnz, const int *rowptr, const int *col,
                            const double *val, const int *perm, hhp_mat **out);
/* Same, from device arrays (copied; the caller keeps ownership). */
hhp_status hhp_mat_from_csr_dev(hhp_ctx *ctx, int m, int n, int nnz, const int *rowptr_dev, const int *col_dev,
                                const double *val_dev, hhp_mat **out);
/* Matrix Market coordinate real/integer general file (readMatrixMarketFromFile,
 * src/util/hhp_wrap_bora.c:13-104): rows in order, entries of a row in file order. Large files
 * are parsed by all host cores (same result as a serial parse). A binary CSR file written by
 * hhp_csr_file_write is accepted at the same path argument and loaded without text parsing. */
hhp_status hhp_mat_from_mtx(hhp_ctx *ctx, const char *path, hhp_mat **out);
void hhp_mat_destroy(hhp_mat *mat);
hhp_status hhp_mat_shape(const hhp_mat *mat, int *m, int *n, int *nnz);
/* Replace the values (same pattern) from host or device memory; derived copies are refreshed. */
hhp_status hhp_mat_set_values(hhp_mat *mat, const double *val);
hhp_status hhp_mat_set_values_dev(hhp_mat *mat, const double *val_dev);
/* Copy the device CSR back to host arrays (m+1, nnz, nnz; any may be NULL). */
hhp_status hhp_mat_get_csr(const hhp_mat *mat, int *rowptr, int *col, double *val);
/* Solve-only matrices: builds the FP64 SpMV layout (and the FP32 one when keep_fp32 != 0, for the
 * mixed form), then frees the canonical CSR's column and value arrays (12 bytes per nonzero) and
 * the FP32 value copy, keeping the sliced copies the SpMV reads. Afterwards the matrix still
 * serves SpMV and solves (FP64; mixed if keep_fp32) and everything built before the call (the
 * transpose, Jacobi scaling, ILU(0) factors, which keep the column array: 4 bytes per nonzero);
 * whatever needs the CSR later -- new values,
 * hhp_mat_get_csr, a first transpose, dL/dA, a first preconditioner, a layout not built --
 * returns HHP_ERR_STATE. HHP_ERR_ARG when rows longer than the slice limit exist (their chunks
 * are read from the CSR). Idempotent. */
hhp_status hhp_mat_drop_csr(hhp_mat *mat, int keep_fp32);
/* Host CSR of A^T built on the device (a stable radix sort of A's entries by column; within a row
 * of A^T entries are in increasing row order of A, as CSR_to_CSC src/util/hhp_matrix.c:1476-1535).
 * Arrays n+1, nnz, nnz. */
hhp_status hhp_mat_get_transpose(hhp_mat *mat, int *t_rowptr, int *t_col, double *t_val);

/* ---- SpMV: replaces device_csr_spmv (src/util/hhp_cuda.c:226-236): y = alpha*A*x + beta*y ---- */
hhp_status hhp_spmv_dev(hhp_ctx *ctx, hhp_mat *mat, double alpha, const double *x_dev, double beta, double *y_dev);
/* FP32 values (a rounded copy of A) and FP32 vectors, FP32 accumulation. */
hhp_status hhp_spmv_f32_dev(hhp_ctx *ctx, hhp_mat *mat, const float *x_dev, float *y_dev);
/* y = A^T x on the device-built transpose. */
hhp_status hhp_spmv_t_dev(hhp_ctx *ctx, hhp_mat *mat, const double *x_dev, double *y_dev);
/* Host-buffer SpMV, y = A x (copies in and out; the spmv-gpu path, src/entry/spmv_gpu.c:100-130). */
hhp_status hhp_spmv(hhp_ctx *ctx, hhp_mat *mat, const double *x, double *y);

/* ---- BiCGStab: replaces gpu_BiCGStab (src/entry/bicgstab_gpu.c:106-310) and the loop of
 *      bicgstab-gpu-dp (src/entry/bicgstab_gpu_dp.c:123-208) ---------------------------------- */
/* Host pointers: b (m), x (n; in: X_init, out: X), x_target (nullable). opts NULL = defaults
 * (rtol 1e-10, maxit 2000, FP64). info may be NULL. Returns HHP_OK when the true relative
 * residual reached rtol, HHP_ERR_MAXIT / HHP_ERR_BREAKDOWN otherwise (x holds the last iterate). */
hhp_status hhp_bicgstab(hhp_ctx *ctx, hhp_mat *mat, const double *b, double *x, const double *x_target,
                        const hhp_solve_opts *opts, hhp_solve_info *info);
/* Device pointers, same semantics. */
hhp_status hhp_bicgstab_dev(hhp_ctx *ctx, hhp_mat *mat, const double *b_dev, double *x_dev,
                            const double *x_target_dev, const hhp_solve_opts *opts, hhp_solve_info *info);

/* ---- adjoint (no reference counterpart): given x = A^-1 b and g = dL/dx, solve A^T lambda = g
 *      with the same BiCGStab on the transpose, then dL/db = lambda and
 *      dL/dA_ij = -lambda_i * x_j over A's sparsity pattern (one value per stored entry). ------- */
hhp_status hhp_bicgstab_backward_dev(hhp_ctx *ctx, hhp_mat *mat, const double *x_dev, const double *dldx_dev,
                                     double *dldb_dev, double *dlda_vals_dev, const hhp_solve_opts *opts,
                                     hhp_solve_info *info);
hhp_status hhp_bicgstab_backward(hhp_ctx *ctx, hhp_mat *mat, const double *x, const double *dldx, double *dldb,
                                 double *dlda_vals, const hhp_solve_opts *opts, hhp_solve_info *info);

/* ---- vector files: vector_read / vector_write (src/util/hhp_cpu.c:411-442) ------------------- */
/* Reads exactly `size` whitespace-separated doubles; HHP_ERR_IO if the file is missing or short. */
hhp_status hhp_vector_read(const char *path, int size, double *out);
/* exact = 0: "%lf" (6 decimals, as the reference); exact = 1: "%.17g" (round-trip). */
hhp_status hhp_vector_write(const char *path, int size, const double *v, int exact);

/* Host-only Matrix Market read (no device needed), same rules as hhp_mat_from_mtx. The arrays
 * are allocated with malloc (m+1, nnz, nnz); release each with hhp_free. */
hhp_status hhp_mtx_read(const char *path, int *m, int *n, int *nnz, int **rowptr, int **col, double **val);
void hhp_free(void *p);
/* Binary CSR file for fast re-reads (the reference re-parses text on every run,
 * src/util/hhp_wrap_bora.c:13-104): "HHPCSR01", int64 m, n, nnz, int32 rowptr[m+1], int32
 * col[nnz], FP64 val[nnz], little-endian. Read back by hhp_mtx_read / hhp_mat_from_mtx. */
hhp_status hhp_csr_file_write(const char *path, int m, int n, int nnz, const int *rowptr, const int *col,
                              const double *val);

/* ---- BLAS-1 on device vectors: replace device_vector_dot / _scale / _axpy / _GPUtoGPU
 *      (src/util/hhp_cuda.c:163-202, cuBLAS Ddot/Dscal/Daxpy and a D2D copy) and the
 *      device-pointer-mode cublasDdot of the dp loop (src/entry/bicgstab_gpu_dp.c:163-190) ------ */
/* sum_i x[i] y[i] into device memory, asynchronously on the context's stream (cublasDdot with
 * CUBLAS_POINTER_MODE_DEVICE). Deterministic: the same inputs give the same bits on every call. */
hhp_status hhp_dot_dev(hhp_ctx *ctx, int n, const double *x_dev, const double *y_dev, double *result_dev);
/* The same, result to host memory; synchronises the stream (cublasDdot with a host pointer). */
hhp_status hhp_dot(hhp_ctx *ctx, int n, const double *x_dev, const double *y_dev, double *result);
/* y += alpha x (cublasDaxpy), x *= alpha (cublasDscal), dst = src (device_vector_GPUtoGPU). */
hhp_status hhp_axpy_dev(hhp_ctx *ctx, int n, double alpha, const double *x_dev, double *y_dev);
hhp_status hhp_scal_dev(hhp_ctx *ctx, int n, double alpha, double *x_dev);
hhp_status hhp_copy_dev(hhp_ctx *ctx, int n, const double *src_dev, double *dst_dev);

/* ---- locality reordering ------------------------------------------------------------------ */
/* Reverse Cuthill-McKee order of the symmetrised pattern A + A^T of a square CSR (host only, no
 * device needed): perm[m] in csr_permute's convention (src/util/hhp_dp_helpers.c:18-37), ready for
 * hhp_mat_from_csr's perm argument. Replaces the offline PaToH partition files the reference
 * orders rows by (src/entry/bicgstab_hybrid_dist_dp.c:217-233) when none is at hand. Deterministic;
 * HHP_ERR_ARG for a malformed CSR. */
hhp_status hhp_reorder_rcm(int m, const int *rowptr, const int *col, int *perm);

/* Multicolour order for ILU(0): a greedy colouring of the pattern of A + A^T (rows in ascending
 * order take the smallest colour none of their coloured neighbours has), rows then grouped by
 * colour, ascending inside a colour. perm[m] in csr_permute's convention; *n_colors (nullable)
 * receives the number of colours, which bounds the dependency levels of the reordered matrix's
 * triangles. Host only; HHP_ERR_ARG for a malformed or non-square CSR. */
hhp_status hhp_reorder_color(int m, const int *rowptr, const int *col, int *perm, int *n_colors);

/* ---- ILU(0) factors (the csrilu02 and SpSV steps of the same path) ------------------------------ */
/* Builds the ILU(0) factors of A on the device if they do not exist yet (as a solve with
 * HHP_PRECOND_ILU0 would). lu (nullable, host, nnz doubles) receives them in A's CSR order: L's
 * multipliers below the diagonal (L has a unit diagonal), U on and above it. levels (nullable,
 * 2 ints) receives the dependency levels of L and of U. */
hhp_status hhp_ilu0_factor(hhp_ctx *ctx, hhp_mat *A, double *lu, int *levels);
/* z = U^-1 L^-1 r for device vectors of length m (z may be r), factoring A first if needed.
 * Ordered on the context's stream; returns after the work is queued. */
hhp_status hhp_ilu0_apply_dev(hhp_ctx *ctx, hhp_mat *A, const double *r_dev, double *z_dev);

/* ---- host-side helpers exposed for testing the work plan without a GPU ---------------------- */
/* The SpMV work plan of a host CSR (rows_per_lane 2 = the FP64 kernel's slices of 64 rows, 4 =
 * the FP32 kernel's slices of 128 rows): number of slices, of long rows (cut into chunks of at
 * most `cap` nonzeros) and chunks, whether rows were length-sorted inside windows, and the
 * storage padding ratio of the slices. */
hhp_status hhp_plan_stats(int m, int nnz, const int *rowptr, int rows_per_lane, int cap, int *n_slices,
                          int *n_long_rows, int *n_chunks, int *sorted, double *padding);
/* The plan itself: slice_rows receives, for every slice position (n_slices * 32 * rows_per_lane
 * ints), the row placed there (-1 = padding); chunks receives 4 ints per chunk (row, chunk id,
 * first nonzero, end). capacity counts both arrays' ints. *n_slices and *n_chunks are always set;
 * HHP_ERR_ARG if capacity is too small. */
hhp_status hhp_plan_dump(int m, int nnz, const int *rowptr, int rows_per_lane, int cap, int capacity,
                         int *slice_rows, int *chunks, int *n_slices, int *n_chunks);

/* ---- drop-ins for the reference's device-pointer launchers (src/include/hhp_dp_kernels.h:37-59).
 *      Same names, arguments and meaning; `s` is a cudaStream_t. Unlike the reference's
 *      one-thread kernels, the scalar updates here are single-thread kernels too (there is no
 *      work to spread), and the vector ops use 128-bit loads. ---------------------------------- */
void hhp_dp_vecop_P(double *P, const double *V, const double *R, const double *omega, const double *beta, int n,
                    void *s);
void hhp_dp_vecop_S(double *S, const double *R, const double *V, const double *neg_alpha, int n, void *s);
void hhp_dp_vecop_XR(double *X, double *R, const double *P, const double *S, const double *T,
                     const double *alpha, const double *omega, const double *neg_omega, int n, void *s);
void hhp_dp_update_beta(double *beta, double *rho_old, const double *rho_new, const double *alpha,
                        const double *omega, void *s);
void hhp_dp_update_alpha(double *alpha, double *neg_alpha, const double *rho, const double *rv, void *s);
void hhp_dp_update_omega(double *omega, double *neg_omega, const double *ts, const double *tt, void *s);

/* ---- allocation-free SpMV (no counterpart in the reference) -------------------------------------
 * y = alpha*A*x + beta*y straight from caller-owned device CSR arrays (rowptr m+1, col nnz, val nnz
 * FP64; x n, y m), with no context, no matrix object and no device allocation. For callers that
 * must not call cudaMalloc: a host application that owns and pre-sizes all device memory, or code
 * between stream operations where cudaMalloc's implicit device synchronisation is not allowed.
 * Work is split evenly over rows plus nonzeros; the only scratch, one partial sum per CTA for rows
 * split between CTAs, is a 48 KB array built into the library (held on every GPU that loads it).
 * Limit: m + nnz <= 2^28, else HHP_ERR_ARG. Runs on `stream` (a cudaStream_t; NULL = default
 * stream) of the current device. The first call on a device looks up the scratch array's address
 * there: make it before any stream capture. Calls share that array, so calls that overlap on one
 * GPU race and give wrong results; serialise them. Rows split between CTAs are summed in another
 * order than hhp_spmv_dev, so results agree to rounding, not bit for bit.
 * Preconditions, NOT checked (checking them would need a device-to-host copy): rowptr[0] == 0,
 * rowptr[m] == nnz, rowptr non-decreasing, and 0 <= col[k] < n for every k. A CSR that breaks
 * them gives wrong results (a row past the end is never finished) or out-of-range reads. */
hhp_status hhp_spmv_csr_noalloc(int m, int n, int nnz, const int *rowptr_dev, const int *col_dev,
                                const double *val_dev, double alpha, const double *x_dev, double beta,
                                double *y_dev, void *stream);

#ifdef __cplusplus
}
#endif
#endif /* HHP_GPU_H */
