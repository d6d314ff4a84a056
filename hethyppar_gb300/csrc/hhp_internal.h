// hhp_internal.h -- host-side structures shared by the translation units of libhhp_gpu.so.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>
#include <exception>
#include <new>
#include <cstdio>
#include <string>
#include <vector>

#include "hhp_gpu.h"

namespace hhp {

// ---- error plumbing ----------------------------------------------------------------------------
void set_error(const char *fmt, ...);
hhp_status cuda_fail(cudaError_t e, const char *what, const char *file, int line);

// No C++ exception crosses the C ABI: every entry point that allocates host memory or starts
// threads runs its body inside HHP_API_BEGIN / HHP_API_END, which turn an exception into a status
// (std::bad_alloc -> HHP_ERR_OOM, anything else -> HHP_ERR_STATE) with the message recorded.
inline hhp_status api_exception() {
    try {
        throw;
    } catch (const std::bad_alloc &) {
        set_error("out of host memory");
        return HHP_ERR_OOM;
    } catch (const std::exception &e) {
        set_error("internal error: %s", e.what());
        return HHP_ERR_STATE;
    } catch (...) {
        set_error("internal error");
        return HHP_ERR_STATE;
    }
}
#define HHP_API_BEGIN try {
#define HHP_API_END                          \
    }                                        \
    catch (...) {                            \
        return ::hhp::api_exception();       \
    }

#define HHP_CUDA(call)                                                          \
    do {                                                                        \
        cudaError_t _e = (call);                                                \
        if (_e != cudaSuccess) return ::hhp::cuda_fail(_e, #call, __FILE__, __LINE__); \
    } while (0)
#define HHP_TRY(call)                          \
    do {                                       \
        hhp_status _s = (call);                \
        if (_s != HHP_OK) return _s;           \
    } while (0)

// ---- SpMV work plan ----------------------------------------------------------------------------
// Sliced, row-interleaved layout (see hhp_plan.cpp). Positions p = s*H + q (slice s, row q of the
// slice) map to original rows pos_row[p] (-1 for padding). The j-th nonzero of position p is at
// slice_ptr[s] + j*H + q in the slice arrays. Rows longer than long_thr are cut into chunks
// {row, chunk id, k0, k1} read straight from the CSR arrays.
struct SellHost {
    int rpl = 2, H = 64, long_thr = 0, cap = 0, n_slices = 0;
    bool sorted = false, has_perm = false;
    std::vector<int> pos_row, pos_len;   // n_slices * H
    std::vector<long long> slice_ptr;    // n_slices + 1
    long long total = 0, short_nnz = 0;  // slice storage (with padding), nonzeros in slices
    double padding = 1.0;                // total / short_nnz
    std::vector<int4> chunks;            // long-row chunks
    std::vector<int> long_rows, long_first, chunk_long;
};

// Builds the plan from a host rowptr: rpl rows per lane (H = 32*rpl rows per slice), rows longer
// than long_thr go to chunks of at most cap nonzeros, `window` rows per length-sort window.
void build_plan(int m, const int *rowptr, int rpl, int long_thr, int cap, int window, SellHost &out);
// Deals the plan's units (slices, then chunks) to n_warps warps, balancing their step counts;
// warp w processes warp_units[warp_ptr[w] .. warp_ptr[w+1]) in ascending order.
void assign_units(const SellHost &P, int n_warps, std::vector<int> &warp_ptr, std::vector<int> &warp_units,
                  double *imbalance);

// Uniform diagonals (hhp_plan.cpp): true when every entry lies on one of at most max_k diagonals
// col - row, every row's columns ascend, and padding every row to all of them adds at most
// max_pad of the nonzeros; then doff[0..K) are the offsets ascending and mask[i] has bit k set
// when row i stores an entry on diagonal doff[k].
constexpr int kMaxDiag = 16;
bool uniform_diagonals(int m, const int *rowptr, const int *col, int max_k, double max_pad, int *doff, int &K,
                       std::vector<int> &mask);

// Long rows whose SpMV epilogue records are folded together inside the SpMV (see fold_long_group).
constexpr int kLongGroup = 32;

struct PlanDev {
    int rpl = 0, H = 0, n_slices = 0, n_long = 0, n_chunks = 0, ctas = 0, warps_per_cta = 0, unroll = 4;
    bool has_perm = false, sorted = false, d16 = false;  // d16: 16-bit column offsets (scol16)
    bool uni = false;                 // uniform diagonals: no index stream, see uniform_diagonals
    int K = 0;                        // number of diagonals (slice width) when uni
    int doff[kMaxDiag] = {};          // their offsets col - row, ascending
    long long total = 0;
    double padding = 1.0;
    long long *slice_ptr = nullptr;   // n_slices + 1
    int *pos_row = nullptr;           // n_slices * H (original row, -1 = padding)
    int *pos_len = nullptr;           // n_slices * H
    int *warp_ptr = nullptr;          // n_warps + 1
    int *warp_units = nullptr;        // unit ids (slice s < n_slices, else chunk n_slices + c)
    int4 *unit_rec = nullptr;         // per entry of warp_units: {unit, slice steps, slice start
                                      // (low, high 32 bits)}, so a warp starts a slice's streams
                                      // one dependent load after its unit id
    double imbalance = 1.0;           // max warp cost / mean warp cost
    void *sval = nullptr;             // total values (double or float), padding zero
    int *scol = nullptr;              // total column indices (when !d16)
    short *scol16 = nullptr;          // total offsets col - row (when d16)
    int4 *chunks = nullptr;
    int *long_first = nullptr, *chunk_long = nullptr;
    double *chunk_part = nullptr;     // n_chunks
    unsigned *long_cnt = nullptr;     // n_long (kept at zero between launches)
    double *long_dot = nullptr;       // n_long * 4 epilogue contributions of long rows
    int n_groups = 0;                 // long rows folded by groups of kLongGroup
    unsigned *group_cnt = nullptr;    // n_groups (kept at zero between launches)
    double *group_dot = nullptr;      // n_groups * 4: each group's long_dot records summed (the
                                      // records the consumers reduce beside the CTA partials)
    double *cta_part = nullptr;       // ctas * 4 epilogue partials (records of 2, or 4 for EP_DOT3)
    bool built() const { return slice_ptr != nullptr; }
    void release();
};

// ---- context and matrix ------------------------------------------------------------------------
struct Solver;  // per-matrix solver workspace (hhp_krylov.cu)
struct IluDev;  // ILU(0) factors and their level-ordered solve layouts (hhp_ilu.cu)

}  // namespace hhp

struct hhp_ctx {
    int device = 0;
    int num_sms = 0;
    size_t smem_optin = 0;
    cudaStream_t stream = nullptr;
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;
    int *dev_err = nullptr;           // device error word (hhp::DEV_*), zeroed
    long long kernel_launches = 0;
    double *dot_part = nullptr;       // BLAS-1 dot: block partials (allocated on first use)
    unsigned *dot_count = nullptr;    // BLAS-1 dot: blocks done (zero between launches)
};

struct hhp_mat {
    hhp_ctx *ctx = nullptr;
    int m = 0, n = 0, nnz = 0;
    // Device CSR, padded: rowptr m+1+4, col nnz+4, val nnz+4 (padding zeroed) so 16-byte TMA
    // copies rounded outwards stay inside the allocations.
    int *rowptr = nullptr, *col = nullptr;
    double *val = nullptr;
    float *val32 = nullptr;           // lazily built FP32 copy of val
    std::vector<int> rowptr_host;     // kept for planning
    hhp::PlanDev plan64, plan32;      // plans for the FP64 and FP32 kernels
    // transpose (lazily built on the device)
    hhp_mat *t = nullptr;
    int *t_map = nullptr;             // t_map[p] = index in A of A^T's entry p
    int *rowidx = nullptr;            // row of each stored entry (built with the transpose)
    hhp::Solver *solver = nullptr;    // FP64/mixed workspace for A (A^T's lives in t->solver)
    // Jacobi preconditioning (lazily built): A with column j scaled by 1/a_jj, and 1/diag(A)
    hhp_mat *jac = nullptr;
    double *dinv = nullptr;
    std::vector<double> dinv_host;
    // row (left) Jacobi: A with row i scaled by 1/a_ii, and room for the scaled right-hand side
    hhp_mat *jac_row = nullptr;
    double *jac_row_b = nullptr;
    hhp::IluDev *ilu = nullptr;       // ILU(0) factors (lazily built)
    bool csr_dropped = false;         // col / val / val32 freed by hhp_mat_drop_csr
};

namespace hhp {

// HHP_ERR_STATE (with the message) when A's CSR arrays were dropped and `what` needs them.
hhp_status csr_needed(const hhp_mat *A, const char *what);

// ---- SpMV launchers (hhp_spmv.cu) ----------------------------------------------------------------
// Epilogue kinds of the fused SpMV.
enum EpKind : int {
    EP_AXPBY = 0,   // y = alpha*(A x) + beta*y
    EP_DOT1 = 1,    // y = A x; partial[0] += y.w1
    EP_DOT2 = 2,    // y = A x; partial[0] += y.w1, partial[1] += y.y
    EP_RESID = 3,   // y = w1 - A x (residual); partial[0] += y.y, partial[1] += w1.w1
    EP_Y = 4,       // y = A x (EP_AXPBY with alpha 1, beta 0; chosen by the launcher)
    EP_DOT3 = 5,    // y = A x; partial[0] += y.w1, partial[1] += y.y, partial[2] += y.w2 (records
                    // of 4 doubles, the last zero; every other epilogue writes records of 2)
};

hhp_status ensure_plan(hhp_mat *A, bool fp32);
// Rewrites the slice values of existing plans from the CSR values (after a value change).
hhp_status refresh_plan_values(hhp_mat *A);
// Launches the FP64 SpMV with an epilogue on `stream` (x, y, w1 length-padded device vectors).
// gate (nullable, device int): the launch does nothing when *gate == 0 at kernel start; stop
// (nullable, device int): the launch does nothing when *stop != 0 (a solver's status word).
hhp_status launch_spmv64(hhp_mat *A, cudaStream_t stream, EpKind ep, const double *x, double *y, const double *w1,
                         double alpha, double beta, const int *gate = nullptr, const double *w2 = nullptr,
                         const int *stop = nullptr);
hhp_status launch_spmv32(hhp_mat *A, cudaStream_t stream, EpKind ep, const float *x, float *y, const float *w1,
                         const int *stop = nullptr, const float *w2 = nullptr);
// Number of partial records (ctas) and long-row records of the last-used plan, for the reducers.
inline int plan_ctas(const hhp_mat *A, bool fp32) { return fp32 ? A->plan32.ctas : A->plan64.ctas; }

// ---- BLAS-1 (hhp_blas1.cu) -----------------------------------------------------------------------
void release_blas1(hhp_ctx *ctx);

// ---- Krylov solver (hhp_krylov.cu) ---------------------------------------------------------------
// b, x, xt are device pointers when host == false, host pointers when host == true.
hhp_status solve_any(hhp_mat *A, const double *b, double *x, const double *xt, const hhp_solve_opts *o,
                     hhp_solve_info *info, bool host);
inline hhp_status solve_dev(hhp_mat *A, const double *b, double *x, const double *xt, const hhp_solve_opts *o,
                            hhp_solve_info *info) {
    return solve_any(A, b, x, xt, o, info, false);
}
void solver_release(Solver *s);
// Jacobi (right) preconditioning: builds A->jac / A->dinv; solves through A->jac (hhp_precond.cu).
hhp_status ensure_jacobi(hhp_mat *A);
void release_jacobi(hhp_mat *A);
hhp_status solve_jacobi(hhp_mat *A, const double *b, double *x, const double *xt, const hhp_solve_opts *o,
                        hhp_solve_info *info, bool host);
// Row (left) Jacobi: BiCGStab on diag(A)^-1 A x = diag(A)^-1 b until b - A x meets rtol.
hhp_status solve_jacobi_row(hhp_mat *A, const double *b, double *x, const double *xt, const hhp_solve_opts *o,
                            hhp_solve_info *info, bool host);
// ILU(0) (hhp_ilu.cu): factors A on the device (levels[2], nullable: the level counts of L and U);
// out = U^-1 L^-1 in as two cooperative launches on `st` (nothing when *stop != 0); the factors
// in A's CSR order, to the host.
hhp_status ensure_ilu(hhp_mat *A, int *levels = nullptr);
void release_ilu(hhp_mat *A);
// Before hhp_mat_drop_csr frees A->col: factors that read their columns there take it over.
void ilu_keep_col(hhp_mat *A);
hhp_status launch_ilu_apply(hhp_mat *A, cudaStream_t st, const double *in, double *out, const int *stop);
hhp_status ilu_factors(hhp_mat *A, double *lu_host);
// Identifies the current factorization (0: none); graphs that captured its arrays compare it.
long long ilu_generation(const hhp_mat *A);
// Adjoint: lambda = A^-T g; dlda[k] = -lambda[row(k)] * x[col(k)].
hhp_status backward_dev(hhp_mat *A, const double *x_dev, const double *g_dev, double *dldb_dev, double *dlda_dev,
                        const hhp_solve_opts *o, hhp_solve_info *info);

// ---- transpose (hhp_transpose.cu) -----------------------------------------------------------------
hhp_status ensure_transpose(hhp_mat *A);
hhp_status refresh_transpose_values(hhp_mat *A);
hhp_status launch_dlda(hhp_mat *A, cudaStream_t s, const double *lambda, const double *x, double *dlda);

// ---- files (hhp_io.cpp) ----------------------------------------------------------------------------
hhp_status read_mtx(const char *path, int &m, int &n, int &nnz, std::vector<int> &rowptr, std::vector<int> &col,
                    std::vector<double> &val);

// ---- matrix helpers (hhp_api.cpp) ------------------------------------------------------------------
hhp_status mat_create_dev(hhp_ctx *ctx, int m, int n, int nnz, hhp_mat **out);  // allocates, zero padding
hhp_status mat_refresh_derived(hhp_mat *A);                                      // after value changes
inline int pad4(int n) { return (n + 3) & ~3; }

// Kernel tuning knobs (environment overrides read once).
struct Tuning {
    // ctas_per_sm, spmv_unroll, rpl64: 0 = chosen per matrix at plan time; d16 0: never 16-bit offsets
    int cap = 2048, long_thr = 256, window = 8192, wpc = 8, ctas_per_sm = 0, vec_blocks_per_sm = 1,
        unroll_iters = 4, spmv_unroll = 0, rpl64 = 0, rpl32 = 4, d16 = 1, uni = 1;
};
const Tuning &tuning();

// Reads an environment integer with a default.
int env_int(const char *name, int dflt);

}  // namespace hhp
