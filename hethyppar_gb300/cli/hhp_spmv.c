/*
 * hhp-spmv -- SpMV-only benchmark on one GB300 through libhhp_gpu.so.
 *
 * Drop-in for the reference's spmv-gpu (src/entry/spmv_gpu.c): the same argp flags (-m matrix,
 * -x input vector, -o output vector, -n repetitions), the same flow (read, one warm-up SpMV, n
 * timed SpMVs between device synchronisations, y copied back and compared with [1, 2, ..., m],
 * the known answer when x came from prepare_spmv_input.m) and the same "key : value" stdout
 * (spmv_gpu.c:139-151). The SpMV is the library's (hhp_spmv_dev) instead of cuSPARSE.
 *
 *   --out-format F    compat (default, "%lf" like vector_write) | exact ("%.17g")
 */
#include <argp.h>
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>
#include <unistd.h>

#include <cuda_runtime_api.h>

#include "hhp_gpu.h"

enum { OPT_OUTFMT = 1000, OPT_DEVICE };

struct arguments {
    char *input_matrix, *input_x, *output_y;
    int n_iters, exact, device;
};

static struct argp_option options[] = {
    {"input-matrix", 'm', "FILE", 0, "Input matrix market file path (or a binary CSR file)", 0},
    {"input-x", 'x', "FILE", 0, "Input X vector file path", 0},
    {"output-y", 'o', "FILE", 0, "Output Y vector file path", 0},
    {"n-iters", 'n', "POSITIVE-INTEGER", 0, "Number of SpMV repetitions", 0},
    {"out-format", OPT_OUTFMT, "compat|exact", 0, "Output vector format (default compat: %lf)", 0},
    {"device", OPT_DEVICE, "N", 0, "CUDA device (default 0)", 0},
    {0}};

static error_t parse_opt(int key, char *arg, struct argp_state *state) {
    struct arguments *a = state->input;
    char *end = NULL;
    switch (key) {
        case 'm': a->input_matrix = arg; break;
        case 'x': a->input_x = arg; break;
        case 'o': a->output_y = arg; break;
        case 'n': a->n_iters = (int)strtol(arg, &end, 10); break;
        case OPT_OUTFMT:
            if (strcmp(arg, "exact") == 0) a->exact = 1;
            else if (strcmp(arg, "compat") == 0) a->exact = 0;
            else argp_error(state, "unknown output format '%s'", arg);
            break;
        case OPT_DEVICE: a->device = (int)strtol(arg, &end, 10); break;
        case ARGP_KEY_ARG: return 0;
        default: return ARGP_ERR_UNKNOWN;
    }
    return 0;
}

static struct argp argp = {options, parse_opt, "",
                           "SpMV-only GPU benchmark -- repeatedly computes Y = A*X on the GPU and times it", 0, 0, 0};

static double now_s(void) {
    struct timespec t;
    clock_gettime(CLOCK_MONOTONIC, &t);
    return (double)t.tv_sec + 1e-9 * (double)t.tv_nsec;
}

#define FAIL(...)                                       \
    do {                                                \
        fprintf(stderr, "hhp-spmv: " __VA_ARGS__);      \
        fprintf(stderr, "\n");                          \
        return EXIT_FAILURE;                            \
    } while (0)
#define CHECK(call)                                                                                   \
    do {                                                                                              \
        hhp_status st_ = (call);                                                                      \
        if (st_ != HHP_OK) FAIL("%s: %s (%s)", #call, hhp_status_str(st_), hhp_last_error());       \
    } while (0)
#define CHECK_CUDA(call)                                                                              \
    do {                                                                                              \
        cudaError_t e_ = (call);                                                                      \
        if (e_ != cudaSuccess) FAIL("%s: %s", #call, cudaGetErrorString(e_));                         \
    } while (0)

int main(int argc, char **argv) {
    struct arguments a;
    memset(&a, 0, sizeof a);
    a.n_iters = 1;
    argp_parse(&argp, argc, argv, 0, 0, &a);
    if (!a.input_matrix || !a.input_x || !a.output_y) FAIL("-m, -x, and -o must all be specified.");
    if (access(a.input_matrix, F_OK) == -1) FAIL("Input matrix file '%s' does not exist", a.input_matrix);
    if (access(a.input_x, F_OK) == -1) FAIL("Input vector file '%s' does not exist", a.input_x);
    const int niters = a.n_iters < 1 ? 1 : a.n_iters;

    const double t_begin = now_s();
    hhp_ctx *ctx = NULL;
    CHECK(hhp_ctx_create(a.device, &ctx));
    const double t_read0 = now_s();
    hhp_mat *A = NULL;
    CHECK(hhp_mat_from_mtx(ctx, a.input_matrix, &A));
    int m = 0, n = 0, nnz = 0;
    CHECK(hhp_mat_shape(A, &m, &n, &nnz));
    double *xh = malloc(sizeof(double) * (size_t)(n > 0 ? n : 1));
    double *yh = malloc(sizeof(double) * (size_t)(m > 0 ? m : 1));
    if (!xh || !yh) FAIL("out of host memory");
    CHECK(hhp_vector_read(a.input_x, n, xh));
    double *xd = NULL, *yd = NULL;
    CHECK_CUDA(cudaMalloc((void **)&xd, sizeof(double) * (size_t)(n > 0 ? n : 1)));
    CHECK_CUDA(cudaMalloc((void **)&yd, sizeof(double) * (size_t)(m > 0 ? m : 1)));
    CHECK_CUDA(cudaMemcpy(xd, xh, sizeof(double) * (size_t)n, cudaMemcpyHostToDevice));
    CHECK_CUDA(cudaMemset(yd, 0, sizeof(double) * (size_t)(m > 0 ? m : 1)));
    /* the library works on its own non-blocking stream: the copies above must have landed */
    CHECK_CUDA(cudaDeviceSynchronize());
    const double t_read1 = now_s();
    printf("Matrix name : %s\n", a.input_matrix);

    /* warm-up (the first call builds the slice layout), then the timed repetitions */
    CHECK(hhp_spmv_dev(ctx, A, 1.0, xd, 0.0, yd));
    CHECK(hhp_ctx_sync(ctx));
    const double t0 = now_s();
    for (int i = 0; i < niters; ++i) CHECK(hhp_spmv_dev(ctx, A, 1.0, xd, 0.0, yd));
    CHECK(hhp_ctx_sync(ctx));
    const double t1 = now_s();

    CHECK_CUDA(cudaMemcpy(yh, yd, sizeof(double) * (size_t)m, cudaMemcpyDeviceToHost));
    double max_abs_err = 0.0;
    for (int i = 0; i < m; ++i) {
        const double err = fabs(yh[i] - (double)(i + 1));
        if (err > max_abs_err) max_abs_err = err;
    }
    const double spmv_total = t1 - t0;
    printf("n_iters : %d \n"
           "spmv : %lf \n"
           "spmv_per_iter : %e \n"
           "file_read : %lf \n"
           "max_abs_err_vs_1ton : %e \n",
           niters, spmv_total, spmv_total / niters, t_read1 - t_read0, max_abs_err);
    printf("everything_total : %lf\n", now_s() - t_begin);
    printf("\n----------------------------------------------------------------------\n");
    CHECK(hhp_vector_write(a.output_y, m, yh, a.exact));

    cudaFree(xd);
    cudaFree(yd);
    free(xh);
    free(yh);
    hhp_mat_destroy(A);
    hhp_ctx_destroy(ctx);
    return EXIT_SUCCESS;
}
