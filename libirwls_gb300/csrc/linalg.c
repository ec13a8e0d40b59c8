/*
 * linalg.c -- the reference's public linear-algebra entry points
 * (src/ParallelAlgorithms.c:91-156, :228-241, :361-388, :1318-1371), run on
 * the GPU. Matrices are column-major host arrays; the reference's thread
 * counts are accepted and ignored.
 */
#include <stdlib.h>
#include <string.h>

#include "ParallelAlgorithms.h"
#include "irwls_dev.h"
#include "irwls_gpu.h"

/* The reference allocates per-thread scratch here; this library creates its
 * device context (and fails every later call if there is no GPU). */
void initMemory(int Threads, int size) {
    (void)Threads;
    (void)size;
    irwls_dev_init();
}

void freeMemory(int Threads) {
    (void)Threads;
    irwls_dev_release_workspace();
}

/* Device scratch grows on demand; nothing to do. */
void updateMemory(int Threads, int size) {
    (void)Threads;
    (void)size;
}

/* Copies the n x n block at (ro, co) of an r-row column-major matrix into a
 * device matrix with leading dimension n + 1, factors (and solves when b is
 * given), and writes the lower factor back with a zero upper part. */
static int block_solve(double *matrix, int r, int ro, int co, int n, const double *b, double *x) {
    irwls_clear_error();
    if (irwls_dev_init()) return -1;
    const int ld = n + 1;
    double *h = NULL, *d = NULL, *dx = NULL;
    int rc = irwls_dev_host_alloc((void **)&h, (size_t)ld * ld * sizeof(double));
    if (rc) return -1;
    memset(h, 0, (size_t)ld * ld * sizeof(double));
    for (int c = 0; c < n; c++) memcpy(h + (size_t)c * ld, matrix + (size_t)(co + c) * r + ro, n * sizeof(double));
    if (b)
        for (int c = 0; c < n; c++) h[(size_t)c * ld + n] = b[c];
    rc |= irwls_dev_malloc((void **)&d, (size_t)ld * ld * sizeof(double));
    rc |= irwls_dev_malloc((void **)&dx, (size_t)(n + 1) * sizeof(double));
    if (!rc) {
        rc |= irwls_dev_h2d(d, h, (size_t)ld * ld * sizeof(double));
        rc |= irwls_dev_chol_solve(d, n, ld, NULL, b ? dx : NULL);
        rc |= irwls_dev_zero_upper(d, n, ld);
        rc |= irwls_dev_d2h(h, d, (size_t)ld * ld * sizeof(double));
        if (b) rc |= irwls_dev_d2h(x, dx, n * sizeof(double));
        rc |= irwls_dev_sync();
    }
    int info = 0;
    if (!rc) rc |= irwls_dev_pivot_status(&info);
    if (!rc && info)
        irwls_set_warning(IRWLS_WARN_PIVOT,
                          "pivot %d of the order-%d system is not positive: it is stored without its square root "
                          "and the factorization goes on, as LAPACK dpotrf leaves it for the reference's solve",
                          info, n);
    if (!rc)
        for (int c = 0; c < n; c++) memcpy(matrix + (size_t)(co + c) * r + ro, h + (size_t)c * ld, n * sizeof(double));
    irwls_dev_free(d);
    irwls_dev_free(dx);
    irwls_dev_host_free(h);
    return rc;
}

void ParallelChol(double *matrix, int r, int c, int ro, int co, int n, int nCores, int deep) {
    (void)c;
    (void)nCores;
    (void)deep;
    if (n > 0) block_solve(matrix, r, ro, co, n, NULL, NULL);
}

void ParallelLinearSystem(double *matrix1, int r1, int c1, int ro1, int co1, double *matrix2, int r2, int c2,
                          int ro2, int co2, int n, int m, double *result, int rr, int cr, int ror, int cor,
                          int nCores) {
    (void)c1;
    (void)c2;
    (void)m;
    (void)cr;
    (void)nCores;
    if (n <= 0) return;
    double *b = (double *)malloc(n * sizeof(double));
    double *x = (double *)malloc(n * sizeof(double));
    memcpy(b, matrix2 + (size_t)co2 * r2 + ro2, n * sizeof(double));
    if (block_solve(matrix1, r1, ro1, co1, n, b, x) == 0) memcpy(result + (size_t)cor * rr + ror, x, n * sizeof(double));
    free(b);
    free(x);
}

static void vec_mat(double *v, int size, double *M, double *out, int trans) {
    irwls_clear_error();
    if (size <= 0 || irwls_dev_init()) return;
    double *dM = NULL, *dv = NULL, *dout = NULL;
    int rc = 0;
    rc |= irwls_dev_malloc((void **)&dM, (size_t)size * size * sizeof(double));
    rc |= irwls_dev_malloc((void **)&dv, (size_t)size * sizeof(double));
    rc |= irwls_dev_malloc((void **)&dout, (size_t)size * sizeof(double));
    if (!rc) {
        rc |= irwls_dev_h2d(dM, M, (size_t)size * size * sizeof(double));
        rc |= irwls_dev_h2d(dv, v, (size_t)size * sizeof(double));
        rc |= irwls_dev_gemv(dM, dv, dout, size, trans);
        rc |= irwls_dev_d2h(out, dout, (size_t)size * sizeof(double));
        rc |= irwls_dev_sync();
    }
    irwls_dev_free(dM);
    irwls_dev_free(dv);
    irwls_dev_free(dout);
}

/* result = m2 m1 (src/ParallelAlgorithms.c:1318-1337). */
void ParallelVectorMatrixT(double *m1, int size, double *m2, double *result, int numThreads) {
    (void)numThreads;
    vec_mat(m1, size, m2, result, 0);
}

/* result = m1^T m2 (src/ParallelAlgorithms.c:1352-1371). */
void ParallelVectorMatrix(double *m1, int size, double *m2, double *result, int numThreads) {
    (void)numThreads;
    vec_mat(m1, size, m2, result, 1);
}
