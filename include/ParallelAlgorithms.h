/*
 * ParallelAlgorithms.h -- public linear-algebra entry points of the drop-in
 * library, executed on the GPU. Matrices are column-major doubles in host
 * memory; (r, c, ro, co) address an n x n block starting at row ro, column co
 * of an r x c matrix, as in the reference.
 *
 * The reference's per-thread recursive helpers (Chol, LinearSystem,
 * TriangleInversion, the *Product family, MoveMatrix, get/putSubMatrix) split
 * work over OpenMP thread ids; they have no meaning on a GPU and are not
 * exported.
 */
#ifndef IRWLS_GB300_PARALLEL_ALGORITHMS_H
#define IRWLS_GB300_PARALLEL_ALGORITHMS_H

#ifdef __cplusplus
extern "C" {
#endif

/* Creates the device context and a workspace for matrices of order `size`.
 * Must precede any training call, as in the reference
 * (reference include/ParallelAlgorithms.h:53, src/ParallelAlgorithms.c:91-104). */
void initMemory(int Threads, int size);

/* Releases the workspace (reference include/ParallelAlgorithms.h:66,
 * src/ParallelAlgorithms.c:118-131). */
void freeMemory(int Threads);

/* Grows the workspace to order `size` (reference include/ParallelAlgorithms.h:80,
 * src/ParallelAlgorithms.c:147-156). */
void updateMemory(int Threads, int size);

/* In-place lower Cholesky factor of the n x n block; the strict upper part of
 * the block is zeroed. A non-positive pivot at the last row is stored
 * unsquare-rooted, as LAPACK dpotrf leaves it
 * (reference include/ParallelAlgorithms.h:138, src/ParallelAlgorithms.c:228-241). */
void ParallelChol(double *matrix, int r, int c, int ro, int co, int n, int nCores, int deep);

/* Solves block(matrix1) x = block(matrix2) for one right-hand side via the
 * Cholesky factor (matrix1 is overwritten by the factor, as in the reference)
 * and writes x to result
 * (reference include/ParallelAlgorithms.h:170, src/ParallelAlgorithms.c:361-388). */
void ParallelLinearSystem(double *matrix1, int r1, int c1, int ro1, int co1,
                          double *matrix2, int r2, int c2, int ro2, int co2,
                          int n, int m, double *result, int rr, int cr, int ror, int cor,
                          int nCores);

/* result = m2 * m1 for a size x size column-major m2
 * (reference include/ParallelAlgorithms.h:185, src/ParallelAlgorithms.c:1318-1337). */
void ParallelVectorMatrixT(double *m1, int size, double *m2, double *result, int numThreads);

/* result = m1^T * m2 (row vector times matrix)
 * (reference include/ParallelAlgorithms.h:200, src/ParallelAlgorithms.c:1352-1371). */
void ParallelVectorMatrix(double *m1, int size, double *m2, double *result, int numThreads);

#ifdef __cplusplus
}
#endif

#endif
