/*
 * irwls_port.c -- CPU ORACLE (test and benchmark infrastructure only).
 *
 * A plain-C restatement of the LIBIRWLS training and prediction hot path,
 * used as the checker of the GPU library and as the timed CPU baseline when
 * the reference itself cannot be compiled on the machine. It is never linked
 * into the product library.
 *
 * Every routine follows one reference routine (file:line in RobeDM/LIBIRWLS)
 * and keeps its arithmetic order: same loop orders, same a*b+c groupings
 * (build with -ffp-contract=off), and the same BLAS/LAPACK calls with the same
 * arguments, taken from the OpenBLAS bundled with scipy. With Threads == 1 its
 * results are therefore bit-identical to the reference run with -t 1.
 * With Threads > 1 the kernel loops run under OpenMP; the linear solves and
 * the SGMA candidate draws keep their single-thread order (the reference draws
 * SGMA candidates with rand() inside an OpenMP loop, which races).
 *
 * It exports the reference's API names (trainFULL, SGMA, ...) from its own
 * shared object; load it with RTLD_LOCAL and link with -Bsymbolic.
 */
#include <math.h>
#include <omp.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>

#include "IOStructures.h"

/* LAPACK / BLAS from scipy's OpenBLAS (Fortran ABI, LP64). */
extern void scipy_dgemm_(char *, char *, int *, int *, int *, double *, double *, int *,
                         double *, int *, double *, double *, int *);
extern void scipy_dpotrf_(char *, int *, double *, int *, int *);
extern void scipy_dpotrs_(char *, int *, int *, double *, int *, double *, int *, int *);
extern void scipy_dtrtri_(char *, char *, int *, double *, int *, int *);
extern void scipy_dsyrk_(char *, char *, int *, int *, double *, double *, int *, double *,
                         double *, int *);
extern void scipy_dtrmm_(char *, char *, char *, char *, int *, int *, double *, double *, int *,
                         double *, int *);

/* ------------------------------------------------------------------------ */
/* Kernel functions: src/kernels.c:63-118 and :137-183                       */
/* ------------------------------------------------------------------------ */

/* Merge-join dot product of two index-sorted rows; the products are added in
 * ascending index order (src/kernels.c:73-84). */
static double sparse_dot(const svm_sample *a, const svm_sample *b) {
    double acc = 0.0;
    while (a->index != -1 && b->index != -1) {
        if (a->index == b->index) {
            acc += a->value * b->value;
            a++;
            b++;
        } else if (a->index > b->index) {
            b++;
        } else {
            a++;
        }
    }
    return acc;
}

/* q1 + q2 followed by "+ (-2 a) b" for every shared index, in index order
 * (src/kernels.c:101-114, :163-178). */
static double norm_form_distance(double q1, double q2, const svm_sample *a, const svm_sample *b) {
    double d2 = q1 + q2;
    while (a->index != -1 && b->index != -1) {
        if (a->index == b->index) {
            d2 += -2.0 * a->value * b->value;
            a++;
            b++;
        } else if (a->index < b->index) {
            a++;
        } else {
            b++;
        }
    }
    return d2;
}

double kernelFunction(svm_dataset ds, int i1, int i2, properties props) {
    const svm_sample *a = ds.x[i1];
    const svm_sample *b = ds.x[i2];
    if (props.kernelType == 0) return sparse_dot(a, b);
    double d2;
    if (ds.sparse == 0) {
        /* maxdim raw values read in storage order (src/kernels.c:90-97) */
        d2 = 0.0;
        for (int t = 0; t < ds.maxdim; t++) {
            double diff = a[t].value - b[t].value;
            d2 += diff * diff;
        }
    } else {
        d2 = norm_form_distance(ds.quadratic_value[i1], ds.quadratic_value[i2], a, b);
    }
    return exp(-(props.Kgamma) * d2);
}

double kernelTest(svm_dataset ds, int i1, model m, int i2) {
    const svm_sample *a = ds.x[i1];
    const svm_sample *b = m.x[i2];
    if (m.kernelType == 0) return sparse_dot(a, b);
    double d2 = norm_form_distance(ds.quadratic_value[i1], m.quadratic_value[i2], a, b);
    return exp(-(m.Kgamma) * d2);
}

/* ------------------------------------------------------------------------ */
/* Linear solve: src/ParallelAlgorithms.c:361-447 with one thread            */
/* ------------------------------------------------------------------------ */

/* Copies the rows x cols block at (r0, c0) of a column-major matrix with
 * leading dimension ld into a contiguous buffer, or back. */
static void block_get(const double *M, int ld, int r0, int c0, int rows, int cols, double *out) {
    for (int j = 0; j < cols; j++) memcpy(out + (size_t)j * rows, M + (size_t)(c0 + j) * ld + r0, rows * sizeof(double));
}
static void block_put(double *M, int ld, int r0, int c0, int rows, int cols, const double *in) {
    for (int j = 0; j < cols; j++) memcpy(M + (size_t)(c0 + j) * ld + r0, in + (size_t)j * rows, rows * sizeof(double));
}

/* dpotrf('L') of the n x n block at (o, o), strict upper part zeroed
 * (the leaf of src/ParallelAlgorithms.c:269-293). A failed pivot is left as
 * dpotrf leaves it. */
static void leaf_cholesky(double *M, int ld, int o, int n) {
    if (n <= 0) return;
    double *blk = (double *)malloc((size_t)n * n * sizeof(double));
    block_get(M, ld, o, o, n, n, blk);
    char lo = 'L';
    int info = 0;
    scipy_dpotrf_(&lo, &n, blk, &n, &info);
    for (int c = 1; c < n; c++)
        for (int r = 0; r < c; r++) blk[(size_t)c * n + r] = 0.0;
    block_put(M, ld, o, o, n, n, blk);
    free(blk);
}

/* One level of the reference's recursive Cholesky (Chol with deep = 2 and a
 * single thread, src/ParallelAlgorithms.c:294-327): factor A11, invert L11 with
 * dtrtri, L21 = A21 L11^-T by dtrmm, A22 -= L21 L21^T by dsyrk, factor A22. */
static void split_cholesky(double *M, int n) {
    if (n < 8) {
        leaf_cholesky(M, n, 0, n);
        return;
    }
    int n1 = (int)ceil(0.5 * n);
    int n2 = n - n1;
    leaf_cholesky(M, n, 0, n1);

    double *Linv = (double *)malloc((size_t)n1 * n1 * sizeof(double));
    block_get(M, n, 0, 0, n1, n1, Linv);
    char lo = 'L', nu = 'N', rt = 'R', tr = 'T';
    int info = 0;
    scipy_dtrtri_(&lo, &nu, &n1, Linv, &n1, &info);

    double *L21 = (double *)malloc((size_t)n2 * n1 * sizeof(double));
    block_get(M, n, n1, 0, n2, n1, L21);
    double one = 1.0, minus_one = -1.0;
    scipy_dtrmm_(&rt, &lo, &tr, &nu, &n2, &n1, &one, Linv, &n1, L21, &n2);
    block_put(M, n, n1, 0, n2, n1, L21);

    double *A22 = (double *)malloc((size_t)n2 * n2 * sizeof(double));
    block_get(M, n, n1, n1, n2, n2, A22);
    scipy_dsyrk_(&lo, &nu, &n2, &n1, &minus_one, L21, &n2, &one, A22, &n2);
    for (int i = 0; i < n2; i++)
        for (int j = i; j < n2; j++) A22[(size_t)j * n2 + i] = A22[(size_t)i * n2 + j];
    block_put(M, n, n1, n1, n2, n2, A22);
    for (int c = n1; c < n; c++)
        for (int r = 0; r < n1; r++) M[(size_t)c * n + r] = 0.0;

    leaf_cholesky(M, n, n1, n2);
    free(Linv);
    free(L21);
    free(A22);
}

/* Solves M x = b for the n x n column-major M (overwritten with its factor),
 * following ParallelLinearSystem with nCores == 1. */
static void port_linear_system(double *M, int n, const double *b, double *x) {
    char lo = 'L';
    int one = 1, info = 0;
    if (n <= 1) {
        /* n <= nCores: plain dpotrf + dpotrs (src/ParallelAlgorithms.c:378-387) */
        scipy_dpotrf_(&lo, &n, M, &n, &info);
        memcpy(x, b, n * sizeof(double));
        scipy_dpotrs_(&lo, &n, &one, M, &n, x, &n, &info);
        return;
    }
    split_cholesky(M, n);
    for (int c = 0; c < n; c++)
        for (int r = 0; r < c; r++) M[(size_t)c * n + r] = 0.0;
    memcpy(x, b, n * sizeof(double));
    scipy_dpotrs_(&lo, &n, &one, M, &n, x, &n, &info);
}

/* Exported for the linear-algebra unit tests: solve of an n x n system with
 * the single-thread reference algorithm. */
void port_solve(double *M, int n, const double *b, double *x) { port_linear_system(M, n, b, x); }

/* Host initMemory/freeMemory/updateMemory have no state to keep here. */
void initMemory(int Threads, int size) { (void)Threads; (void)size; }
void freeMemory(int Threads) { (void)Threads; }

/* ------------------------------------------------------------------------ */
/* Full IRWLS: src/full-train.c                                              */
/* ------------------------------------------------------------------------ */

/* Fisher-Yates with rand() (src/full-train.c:65-77). */
int *rpermute(int n) {
    int *p = (int *)malloc((n > 0 ? n : 1) * sizeof(int));
    for (int k = 0; k < n; k++) p[k] = k;
    for (int k = n - 1; k > 0; k--) {
        int j = rand() % (k + 1);
        int t = p[j];
        p[j] = p[k];
        p[k] = t;
    }
    return p;
}

/* Inner IRWLS on the working-set dataset (src/full-train.c:96-362). */
double *subIRWLS(svm_dataset ds, properties props, double *GIN, double *e, double *beta) {
    const int l = ds.l;
    const double C = props.C;
    double *a = (double *)calloc(l > 0 ? l : 1, sizeof(double));
    int *grp = (int *)calloc(l > 0 ? l : 1, sizeof(int));
    double *bnew = (double *)calloc(l + 1, sizeof(double));
    double *bsol = (double *)calloc(l + 1, sizeof(double));
    double *bbest = (double *)calloc(l + 1, sizeof(double));
    int *S1 = (int *)calloc(l + 1, sizeof(int));
    int *S3 = (int *)calloc(l > 0 ? l : 1, sizeof(int));
    double *H = (double *)calloc((size_t)(l + 1) * (l + 1), sizeof(double));
    double *rhs = (double *)calloc(l + 1, sizeof(double));
    double *G13 = (double *)calloc(l + 1, sizeof(double));
    int nS1 = 0, nS3 = 0;

    for (int i = 0; i < l; i++) {
        a[i] = (e[i] * ds.y[i] < 0) ? 0.0 : 1.0 * ds.y[i] * C / e[i];
        if (a[i] == 0) {
            grp[i] = 2;
        } else if (beta[i] == ds.y[i] * C) {
            S3[nS3++] = i;
            grp[i] = 3;
        } else {
            S1[nS1++] = i;
            grp[i] = 1;
        }
    }
    S1[nS1] = l;

    int iter = 0, since_best = 0;
    double dW = 1e9, nW = 1.0, best = 1e9, bmax = 0.0, bmin = 0.0;
    /* "&&" binds tighter than "||" in the reference condition (src/full-train.c:158) */
    while ((iter < 5) || ((bmin < 0.0) || (bmax > C)) && (iter < 1000) && (since_best < 5) &&
                             (dW / nW > 1e-6)) {
        iter++;
        const int n = nS1 + 1;
        memset(bsol, 0, n * sizeof(double));
        memset(rhs, 0, n * sizeof(double));
        memset(H, 0, (size_t)n * n * sizeof(double));
#pragma omp parallel for schedule(static) if (props.Threads > 1)
        for (int i = 0; i < nS1; i++) {
            const int si = S1[i];
            H[(size_t)i * n + nS1] = ds.y[si];
            H[(size_t)nS1 * n + i] = ds.y[si];
            rhs[i] = 1.0 - G13[i] - GIN[si];
            for (int j = 0; j < nS1; j++) {
                H[(size_t)i * n + j] = kernelFunction(ds, si, S1[j], props) * ds.y[si] * ds.y[S1[j]];
                if (i == j) H[(size_t)i * n + j] += (1.0 / (a[si]));
            }
        }
        H[(size_t)nS1 * n + nS1] = 0.0;
        rhs[nS1] = -G13[nS1] - GIN[l];

        port_linear_system(H, n, rhs, bsol);

        dW = 0.0;
        nW = 0.0;
        bmax = 0.0;
        bmin = 0.0;
        memset(bnew, 0, (l + 1) * sizeof(double));
        for (int i = 0; i < nS1; i++) {
            if (bsol[i] > bmax) bmax = bsol[i];
            if (bsol[i] < bmin) bmin = bsol[i];
            bnew[S1[i]] = bsol[i] * ds.y[S1[i]];
        }
        for (int i = 0; i < nS3; i++) bnew[S3[i]] = C * ds.y[S3[i]];
        bnew[l] = bsol[nS1];
        for (int i = 0; i < l + 1; i++) {
            double d = bnew[i] - beta[i];
            dW += d * d;
            nW += beta[i] * beta[i];
        }

#pragma omp parallel for schedule(static) if (props.Threads > 1)
        for (int i = 0; i < l; i++) {
            for (int j = 0; j < l; j++)
                if (bnew[j] != beta[j]) e[i] = e[i] - kernelFunction(ds, i, j, props) * (bnew[j] - beta[j]);
            e[i] = e[i] - (bnew[l] - beta[l]);
        }

        if (dW / nW < best) {
            best = dW / nW;
            since_best = 0;
            memcpy(bbest, bnew, (l + 1) * sizeof(double));
        } else {
            since_best += 1;
        }

        for (int i = 0; i < l; i++) {
            const double ey = e[i] * ds.y[i];
            if (ey < 0.0) a[i] = 0.0;
            else if (ey < (1.0 / 10000)) a[i] = C * 10000.0;
            else a[i] = 1.0 * ds.y[i] * C / e[i];
            if (ey < 0.0 && grp[i] != 2) grp[i] = 2;
            if (grp[i] == 1 && ds.y[i] * bnew[i] >= 0.99 * C && ds.y[i] * bnew[i] <= 1.01 * C) grp[i] = 3;
            if (a[i] == 0.0 && grp[i] == 1) grp[i] = 2;
            if (grp[i] == 2 && a[i] != 0.0) grp[i] = 1;
            beta[i] = bnew[i];
        }
        beta[l] = bnew[l];

        nS1 = 0;
        nS3 = 0;
        for (int i = 0; i < l; i++) {
            if (grp[i] == 1) S1[nS1++] = i;
            else if (grp[i] == 3) {
                S3[nS3] = i;
                rhs[nS3] = C; /* the reference keeps C per S3 entry in its rhs buffer */
                nS3++;
            }
        }
        S1[nS1] = l;
        memset(G13, 0, (nS1 + 1) * sizeof(double));
        if (nS3 > 0) {
#pragma omp parallel for schedule(static) if (props.Threads > 1)
            for (int i = 0; i < nS1 + 1; i++) {
                if (i < nS1) {
                    for (int o = 0; o < nS3; o++)
                        G13[i] += rhs[o] * kernelFunction(ds, S1[i], S3[o], props) * ds.y[S1[i]] * ds.y[S3[o]];
                } else {
                    for (int o = 0; o < nS3; o++) G13[nS1] += rhs[o] * ds.y[S3[o]];
                }
            }
        }
    }
    free(a);
    free(grp);
    free(bsol);
    free(bnew);
    free(S3);
    free(S1);
    free(rhs);
    free(G13);
    free(H);
    return bbest;
}

/* Outer working-set loop (src/full-train.c:373-668). */
double *trainFULL(svm_dataset ds, properties props) {
    if (props.verbose == 1) printf("\n");
    const int W = props.MaxSize, l = ds.l;
    const double C = props.C, thr = 0.001;
    svm_dataset sub;
    sub.sparse = ds.sparse;
    sub.maxdim = ds.maxdim;
    sub.y = (double *)calloc(W, sizeof(double));
    sub.quadratic_value = (double *)calloc(W, sizeof(double));
    sub.x = (svm_sample **)calloc(W, sizeof(svm_sample *));
    sub.features = NULL;

    double *e = (double *)calloc(l, sizeof(double));
    double *beta = (double *)calloc(l + 1, sizeof(double));
    double *bnew = (double *)calloc(l + 1, sizeof(double));
    double *bbest = (double *)calloc(l + 1, sizeof(double));
    int *SW = (int *)calloc(W, sizeof(int));
    int *SIN = (int *)calloc(l, sizeof(int));
    int *SC = (int *)calloc(l, sizeof(int));
    double *GIN = (double *)calloc(W + 1, sizeof(double));
    double *esub = (double *)calloc(W + 1, sizeof(double));
    double *bsub = (double *)calloc(W + 1, sizeof(double));
    int nSW = 0, nSIN = 0, nSC = 0;

    for (int i = 0; i < l; i++) {
        if (i % 10 < 1 && nSW < W) SW[nSW++] = i;
        else SIN[nSIN++] = i;
        e[i] = ds.y[i];
    }

    int stop = 0, since_best = 0;
    double best = 1e20;
    while (stop == 0 && since_best < 300) {
        if (nSIN > 0) {
            memset(GIN, 0, (nSW + 1) * sizeof(double));
#pragma omp parallel for schedule(static) if (props.Threads > 1)
            for (int i = 0; i < nSW + 1; i++) {
                if (i < nSW) {
                    for (int o = 0; o < nSIN; o++)
                        if (bnew[SIN[o]] != 0.0)
                            GIN[i] += bnew[SIN[o]] * kernelFunction(ds, SW[i], SIN[o], props) * ds.y[SW[i]];
                } else {
                    for (int o = 0; o < nSIN; o++) GIN[nSW] += bnew[SIN[o]];
                }
            }
        }
        sub.l = nSW;
        for (int i = 0; i < nSW; i++) {
            sub.y[i] = ds.y[SW[i]];
            sub.quadratic_value[i] = ds.quadratic_value[SW[i]];
            sub.x[i] = ds.x[SW[i]];
            bsub[i] = beta[SW[i]];
            esub[i] = e[SW[i]];
        }
        bsub[nSW] = beta[l];

        double *bt = subIRWLS(sub, props, GIN, esub, bsub);

        memcpy(bnew, beta, (l + 1) * sizeof(double));
        for (int i = 0; i < nSW; i++) bnew[SW[i]] = bt[i];
        bnew[l] = bt[sub.l];
#pragma omp parallel for schedule(static) if (props.Threads > 1)
        for (int i = 0; i < l; i++) {
            for (int j = 0; j < nSW; j++) e[i] = e[i] - kernelFunction(ds, i, SW[j], props) * (bnew[SW[j]] - beta[SW[j]]);
            e[i] = e[i] - (bnew[l] - beta[l]);
        }
        free(bt);

        double dW = 0.0, nW = 0.0;
        for (int i = 0; i < l + 1; i++) {
            double d = beta[i] - bnew[i];
            dW = dW + d * d;
            nW = nW + beta[i] * beta[i];
        }
        if (dW / nW < props.Eta) stop = 1;
        memcpy(beta, bnew, (l + 1) * sizeof(double));
        if (dW / nW < best) {
            best = dW / nW;
            since_best = 0;
            memcpy(bbest, bnew, (l + 1) * sizeof(double));
        } else {
            since_best += 1;
        }

        /* Classification (src/full-train.c:540-615): the first violator of
         * each (kind, label) pair enters the working set directly. */
        int found[6] = {0, 0, 0, 0, 0, 0}; /* at C: -1,+1 ; at 0: -1,+1 ; free: -1,+1 */
        nSW = 0;
        nSIN = 0;
        nSC = 0;
        for (int i = 0; i < l; i++) {
            const double by = bnew[i] * ds.y[i];
            int kind = -1, violator = 0;
            if (by == C) {
                kind = 0;
                violator = e[i] * ds.y[i] < -1.0 * thr;
                if (!violator) { SIN[nSIN++] = i; continue; }
            } else if (bnew[i] == 0.0) {
                kind = 1;
                violator = e[i] * ds.y[i] > thr;
                if (!violator) { SIN[nSIN++] = i; continue; }
            } else if (by != 0.0 && by != C) {
                kind = 2;
                violator = fabs(e[i] * ds.y[i]) > thr;
                if (!violator) { SC[nSC++] = i; continue; }
            } else {
                continue;
            }
            int slot = -1;
            if (ds.y[i] == -1) slot = 2 * kind;
            else if (ds.y[i] == 1) slot = 2 * kind + 1;
            if (slot >= 0 && found[slot] == 0) {
                found[slot] = 1;
                SW[nSW++] = i;
            } else {
                SC[nSC++] = i;
            }
        }
        if (props.verbose == 1) {
            printf("%s", ".");
            fflush(stdout);
        }
        if (nSC < (W - nSW)) {
            for (int i = 0; i < nSC; i++) SW[nSW++] = SC[i];
        } else {
            int *perm = rpermute(nSC);
            const int space = W - nSW;
            for (int i = 0; i < nSC; i++) {
                if (i < space) SW[nSW++] = SC[perm[i]];
                else SIN[nSIN++] = SC[perm[i]];
            }
            free(perm);
        }
    }
    free(e);
    free(beta);
    free(bbest);
    free(GIN);
    free(esub);
    free(bsub);
    free(SW);
    free(SIN);
    free(SC);
    free(sub.y);
    free(sub.quadratic_value);
    free(sub.x);
    if (props.verbose == 1) printf("\n");
    return bnew;
}

/* ------------------------------------------------------------------------ */
/* Budgeted IRWLS: src/budgeted-train.c                                      */
/* ------------------------------------------------------------------------ */

int *randomCentroids(svm_dataset ds, properties props) {
    int *p = (int *)malloc(ds.l * sizeof(int));
    for (int i = 0; i < ds.l; ++i) p[i] = i;
    for (int i = ds.l - 1; i >= 0; --i) {
        int j = rand() % (i + 1);
        int t = p[i];
        p[i] = p[j];
        p[j] = t;
    }
    int *c = (int *)malloc(props.size * sizeof(int));
    for (int i = 0; i < props.size; i++) c[i] = p[i];
    free(p);
    return c;
}

/* Row-partitioned dgemm products of src/ParallelAlgorithms.c:1318-1371. */
static void vec_mat_T(double *v, int size, double *M, double *out, int parts) {
    char nn = 'N';
    int one = 1;
    double fone = 1.0, zero = 0.0;
#pragma omp parallel for schedule(static) if (parts > 1)
    for (int p = 0; p < parts; p++) {
        int c0 = (int)round(p * size / parts), c1 = (int)round((p + 1) * size / parts) - 1;
        int len = c1 - c0 + 1;
        if (len > 0) scipy_dgemm_(&nn, &nn, &len, &one, &size, &fone, &M[c0], &size, v, &size, &zero, &out[c0], &size);
    }
}
static void vec_mat(double *v, int size, double *M, double *out, int parts) {
    char nn = 'N';
    int one = 1;
    double fone = 1.0, zero = 0.0;
#pragma omp parallel for schedule(static) if (parts > 1)
    for (int p = 0; p < parts; p++) {
        int c0 = (int)round(p * size / parts), c1 = (int)round((p + 1) * size / parts) - 1;
        int len = c1 - c0 + 1;
        if (len > 0) scipy_dgemm_(&nn, &nn, &one, &len, &size, &fone, v, &one, &M[(size_t)size * c0], &size, &zero, &out[c0], &one);
    }
}

/* SGMA (src/budgeted-train.c:114-309). Candidates of a step are drawn first,
 * in the single-thread order, then scored (in parallel when Threads > 1). */
int *SGMA(svm_dataset ds, properties props) {
    const int m = props.size, l = ds.l, NC = 64;
    double *score = (double *)malloc(NC * sizeof(double));
    int *cand = (int *)malloc(NC * sizeof(int));
    int *cent = (int *)malloc(m * sizeof(int));
    double *eta = (double *)malloc(NC * sizeof(double));
    double *KSC = (double *)malloc((size_t)l * m * sizeof(double));
    double *L = (double *)calloc((size_t)m * m, sizeof(double));
    double *Li = (double *)calloc((size_t)m * m, sizeof(double));
    double *Ln = (double *)calloc((size_t)m * m, sizeof(double));
    double *Lin = (double *)calloc((size_t)m * m, sizeof(double));
    double *L2 = (double *)calloc(m, sizeof(double));
    double *IL2 = (double *)calloc(m, sizeof(double));
    double *KNC = (double *)malloc((size_t)NC * m * sizeof(double));
    double *KSM = (double *)malloc((size_t)NC * l * sizeof(double));
    double *Z = (double *)malloc((size_t)NC * m * sizeof(double));
    int best_c = 0;
    double value = 0.0;

    for (int s = 0; s < m; s++) {
        if (s > 1) {
            for (int i = 0; i < NC; i++) {
                const double want = (i % 2) * 2.0 - 1;
                int pick = rand() % l;
                while (ds.y[pick] != want) pick = rand() % l;
                cand[i] = pick;
            }
#pragma omp parallel for schedule(static) if (props.Threads > 1)
            for (int i = 0; i < NC; i++) {
                double *ksm = KSM + (size_t)i * l, *knc = KNC + (size_t)i * m, *z = Z + (size_t)i * m;
                for (int r = 0; r < l; r++) ksm[r] = kernelFunction(ds, cand[i], r, props);
                for (int r = 0; r < s; r++) {
                    double v = kernelFunction(ds, cand[i], cent[r], props);
                    knc[r] = v;
                    z[r] = v;
                }
                char lo = 'L', nn = 'N';
                int ss = s, one = 1, info = 0;
                double fone = 1.0, mone = -1.0;
                scipy_dpotrs_(&lo, &ss, &one, L, &ss, z, &ss, &info);
                double v = 1.0;
                for (int r = 0; r < s; r++) v = v - (knc[r] * z[r]);
                eta[i] = v;
                int ll = l;
                scipy_dgemm_(&nn, &nn, &ll, &one, &ss, &fone, KSC, &ll, z, &ss, &mone, ksm, &ll);
                double acc = 0.0;
                for (int r = 0; r < l; r++) acc += ksm[r] * ksm[r];
                score[i] = (eta[i] > 0.0) ? (1.0 / eta[i]) * acc : 0.0;
            }
            value = score[0];
            best_c = 0;
            for (int i = 1; i < NC; i++)
                if (score[i] > value) {
                    value = score[i];
                    best_c = i;
                }
            cent[s] = cand[best_c];
        } else {
            if (s == 0) {
                cent[s] = l;
            } else {
                cent[s] = l + 1;
                KNC[0] = kernelFunction(ds, cent[0], cent[1], props);
            }
            value = 1.0;
            best_c = 0;
        }
        if (props.verbose == 1) {
            if (s == 0) printf("Best Error Descent %f, Average of positive data is centroid %d\n", value, s);
            if (s == 1) printf("Best Error Descent %f, Average of negative data is centroid %d\n", value, s);
            if (s > 1) printf("Best Error Descent %f, Data with index %d is centroid %d\n", value, cent[s], s);
        }
#pragma omp parallel for schedule(static) if (props.Threads > 1)
        for (int r = 0; r < l; r++) KSC[(size_t)s * l + r] = kernelFunction(ds, r, cent[s], props);

        if (s == 0) {
            Ln[0] = pow(kernelFunction(ds, cent[0], cent[0], props) + 0.000001, 0.5);
            Lin[0] = 1.0 / Ln[0];
        } else {
            vec_mat_T(KNC + (size_t)best_c * m, s, Li, L2, props.Threads);
            double l3 = kernelFunction(ds, cent[s], cent[s], props) + 0.00001;
            for (int r = 0; r < s; r++) l3 = l3 - (L2[r] * L2[r]);
            l3 = pow(l3, 0.5);
            double il3 = 1.0 / l3;
            vec_mat(L2, s, Li, IL2, props.Threads);
            for (int r = 0; r < s; r++)
                for (int c = 0; c < s; c++) {
                    Ln[r * (s + 1) + c] = L[r * s + c];
                    Lin[r * (s + 1) + c] = Li[r * s + c];
                }
            Ln[(s + 1) * (s + 1) - 1] = l3;
            Lin[(s + 1) * (s + 1) - 1] = il3;
            for (int r = 0; r < s; r++) {
                Ln[r * (s + 1) + s] = L2[r];
                Lin[r * (s + 1) + s] = -il3 * IL2[r];
            }
        }
        double *t;
        t = L; L = Ln; Ln = t;
        t = Li; Li = Lin; Lin = t;
    }
    free(score); free(cand); free(eta); free(KSC); free(L); free(Li); free(Ln); free(Lin);
    free(L2); free(IL2); free(KNC); free(KSM); free(Z);
    return cent;
}

/* IRWLS of the budgeted model (src/budgeted-train.c:324-505). */
double *IRWLSpar(svm_dataset ds, int *idx, properties props) {
    const int m = props.size, l = ds.l;
    double *KC = (double *)calloc((size_t)m * m, sizeof(double));
    double *KSC = (double *)calloc((size_t)l * m, sizeof(double));
    double *KSCA = (double *)calloc((size_t)l * m, sizeof(double));
    double *Da = (double *)calloc(l, sizeof(double));
    double *Day = (double *)calloc(l, sizeof(double));
#pragma omp parallel for schedule(static) if (props.Threads > 1)
    for (int i = 0; i < m; i++)
        for (int j = 0; j < m; j++) {
            KC[(size_t)i * m + j] = kernelFunction(ds, idx[i], idx[j], props);
            if (i == j) KC[(size_t)i * m + j] += pow(10, -5);
        }
    double M = 10000.0;
#pragma omp parallel for schedule(static) if (props.Threads > 1)
    for (int i = 0; i < l; i++) {
        Da[i] = M;
        Day[i] = ds.y[i] * M;
        for (int j = 0; j < m; j++) {
            double kv = kernelFunction(ds, i, idx[j], props);
            KSC[(size_t)i * m + j] = kv;
            KSCA[(size_t)i * m + j] = kv;
        }
    }
    double *K1 = (double *)calloc((size_t)m * m, sizeof(double));
    double *K2 = (double *)calloc(m, sizeof(double));
    double *beta = (double *)calloc(m, sizeof(double));
    double *bnew = (double *)calloc(m, sizeof(double));
    double *bbest = (double *)calloc(m, sizeof(double));
    double *e = (double *)calloc(l, sizeof(double));
    int *act = (int *)calloc(l, sizeof(int));
    char nn = 'N', tt = 'T';
    int one = 1;
    double fone = 1.0, mone = -1.0, zero = 0.0;
    double dW = 1e9, nW = 1.0, old = 0.0, best = 1e9;
    int iter = 0, since_best = 0;
    const int parts = (m < props.Threads) ? m : props.Threads;
    int nsv = l;
    while ((iter < 500) && (dW / nW > 1e-6) && (since_best < 5)) {
        memcpy(K1, KC, (size_t)m * m * sizeof(double));
        if (nsv > 0) {
#pragma omp parallel for schedule(static) if (parts > 1)
            for (int p = 0; p < parts; p++) {
                int c0 = (int)round(p * m / parts), c1 = (int)round((p + 1) * m / parts) - 1;
                int len = c1 - c0 + 1, mm = m, ns = nsv;
                if (len > 0) {
                    scipy_dgemm_(&nn, &nn, &len, &one, &ns, &fone, &KSCA[c0], &mm, Day, &ns, &zero, &K2[c0], &mm);
                    scipy_dgemm_(&nn, &tt, &len, &mm, &ns, &fone, &KSCA[c0], &mm, KSCA, &mm, &fone, &K1[c0], &mm);
                }
            }
        } else {
            memset(K2, 0, m * sizeof(double));
        }
        memset(bnew, 0, m * sizeof(double));
        port_linear_system(K1, m, K2, bnew);
        dW = 0.0;
        nW = 0.0;
        for (int i = 0; i < m; i++) {
            double d = bnew[i] - beta[i];
            dW += d * d;
            nW += bnew[i] * bnew[i];
            beta[i] = bnew[i];
        }
        memcpy(e, ds.y, l * sizeof(double));
#pragma omp parallel for schedule(static) if (parts > 1)
        for (int p = 0; p < parts; p++) {
            int r0 = (int)round(p * l / parts), r1 = (int)round((p + 1) * l / parts) - 1;
            int len = r1 - r0 + 1, mm = m;
            if (len > 0) scipy_dgemm_(&nn, &nn, &one, &len, &mm, &mone, beta, &one, &KSC[(size_t)r0 * m], &mm, &fone, &e[r0], &one);
        }
#pragma omp parallel for schedule(static) if (props.Threads > 1)
        for (int i = 0; i < l; i++) {
            if (e[i] * ds.y[i] < 0.0) Da[i] = 0.0;
            else Da[i] = 1.0 * props.C / (ds.y[i] * e[i]);
            if (Da[i] > M) Da[i] = M;
        }
        nsv = 0;
        for (int i = 0; i < l; i++)
            if (Da[i] != 0.0) act[nsv++] = i;
#pragma omp parallel for schedule(static) if (props.Threads > 1)
        for (int i = 0; i < nsv; i++) {
            const double s = sqrt(Da[act[i]]);
            for (int j = 0; j < m; j++) KSCA[(size_t)i * m + j] = s * KSC[(size_t)act[i] * m + j];
            Day[i] = sqrt(Da[act[i]]) * ds.y[act[i]];
        }
        ++iter;
        if (props.verbose == 1) printf("Iteration %d, nSVs %d, ||deltaW||^2/||W||^2=%f\n", iter, nsv, dW / nW);
        if (iter > 10 && dW / nW > 100 * old) M = M / 10.0;
        old = dW / nW;
        if (dW / nW < best) {
            best = dW / nW;
            since_best = 0;
            memcpy(bbest, bnew, m * sizeof(double));
        } else {
            since_best += 1;
        }
    }
    free(KC); free(KSC); free(KSCA); free(Da); free(Day); free(K1); free(K2);
    free(beta); free(bnew); free(e); free(act);
    return bbest;
}

/* ------------------------------------------------------------------------ */
/* Prediction: src/LIBIRWLS-predict.c:56-131                                 */
/* ------------------------------------------------------------------------ */

static double *predict_rows(svm_dataset ds, model m, predictProperties props, int hard) {
    double *out = (double *)malloc((ds.l > 0 ? ds.l : 1) * sizeof(double));
#pragma omp parallel for schedule(static) if (props.Threads > 1)
    for (int i = 0; i < ds.l; i++) {
        double f = m.bias;
        for (int j = 0; j < m.nSVs; j++) f += (m.weights[j]) * kernelTest(ds, i, m, j);
        out[i] = hard ? ((f >= 0.0) ? 1.0 : -1.0) : f;
    }
    if (props.Labels == 1) {
        double hits = 0.0;
        for (int i = 0; i < ds.l; i++) {
            if (out[i] > 0 && ds.y[i] > 0) hits++;
            if (out[i] <= 0 && ds.y[i] <= 0) hits++;
        }
        printf("Accuracy: %f\n", hits / (double)ds.l);
    }
    return out;
}
double *softTest(svm_dataset ds, model m, predictProperties props) { return predict_rows(ds, m, props, 0); }
double *test(svm_dataset ds, model m, predictProperties props) { return predict_rows(ds, m, props, 1); }

/* ------------------------------------------------------------------------ */
/* Timing hooks for the CPU baseline of the benchmark (not reference API).   */
/* ------------------------------------------------------------------------ */

static double now_s(void) {
    struct timespec t;
    clock_gettime(CLOCK_MONOTONIC, &t);
    return t.tv_sec + 1e-9 * t.tv_nsec;
}

/* Times `nsteps` SGMA steps at order s0 (the loop body of SGMA above:
 * candidates drawn and scored, the best one's kernel column built); the
 * first step is untimed. The
 * starting centroids are the first s0 of a rand() permutation, their kernel
 * columns and the Cholesky factor of K_CC + jitter are built untimed.
 * Returns the mean seconds per step. */
double port_sgma_step_seconds(svm_dataset ds, properties props, int s0, int nsteps) {
    const int l = ds.l, NC = 64, m = s0 + nsteps;
    properties pr = props;
    pr.size = s0;
    int *start = randomCentroids(ds, pr);
    int *cent = (int *)malloc(m * sizeof(int));
    memcpy(cent, start, s0 * sizeof(int));
    free(start);
    double *KSC = (double *)malloc((size_t)l * m * sizeof(double));
    double *L = (double *)calloc((size_t)m * m, sizeof(double));
    double *KC = (double *)calloc((size_t)s0 * s0, sizeof(double));
#pragma omp parallel for schedule(static) if (props.Threads > 1)
    for (int r = 0; r < l; r++)
        for (int s = 0; s < s0; s++) KSC[(size_t)s * l + r] = kernelFunction(ds, r, cent[s], props);
    for (int a = 0; a < s0; a++)
        for (int b = 0; b < s0; b++) KC[(size_t)b * s0 + a] = kernelFunction(ds, cent[a], cent[b], props) + (a == b ? 1e-5 : 0.0);
    {
        char lo = 'L';
        int n = s0, info = 0;
        scipy_dpotrf_(&lo, &n, KC, &n, &info);
        for (int c = 0; c < s0; c++)
            for (int r = c; r < s0; r++) L[(size_t)c * s0 + r] = KC[(size_t)c * s0 + r];
    }
    free(KC);
    double *KNC = (double *)malloc((size_t)NC * m * sizeof(double));
    double *KSM = (double *)malloc((size_t)NC * l * sizeof(double));
    double *Z = (double *)malloc((size_t)NC * m * sizeof(double));
    double score[64], eta[64];
    int cand[64];
    double t0 = now_s();
    for (int s = s0; s < s0 + nsteps; s++) {
        if (s == s0 + 1) t0 = now_s();  /* the first step warms caches and threads, untimed */
        for (int i = 0; i < NC; i++) {
            const double want = (i % 2) * 2.0 - 1;
            int pick = rand() % l;
            while (ds.y[pick] != want) pick = rand() % l;
            cand[i] = pick;
        }
#pragma omp parallel for schedule(static) if (props.Threads > 1)
        for (int i = 0; i < NC; i++) {
            double *ksm = KSM + (size_t)i * l, *knc = KNC + (size_t)i * m, *z = Z + (size_t)i * m;
            for (int r = 0; r < l; r++) ksm[r] = kernelFunction(ds, cand[i], r, props);
            for (int r = 0; r < s0; r++) {
                double v = kernelFunction(ds, cand[i], cent[r], props);
                knc[r] = v;
                z[r] = v;
            }
            char lo = 'L', nn = 'N';
            int ss = s0, one = 1, info = 0, ll = l;
            double fone = 1.0, mone = -1.0;
            /* every timed step works at order s0 (the factor is not grown), so
               the mean is the cost of one SGMA step with s0 centroids */
            scipy_dpotrs_(&lo, &ss, &one, L, &ss, z, &ss, &info);
            double v = 1.0;
            for (int r = 0; r < s0; r++) v = v - (knc[r] * z[r]);
            eta[i] = v;
            scipy_dgemm_(&nn, &nn, &ll, &one, &ss, &fone, KSC, &ll, z, &ss, &mone, ksm, &ll);
            double acc = 0.0;
            for (int r = 0; r < l; r++) acc += ksm[r] * ksm[r];
            score[i] = (eta[i] > 0.0) ? (1.0 / eta[i]) * acc : 0.0;
        }
        int best = 0;
        for (int i = 1; i < NC; i++)
            if (score[i] > score[best]) best = i;
        cent[s] = cand[best];
#pragma omp parallel for schedule(static) if (props.Threads > 1)
        for (int r = 0; r < l; r++) KSC[(size_t)s * l + r] = kernelFunction(ds, r, cent[s], props);
    }
    const double dt = (now_s() - t0) / (nsteps > 1 ? nsteps - 1 : 1);
    free(cent); free(KSC); free(L); free(KNC); free(KSM); free(Z);
    return dt;
}

/* Times IRWLSpar's pieces on the given centroids: out[0] = seconds of the
 * kernel-matrix build (KC and K_nm), out[1] = seconds of the first iteration
 * (Gram dgemm over all rows, solve, residual dgemm, weights), out[2] = mean
 * seconds of iterations 2..iters (Gram over the active rows only). */
void port_irwls_seconds(svm_dataset ds, int *idx, properties props, int iters, double *out) {
    const int m = props.size, l = ds.l;
    double *KC = (double *)calloc((size_t)m * m, sizeof(double));
    double *KSC = (double *)calloc((size_t)l * m, sizeof(double));
    double *KSCA = (double *)calloc((size_t)l * m, sizeof(double));
    double *Da = (double *)calloc(l, sizeof(double));
    double *Day = (double *)calloc(l, sizeof(double));
    const double t0 = now_s();
#pragma omp parallel for schedule(static) if (props.Threads > 1)
    for (int i = 0; i < m; i++)
        for (int j = 0; j < m; j++) KC[(size_t)i * m + j] = kernelFunction(ds, idx[i], idx[j], props) + (i == j ? 1e-5 : 0.0);
    const double M = 10000.0;
#pragma omp parallel for schedule(static) if (props.Threads > 1)
    for (int i = 0; i < l; i++) {
        Da[i] = M;
        Day[i] = ds.y[i] * M;
        for (int j = 0; j < m; j++) {
            double kv = kernelFunction(ds, i, idx[j], props);
            KSC[(size_t)i * m + j] = kv;
            KSCA[(size_t)i * m + j] = kv;
        }
    }
    out[0] = now_s() - t0;
    double *K1 = (double *)calloc((size_t)m * m, sizeof(double));
    double *K2 = (double *)calloc(m, sizeof(double));
    double *beta = (double *)calloc(m, sizeof(double));
    double *e = (double *)calloc(l, sizeof(double));
    int *act = (int *)calloc(l, sizeof(int));
    char nn = 'N', tt = 'T';
    int one = 1, nsv = l;
    double fone = 1.0, mone = -1.0, zero = 0.0;
    const int parts = (m < props.Threads) ? m : props.Threads;
    double t1 = now_s();
    for (int it = 0; it < iters; it++) {
        if (it == 1) {
            out[1] = now_s() - t1;
            t1 = now_s();
        }
        memcpy(K1, KC, (size_t)m * m * sizeof(double));
#pragma omp parallel for schedule(static) if (parts > 1)
        for (int p = 0; p < parts; p++) {
            int c0 = (int)round(p * m / parts), c1 = (int)round((p + 1) * m / parts) - 1;
            int len = c1 - c0 + 1, mm = m, ns = nsv;
            if (len > 0) {
                scipy_dgemm_(&nn, &nn, &len, &one, &ns, &fone, &KSCA[c0], &mm, Day, &ns, &zero, &K2[c0], &mm);
                scipy_dgemm_(&nn, &tt, &len, &mm, &ns, &fone, &KSCA[c0], &mm, KSCA, &mm, &fone, &K1[c0], &mm);
            }
        }
        port_linear_system(K1, m, K2, beta);
        memcpy(e, ds.y, l * sizeof(double));
#pragma omp parallel for schedule(static) if (parts > 1)
        for (int p = 0; p < parts; p++) {
            int r0 = (int)round(p * l / parts), r1 = (int)round((p + 1) * l / parts) - 1;
            int len = r1 - r0 + 1, mm = m;
            if (len > 0) scipy_dgemm_(&nn, &nn, &one, &len, &mm, &mone, beta, &one, &KSC[(size_t)r0 * m], &mm, &fone, &e[r0], &one);
        }
        for (int i = 0; i < l; i++) {
            Da[i] = (e[i] * ds.y[i] < 0.0) ? 0.0 : 1.0 * props.C / (ds.y[i] * e[i]);
            if (Da[i] > M) Da[i] = M;
        }
        nsv = 0;
        for (int i = 0; i < l; i++)
            if (Da[i] != 0.0) act[nsv++] = i;
#pragma omp parallel for schedule(static) if (props.Threads > 1)
        for (int i = 0; i < nsv; i++) {
            const double s = sqrt(Da[act[i]]);
            for (int j = 0; j < m; j++) KSCA[(size_t)i * m + j] = s * KSC[(size_t)act[i] * m + j];
            Day[i] = sqrt(Da[act[i]]) * ds.y[act[i]];
        }
    }
    if (iters > 1) out[2] = (now_s() - t1) / (iters - 1);
    else out[1] = now_s() - t1;
    free(KC); free(KSC); free(KSCA); free(Da); free(Day); free(K1); free(K2); free(beta); free(e); free(act);
}
