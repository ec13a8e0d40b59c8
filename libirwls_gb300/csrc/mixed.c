/*
 * mixed.c -- host orchestration of the precision form of budgeted IRWLS
 * (same loops, exit tests and random draws as budgeted_train.c):
 *   SGMA: candidate kernel rows, the factor L of K_CC + jitter and its
 *         inverse (kept explicitly, as the reference keeps invKC) in FP64;
 *         the candidate solves W = K_CN L^-T as one FP64 GEMM; scores from
 *         Q w on the tensor cores (Q = K_nm L^-T and W held as three bf16
 *         pieces each, exactly their FP32 values; six piece products, so
 *         Q w has FP32 accuracy), candidate kernel rows of the score
 *         epilogue in FP32; each new column of Q taken from the score
 *         step's residuals of the winning candidate.
 *   IRWLSpar (budgeted_train.c, irwls_par_dev) forms its Gram on the tensor
 *   cores from exact integer digits of its operand (dev_gram_tc.cu); its
 *   factor, solves, residuals and convergence test stay FP64. Its system
 *   K1 = KC + K_nm^T D_a K_nm carries weights up to 1e4 against a 1e-5
 *   jitter, so its condition number reaches ~1e13: a Gram accumulated from
 *   16-bit-mantissa products (relative error ~1e-5) turns it indefinite
 *   (measured on 200000 rows and 1000 centroids, that variant's primal
 *   objective was off by a factor of 4e6), while the digit products' error
 *   (about 2^-45 of the column scales per row) keeps it definite.
 * Selected with irwls_set_precision(IRWLS_PRECISION_MIXED) or the
 * environment variable IRWLS_PRECISION=mixed; plain FP64 is the default.
 */
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "irwls_dev.h"
#include "irwls_gpu.h"

int irwls_sgma_cand_inv(const irwls_dev_set *X, const int *d_cand, const int *d_cent, int s, const double *d_Linv,
                        int ldi, double *d_KN, int ldz, double *d_wpart, int ldp, double *d_W, void *Wb, int ldq,
                        double *d_eta);
int irwls_sgma_linv_update(const double *d_L, int ldL, double *d_Linv, int ldi, int s, double *d_lpart,
                           float *d_lrow);
size_t irwls_sgma_wpart_count(int m);
size_t irwls_sgma_lpart_count(int m);
int irwls_sgma_tc_select(const float *d_part, int nblk, const double *d_eta, const int *d_cand, int s, int *d_cent,
                         int *d_best, double *d_bestval, float *d_scores);
int irwls_sgma_factor(const irwls_dev_set *X, int s, const int *d_cent, const int *d_best, const double *d_W, int ldz,
                      double *d_L, int ldL);
/* Qb, Wb: the blocked bf16 hi/mid/lo layout of Q and W (blocked_bf16.cuh);
   d_rq: the residuals r = Q w - k of every row against the step's 64
   candidates (64 x rows, candidate-major) */
int irwls_sgma_tc_score(const irwls_dev_set *X, const void *F, int l, const int *d_cand, const void *Qb, int ldq,
                        const void *Wb, int s, float *d_part, float *d_rq);
int irwls_sgma_tc_partials(int l);
int irwls_q_column(const irwls_dev_set *X, const void *F, int l, const int *d_cent, int s, const float *lrow, void *Qb,
                   int ldq, float *d_qn);
int irwls_q_column_resid(int l, const float *d_rq, const int *d_best, int s, const float *lrow, void *Qb, int ldq,
                         float *d_qn);
void *irwls_f32_mirror(const irwls_dev_set *X);
void irwls_f32_mirror_free(void *h);
void irwls_f32_mirror_view(const void *h, const float **X, const float **q);
int irwls_learn_features(const float *X, int ld, int width, int raw, const float *q, float ng, const double *y,
                         const int *d_cand, int nc, const int *d_probe, int np, const float *d_qn, float *d_F);
int irwls_learn_predict(void *mlp, const float *d_F, int n, float *d_pred);
int irwls_learn_topk(const float *d_pred, const int *d_pool, int half, int keep, int nrand, int *d_out);
int irwls_learn_residual_trace(const float *d_qn, int l, double *d_out);
int irwls_mlp_feature_count(void);
int *irwls_draw_sgma_candidates(const svm_dataset *ds, int m);
void irwls_record_run_info(int par_iterations, int active_rows);

static int g_precision = -1;

void irwls_set_precision(int mode) { g_precision = mode; }

int irwls_get_precision(void) {
    if (g_precision < 0) {
        const char *e = getenv("IRWLS_PRECISION");
        g_precision = (e && strcmp(e, "mixed") == 0) ? IRWLS_PRECISION_MIXED : IRWLS_PRECISION_FP64;
    }
    return g_precision;
}

static int round_up(int x, int a) { return (x + a - 1) / a * a; }

/* Learned-proposal form: the network, its pool per step, the probe rows of
 * the features, and trace outputs (host arrays of (m - 2) x 64 x features and
 * (m - 2) x 64 exact scores) when a trace is being recorded. */
enum { NPROBE = 1024, NCAND = 64, NRANDOM = 8 };
static void *g_proposer = NULL;
static int g_pool = 4096;
static float *g_trace_feat = NULL, *g_trace_score = NULL;
static double g_last_residual = -1.0;

void irwls_set_sgma_proposer(void *mlp, int pool) {
    g_proposer = mlp;
    if (pool < 2 * NCAND) pool = 2 * NCAND;
    if (pool > 4096) pool = 4096;
    g_pool = pool & ~1;
}
double irwls_last_nystrom_residual(void) { return g_last_residual; }

/* n row indices with label `want`, drawn uniformly with the context's rand(). */
static void draw_label_rows(const svm_dataset *ds, double want, int n, int *out) {
    for (int k = 0; k < n; k++) {
        int pick = irwls_rand() % ds->l;
        while (ds->y[pick] != want) pick = irwls_rand() % ds->l;
        out[k] = pick;
    }
}

int irwls_sgma_mixed_dev(const irwls_dev_set *X, const svm_dataset *ds, properties props, int *cent_out) {
    const int m = props.size, l = ds->l;
    if (m <= 0) return 0;
    int *cand = irwls_draw_sgma_candidates(ds, m);
    if (!cand) return -1;
    const int ldq = round_up(m, 128), ldL = m, ldz = m;
    const int nblk = irwls_sgma_tc_partials(l);
    int rc = 0;
    int *d_cand = NULL, *d_cent = NULL, *d_best = NULL;
    double *d_L = NULL, *d_W = NULL, *d_KN = NULL, *d_eta = NULL, *d_val = NULL, *d_Linv = NULL, *d_wpart = NULL,
           *d_lpart = NULL;
    float *d_part = NULL;
    float *d_rq = NULL, *lrow = NULL, *d_qn = NULL, *d_F = NULL, *d_pred = NULL, *d_tfeat = NULL, *d_tscore = NULL;
    int *d_probe = NULL, *d_pool = NULL;
    double *d_resid = NULL;
    void *Qb = NULL, *Wb = NULL;
    /* proposals and traces need the RBF kernel's k(x, x) = 1 */
    const int learn = g_proposer != NULL && X->mode != IRWLS_K_LINEAR && m > 2;
    const int trace = g_trace_feat != NULL && m > 2;
    const int nf = irwls_mlp_feature_count(), pool = g_pool, half = g_pool / 2;
    void *F = irwls_f32_mirror(X);
    if (!F) {
        free(cand);
        return -1;
    }
    rc |= irwls_dev_malloc((void **)&d_cand, (size_t)m * 64 * sizeof(int));
    rc |= irwls_dev_malloc((void **)&d_cent, (size_t)m * sizeof(int));
    rc |= irwls_dev_malloc((void **)&d_best, sizeof(int));
    rc |= irwls_dev_malloc((void **)&d_L, (size_t)m * ldL * sizeof(double));
    rc |= irwls_dev_malloc((void **)&d_W, (size_t)64 * ldz * sizeof(double));
    rc |= irwls_dev_malloc((void **)&d_KN, (size_t)64 * ldz * sizeof(double));
    rc |= irwls_dev_malloc((void **)&d_eta, 64 * sizeof(double));
    rc |= irwls_dev_malloc((void **)&d_part, (size_t)nblk * 64 * sizeof(float));
    rc |= irwls_dev_malloc((void **)&d_val, (size_t)m * sizeof(double));
    rc |= irwls_dev_malloc((void **)&d_rq, (size_t)l * 64 * sizeof(float));
    const size_t qb_bytes = (size_t)nblk * 128 * ldq * 6; /* whole 128-row tiles, three pieces */
    rc |= irwls_dev_malloc(&Qb, qb_bytes);
    rc |= irwls_dev_malloc(&Wb, (size_t)64 * ldq * 6);
    rc |= irwls_dev_malloc((void **)&lrow, (size_t)(m + 1) * sizeof(float));
    rc |= irwls_dev_malloc((void **)&d_Linv, (size_t)m * ldL * sizeof(double));
    rc |= irwls_dev_malloc((void **)&d_wpart, irwls_sgma_wpart_count(m) * sizeof(double));
    rc |= irwls_dev_malloc((void **)&d_lpart, irwls_sgma_lpart_count(m) * sizeof(double));
    rc |= irwls_dev_malloc((void **)&d_qn, (size_t)(l + 2) * sizeof(float));
    rc |= irwls_dev_malloc((void **)&d_resid, sizeof(double));
    if (learn || trace) {
        rc |= irwls_dev_malloc((void **)&d_probe, NPROBE * sizeof(int));
        rc |= irwls_dev_malloc((void **)&d_F, (size_t)pool * nf * sizeof(float));
    }
    if (learn) {
        rc |= irwls_dev_malloc((void **)&d_pool, (size_t)m * pool * sizeof(int));
        rc |= irwls_dev_malloc((void **)&d_pred, (size_t)pool * sizeof(float));
    }
    if (trace) {
        rc |= irwls_dev_malloc((void **)&d_tfeat, (size_t)(m - 2) * NCAND * nf * sizeof(float));
        rc |= irwls_dev_malloc((void **)&d_tscore, (size_t)(m - 2) * NCAND * sizeof(float));
    }
    if (rc) goto done;
    {
        int first[2] = {l, l + 1};
        rc |= irwls_dev_h2d(d_cand, cand, (size_t)m * 64 * sizeof(int));
        rc |= irwls_dev_h2d(d_cent, first, (m > 1 ? 2 : 1) * sizeof(int));
        rc |= irwls_dev_memset(d_L, 0, (size_t)m * ldL * sizeof(double));
        rc |= irwls_dev_memset(d_Linv, 0, (size_t)m * ldL * sizeof(double));
        rc |= irwls_dev_memset(d_W, 0, (size_t)64 * ldz * sizeof(double));
        rc |= irwls_dev_memset(Qb, 0, qb_bytes);
        rc |= irwls_dev_memset(d_qn, 0, (size_t)(l + 2) * sizeof(float));
        if (learn || trace) {
            /* probe rows and the proposal pools, drawn after the reference's
               candidates so that those stay the plain run's */
            int *hp = (int *)malloc((size_t)(learn ? m * pool : NPROBE) * sizeof(int) + NPROBE * sizeof(int));
            int *probe = hp + (learn ? (size_t)m * pool : 0);
            for (int k = 0; k < NPROBE; k++) probe[k] = irwls_rand() % l;
            rc |= irwls_dev_h2d(d_probe, probe, NPROBE * sizeof(int));
            if (learn) {
                memset(hp, 0, (size_t)2 * pool * sizeof(int));
                for (int st = 2; st < m; st++) {
                    draw_label_rows(ds, -1.0, half, hp + (size_t)st * pool);
                    draw_label_rows(ds, 1.0, half, hp + (size_t)st * pool + half);
                }
                rc |= irwls_dev_h2d(d_pool, hp, (size_t)m * pool * sizeof(int));
            }
            rc |= irwls_dev_sync();
            free(hp);
        }
        /* centroids 0 and 1 are the class means (src/budgeted-train.c:127-147) */
        for (int s = 0; s < 2 && s < m && !rc; s++) {
            rc |= irwls_sgma_factor(X, s, d_cent, d_best, d_W, ldz, d_L, ldL);
            rc |= irwls_sgma_linv_update(d_L, ldL, d_Linv, ldL, s, d_lpart, lrow);
            rc |= irwls_q_column(X, F, l, d_cent, s, lrow, Qb, ldq, d_qn);
        }
        const float *X32 = NULL, *q32 = NULL;
        irwls_f32_mirror_view(F, &X32, &q32);
        const int raw = X->mode == IRWLS_K_RAW_RBF;
        for (int s = 2; s < m && !rc; s++) {
            int *cs = d_cand + (size_t)s * 64;
            if (learn) {
                /* the network scores the step's pool; per label its best 24
                   and 8 random pool entries replace the step's candidates */
                rc |= irwls_learn_features(X32, X->ld, X->width, raw, q32, (float)X->neg_gamma, X->y,
                                           d_pool + (size_t)s * pool, pool, d_probe, NPROBE, d_qn, d_F);
                rc |= irwls_learn_predict(g_proposer, d_F, pool, d_pred);
                rc |= irwls_learn_topk(d_pred, d_pool + (size_t)s * pool, half, NCAND / 2 - NRANDOM, NRANDOM, cs);
            }
            if (trace)
                rc |= irwls_learn_features(X32, X->ld, X->width, raw, q32, (float)X->neg_gamma, X->y, cs, NCAND,
                                           d_probe, NPROBE, d_qn, d_tfeat + (size_t)(s - 2) * NCAND * nf);
            rc |= irwls_sgma_cand_inv(X, cs, d_cent, s, d_Linv, ldL, d_KN, ldz, d_wpart, m, d_W, Wb, ldq, d_eta);
            rc |= irwls_sgma_tc_score(X, F, l, cs, Qb, ldq, Wb, s, d_part, d_rq);
            irwls_prof_begin(IRWLS_PROF_SGMA_UPDATE);
            rc |= irwls_sgma_tc_select(d_part, nblk, d_eta, cs, s, d_cent, d_best, d_val,
                                       trace ? d_tscore + (size_t)(s - 2) * NCAND : NULL);
            rc |= irwls_sgma_factor(X, s, d_cent, d_best, d_W, ldz, d_L, ldL);
            rc |= irwls_sgma_linv_update(d_L, ldL, d_Linv, ldL, s, d_lpart, lrow);
            rc |= irwls_q_column_resid(l, d_rq, d_best, s, lrow, Qb, ldq, d_qn);
            irwls_prof_end(IRWLS_PROF_SGMA_UPDATE);
        }
        /* Nystrom residual trace(K - K_nm K_mm^-1 K_mn) = sum_i (k_ii - |Q_i|^2) */
        g_last_residual = -1.0;
        if (!rc && X->mode != IRWLS_K_LINEAR && !irwls_learn_residual_trace(d_qn, l, d_resid))
            rc |= irwls_dev_d2h(&g_last_residual, d_resid, sizeof(double));
        if (!rc && trace) {
            rc |= irwls_dev_d2h(g_trace_feat, d_tfeat, (size_t)(m - 2) * NCAND * nf * sizeof(float));
            rc |= irwls_dev_d2h(g_trace_score, d_tscore, (size_t)(m - 2) * NCAND * sizeof(float));
        }
        if (rc) goto done;
        double *val = (double *)malloc((size_t)m * sizeof(double));
        rc |= irwls_dev_d2h(cent_out, d_cent, (size_t)m * sizeof(int));
        rc |= irwls_dev_d2h(val, d_val, (size_t)m * sizeof(double));
        rc |= irwls_dev_sync();
        if (!rc) {
            const int tc = irwls_tc_status();
            if (tc) {
                irwls_set_error(-13, "a tensor-core pipeline wait ran out (code %d)", tc);
                rc = -13;
            }
        }
        if (!rc && props.verbose == 1) {
            for (int s = 0; s < m; s++) {
                if (s == 0) printf("Best Error Descent %f, Average of positive data is centroid %d\n", 1.0, s);
                if (s == 1) printf("Best Error Descent %f, Average of negative data is centroid %d\n", 1.0, s);
                if (s > 1) printf("Best Error Descent %f, Data with index %d is centroid %d\n", val[s], cent_out[s], s);
            }
        }
        free(val);
    }
done:
    free(cand);
    {
        void *bufs[] = {d_cand, d_cent, d_best, d_L, d_W, d_KN, d_eta, d_part, d_val, d_rq, Qb, Wb, lrow,
                        d_Linv, d_wpart, d_lpart, d_qn, d_resid, d_probe, d_F, d_pool, d_pred, d_tfeat, d_tscore};
        for (size_t k = 0; k < sizeof bufs / sizeof bufs[0]; k++) irwls_dev_free(bufs[k]);
        irwls_f32_mirror_free(F);
    }
    return rc ? -1 : 0;
}

/* Records the features and exact scores of the candidates of a precision-form
 * SGMA run on `dataset` (RBF): the random ones, or with a proposer installed
 * the ones it proposes (on-policy traces). feat gets (size - 2) x 64 x
 * irwls_mlp_feature_count() values, score (size - 2) x 64. */
int irwls_sgma_traces(svm_dataset dataset, properties props, float *feat, float *score) {
    irwls_clear_error();
    if (props.size <= 2 || props.kernelType == 0) {
        irwls_set_error(-9, "traces need an RBF kernel and a budget above 2");
        return -9;
    }
    g_trace_feat = feat;
    g_trace_score = score;
    irwls_dev_set X;
    int rc = irwls_check_labels(&dataset, dataset.l);
    if (!rc) rc = irwls_dev_upload(&dataset, dataset.l + 2, props.kernelType, props.Kgamma, 0, 0, &X);
    if (!rc) {
        int *cent = (int *)malloc((size_t)props.size * sizeof(int));
        rc = irwls_sgma_mixed_dev(&X, &dataset, props, cent);
        free(cent);
        irwls_dev_release(&X);
    }
    g_trace_feat = g_trace_score = NULL;
    return rc;
}
