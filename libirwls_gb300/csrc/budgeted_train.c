/*
 * budgeted_train.c -- host orchestration of budgeted IRWLS on the GPU:
 * SGMA centroid selection (reference src/budgeted-train.c:114-309), random
 * centroids (:73-100), IRWLSpar (:324-505) and the model packing (:519-570).
 *
 * SGMA's 64 candidates per step are drawn with rand() (irwls_rand: libc's on
 * the main thread, an identical per-thread generator in batch workers) in
 * exactly the order of the reference run with one thread. The draws depend only on the
 * labels, so all of them are made before the first kernel is launched and
 * the whole selection runs without a host synchronisation; the per-step
 * "Best Error Descent" lines are printed from device records at the end.
 */
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "budgeted-train.h"
#include "irwls_dev.h"
#include "irwls_gpu.h"

int *randomCentroids(svm_dataset dataset, properties props) {
    int *p = (int *)malloc((dataset.l > 0 ? dataset.l : 1) * sizeof(int));
    for (int i = 0; i < dataset.l; ++i) p[i] = i;
    for (int i = dataset.l - 1; i >= 0; --i) {
        const int j = irwls_rand() % (i + 1);
        const int t = p[i];
        p[i] = p[j];
        p[j] = t;
    }
    int *c = (int *)malloc((props.size > 0 ? props.size : 1) * sizeof(int));
    for (int i = 0; i < props.size; i++) c[i] = p[i];
    free(p);
    return c;
}

int irwls_sgma_mixed_dev(const irwls_dev_set *X, const svm_dataset *ds, properties props, int *cent_out);

/* Candidate draws of every SGMA step s >= 2 (src/budgeted-train.c:157-167):
 * candidate i must carry label (i % 2) * 2 - 1. */
int *irwls_draw_sgma_candidates(const svm_dataset *ds, int m) {
    int have_pos = 0, have_neg = 0;
    for (int i = 0; i < ds->l && !(have_pos && have_neg); i++) {
        if (ds->y[i] == 1.0) have_pos = 1;
        if (ds->y[i] == -1.0) have_neg = 1;
    }
    if (m > 2 && !(have_pos && have_neg)) {
        irwls_set_error(-9, "SGMA needs samples labelled +1 and -1");
        return NULL;
    }
    int *cand = (int *)malloc((size_t)(m > 0 ? m : 1) * 64 * sizeof(int));
    for (int s = 2; s < m; s++)
        for (int i = 0; i < 64; i++) {
            const double want = (i % 2) * 2.0 - 1;
            int pick = irwls_rand() % (ds->l);
            while (ds->y[pick] != want) pick = irwls_rand() % (ds->l);
            cand[(size_t)s * 64 + i] = pick;
        }
    return cand;
}

/* SGMA on a resident dataset (rows l and l+1 are the class means). */
int irwls_sgma_dev(const irwls_dev_set *X, const svm_dataset *ds, properties props, int *cent_out) {
    const int m = props.size, l = ds->l;
    if (m <= 0) return 0;
    if (irwls_get_precision() == IRWLS_PRECISION_MIXED) return irwls_sgma_mixed_dev(X, ds, props, cent_out);
    int *cand = irwls_draw_sgma_candidates(ds, m);
    if (!cand) return -1;
    int rc = 0;
    int *d_cand = NULL, *d_cent = NULL, *d_best = NULL;
    double *d_L = NULL, *d_KSC = NULL, *d_W = NULL, *d_Z = NULL, *d_KN = NULL, *d_eta = NULL, *d_part = NULL,
           *d_val = NULL;
    const int ldz = m, ldL = m;
    rc |= irwls_dev_malloc((void **)&d_cand, (size_t)m * 64 * sizeof(int));
    rc |= irwls_dev_malloc((void **)&d_cent, (size_t)m * sizeof(int));
    rc |= irwls_dev_malloc((void **)&d_best, sizeof(int));
    rc |= irwls_dev_malloc((void **)&d_L, (size_t)m * ldL * sizeof(double));
    rc |= irwls_dev_malloc((void **)&d_KSC, (size_t)l * m * sizeof(double));
    rc |= irwls_dev_malloc((void **)&d_W, (size_t)64 * ldz * sizeof(double));
    rc |= irwls_dev_malloc((void **)&d_Z, (size_t)64 * ldz * sizeof(double));
    rc |= irwls_dev_malloc((void **)&d_KN, (size_t)64 * ldz * sizeof(double));
    rc |= irwls_dev_malloc((void **)&d_eta, 64 * sizeof(double));
    rc |= irwls_dev_malloc((void **)&d_part, (size_t)irwls_sgma_partials(l) * 64 * sizeof(double));
    rc |= irwls_dev_malloc((void **)&d_val, (size_t)m * sizeof(double));
    if (rc) goto done;
    {
        int first[2] = {l, l + 1};
        rc |= irwls_dev_h2d(d_cand, cand, (size_t)m * 64 * sizeof(int));
        rc |= irwls_dev_h2d(d_cent, first, (m > 1 ? 2 : 1) * sizeof(int));
        rc |= irwls_dev_memset(d_L, 0, (size_t)m * ldL * sizeof(double));
        rc |= irwls_sgma_first(X, l, d_cent, d_L, ldL, d_KSC);
        if (m > 1) rc |= irwls_sgma_extend(X, l, 1, d_cent, d_best, d_W, ldz, d_L, ldL, d_KSC);
        for (int s = 2; s < m && !rc; s++) {
            rc |= irwls_sgma_score(X, l, d_cand + (size_t)s * 64, 64, d_cent, s, d_L, ldL, d_KSC, d_W, d_Z, d_KN,
                                   ldz, d_eta, d_part);
            irwls_prof_begin(IRWLS_PROF_SGMA_UPDATE);
            rc |= irwls_sgma_select(d_part, l, d_eta, d_cand + (size_t)s * 64, s, d_cent, d_best, d_val);
            rc |= irwls_sgma_extend(X, l, s, d_cent, d_best, d_W, ldz, d_L, ldL, d_KSC);
            irwls_prof_end(IRWLS_PROF_SGMA_UPDATE);
        }
        if (rc) goto done;
        double *val = (double *)malloc((size_t)m * sizeof(double));
        rc |= irwls_dev_d2h(cent_out, d_cent, (size_t)m * sizeof(int));
        rc |= irwls_dev_d2h(val, d_val, (size_t)m * sizeof(double));
        rc |= irwls_dev_sync();
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
    void *bufs[] = {d_cand, d_cent, d_best, d_L, d_KSC, d_W, d_Z, d_KN, d_eta, d_part, d_val};
    for (size_t k = 0; k < sizeof bufs / sizeof bufs[0]; k++) irwls_dev_free(bufs[k]);
    return rc ? -1 : 0;
}

static int g_last_iters = 0, g_last_nact = 0;
static double g_gram_flops = 0.0;
void irwls_last_run_info(int *par_iterations, int *active_rows) {
    *par_iterations = g_last_iters;
    *active_rows = g_last_nact;
}
double irwls_last_gram_flops(void) { return g_gram_flops; }
void irwls_record_run_info(int par_iterations, int active_rows) {
    g_last_iters = par_iterations;
    g_last_nact = active_rows;
}

/* IRWLSpar on a resident dataset; weights_out gets betaBest (m values). */
int irwls_par_dev(const irwls_dev_set *X, int l, const int *idx, properties props, double *weights_out) {
    const int m = props.size;
    const double C = props.C;
    if (m <= 0) return 0;
    int rc = 0;
    int *d_idx = NULL, *d_act = NULL, *d_nact = NULL, *h_nact = NULL;
    double *d_KC = NULL, *d_KSC = NULL, *d_K1 = NULL, *d_part = NULL, *d_sd = NULL, *d_day = NULL, *d_e = NULL,
           *d_Da = NULL, *d_beta = NULL, *d_bnew = NULL, *d_bbest = NULL, *d_nrm = NULL, *h_nrm = NULL;
    const int ld = m + 1;
    /* split-K chunks of the Gram update: about eight CTAs per SM over the
       lower tiles, with at least 512 rows per chunk */
    const int sms = 152;
    const int tiles = ((m + 64) / 64) * ((m + 63) / 64 + 1) / 2;
    int P = (8 * sms + tiles - 1) / tiles;
    if (P > l / 512) P = l / 512;
    if (P < 1) P = 1;
    if (P > 64) P = 64;
    /* precision form: the Gram on the tensor cores through exact integer
       digits of the active rows (dev_gram_tc.cu), which takes as many
       split-K chunks of the P allowed here as fill the SMs */
    const int mixed = irwls_get_precision() == IRWLS_PRECISION_MIXED;
    void *d_A = NULL;
    if (mixed) {
        P = (24 * sms + tiles - 1) / tiles;
        if (P > l / 256) P = l / 256;
        if (P < 1) P = 1;
        if (P > 128) P = 128;
        rc |= irwls_dev_malloc(&d_A, irwls_par_gram_tc_bytes(l, m));
    }
    rc |= irwls_dev_malloc((void **)&d_idx, (size_t)m * sizeof(int));
    rc |= irwls_dev_malloc((void **)&d_act, (size_t)l * sizeof(int));
    rc |= irwls_dev_malloc((void **)&d_nact, sizeof(int));
    rc |= irwls_dev_host_alloc((void **)&h_nact, sizeof(int));
    rc |= irwls_dev_malloc((void **)&d_KC, (size_t)m * m * sizeof(double));
    rc |= irwls_dev_malloc((void **)&d_KSC, (size_t)l * m * sizeof(double));
    rc |= irwls_dev_malloc((void **)&d_K1, (size_t)ld * ld * sizeof(double));
    rc |= irwls_dev_malloc((void **)&d_part, irwls_par_gram_part_bytes(m, P));
    rc |= irwls_dev_malloc((void **)&d_sd, (size_t)l * sizeof(double));
    rc |= irwls_dev_malloc((void **)&d_day, (size_t)l * sizeof(double));
    rc |= irwls_dev_malloc((void **)&d_e, (size_t)l * sizeof(double));
    rc |= irwls_dev_malloc((void **)&d_Da, (size_t)l * sizeof(double));
    rc |= irwls_dev_malloc((void **)&d_beta, (size_t)m * sizeof(double));
    rc |= irwls_dev_malloc((void **)&d_bnew, (size_t)m * sizeof(double));
    rc |= irwls_dev_malloc((void **)&d_bbest, (size_t)m * sizeof(double));
    rc |= irwls_dev_malloc((void **)&d_nrm, 2 * sizeof(double));
    rc |= irwls_dev_host_alloc((void **)&h_nrm, 2 * sizeof(double));
    if (rc) goto done;
    double M = 10000.0;
    rc |= irwls_dev_h2d(d_idx, idx, (size_t)m * sizeof(int));
    rc |= irwls_dev_memset(d_beta, 0, (size_t)m * sizeof(double));
    rc |= irwls_dev_memset(d_bbest, 0, (size_t)m * sizeof(double));
    rc |= irwls_par_build(X, l, d_idx, m, d_KC, d_KSC);
    rc |= irwls_par_first(X->y, l, M, d_act, d_sd, d_day);
    rc |= irwls_dev_sync();
    if (rc) goto done;
    {
        int iter = 0, since_best = 0, nact = l;
        g_gram_flops = 0.0;
        double dW = 1e9, nW = 1.0, old = 0.0, best = 1e9;
        while ((iter < 500) && (dW / nW > 1e-6) && (since_best < 5)) {
            /* K1 = KC + KSCA^T KSCA (lower) and K2 = KSCA^T Day in row m (:401-416) */
            if (mixed ? irwls_par_gram_tc(d_KSC, m, d_act, nact, d_sd, d_day, d_KC, d_K1, ld, d_part, P, d_A)
                      : irwls_par_gram(d_KSC, m, d_act, nact, d_sd, d_day, d_KC, d_K1, ld, d_part, P))
                goto fail;
            g_gram_flops += (double)nact * (m + 1) * m;
            if (irwls_dev_chol_solve(d_K1, m, ld, NULL, d_bnew)) goto fail;
            if (irwls_par_delta(d_bnew, d_beta, m, d_nrm)) goto fail;
            if (irwls_par_residual(d_KSC, l, m, d_beta, X->y, C, M, d_e, d_Da)) goto fail;
            if (irwls_par_weights(d_Da, X->y, l, d_act, d_sd, d_day, d_nact)) goto fail;
            if (irwls_dev_d2h(h_nrm, d_nrm, 2 * sizeof(double)) || irwls_dev_d2h(h_nact, d_nact, sizeof(int)) ||
                irwls_dev_sync())
                goto fail;
            dW = h_nrm[0];
            nW = h_nrm[1];
            nact = *h_nact;
            ++iter;
            if (props.verbose == 1) printf("Iteration %d, nSVs %d, ||deltaW||^2/||W||^2=%f\n", iter, nact, dW / nW);
            if (iter > 10 && dW / nW > 100 * old) M = M / 10.0;
            old = dW / nW;
            if (dW / nW < best) {
                best = dW / nW;
                since_best = 0;
                if (irwls_dev_d2d(d_bbest, d_bnew, (size_t)m * sizeof(double))) goto fail;
            } else {
                since_best += 1;
            }
        }
        g_last_iters = iter;
        g_last_nact = nact;
    }
    if (irwls_dev_d2h(weights_out, d_bbest, (size_t)m * sizeof(double)) || irwls_dev_sync()) goto fail;
    if (mixed) {
        const int tc = irwls_tc_status();
        if (tc) {
            irwls_set_error(-13, "a tensor-core pipeline wait of the Gram ran out (code %d)", tc);
            goto fail;
        }
    }
    goto done;
fail:
    rc = -1;
done:
    {
        void *bufs[] = {d_idx, d_act, d_nact, d_KC, d_KSC, d_K1, d_part, d_sd, d_day, d_e, d_Da, d_beta, d_bnew,
                        d_bbest, d_nrm, d_A};
        for (size_t k = 0; k < sizeof bufs / sizeof bufs[0]; k++) irwls_dev_free(bufs[k]);
        irwls_dev_host_free(h_nact);
        irwls_dev_host_free(h_nrm);
    }
    return rc ? -1 : 0;
}

/* Rows the budgeted path may touch: the l samples plus, when the dataset
 * carries them, the two class-mean rows. */
static int budget_rows(const svm_dataset *ds, const int *idx, int m) {
    int n = ds->l;
    if (idx)
        for (int i = 0; i < m; i++)
            if (idx[i] + 1 > n) n = idx[i] + 1;
    return n;
}

int *SGMA(svm_dataset dataset, properties props) {
    irwls_clear_error();
    irwls_dev_set X;
    if (irwls_check_labels(&dataset, dataset.l) || irwls_dev_upload(&dataset, dataset.l + 2, props.kernelType, props.Kgamma, 0, 0, &X)) return NULL;
    int *cent = (int *)malloc((size_t)(props.size > 0 ? props.size : 1) * sizeof(int));
    if (irwls_sgma_dev(&X, &dataset, props, cent)) {
        free(cent);
        cent = NULL;
    }
    irwls_dev_release(&X);
    return cent;
}

double *IRWLSpar(svm_dataset dataset, int *indexes, properties props) {
    irwls_clear_error();
    irwls_dev_set X;
    const int rows = budget_rows(&dataset, indexes, props.size);
    if (irwls_check_labels(&dataset, dataset.l) || irwls_dev_upload(&dataset, rows, props.kernelType, props.Kgamma, 0, 0, &X)) return NULL;
    double *w = (double *)malloc((size_t)(props.size > 0 ? props.size : 1) * sizeof(double));
    if (irwls_par_dev(&X, dataset.l, indexes, props, w)) {
        free(w);
        w = NULL;
    }
    irwls_dev_release(&X);
    return w;
}

/* Centroids (which may include the class-mean rows) and their weights become
 * the model; bias 0 (src/budgeted-train.c:519-570). */
model calculateBudgetedModel(properties props, svm_dataset dataset, int *centroids, double *beta) {
    model m;
    m.Kgamma = props.Kgamma;
    m.sparse = dataset.sparse;
    m.maxdim = dataset.maxdim;
    m.nSVs = props.size;
    m.bias = 0.0;
    m.kernelType = props.kernelType;
    int nElem = 0;
    for (int i = 0; i < props.size; i++) {
        const svm_sample *p = dataset.x[centroids[i]];
        while (p->index != -1) {
            ++p;
            ++nElem;
        }
        ++nElem;
    }
    m.nElem = nElem;
    m.weights = (double *)calloc(props.size, sizeof(double));
    memcpy(m.weights, beta, props.size * sizeof(double));
    m.quadratic_value = (double *)calloc(props.size, sizeof(double));
    m.x = (svm_sample **)calloc(props.size, sizeof(svm_sample *));
    m.features = (svm_sample *)calloc(nElem, sizeof(svm_sample));
    int f = 0;
    for (int i = 0; i < props.size; i++) {
        m.quadratic_value[i] = dataset.quadratic_value[centroids[i]];
        m.x[i] = &m.features[f];
        const svm_sample *p = dataset.x[centroids[i]];
        while (p->index != -1) {
            m.features[f].index = p->index;
            m.features[f].value = p->value;
            ++p;
            ++f;
        }
        m.features[f].index = -1;
        ++f;
    }
    return m;
}
