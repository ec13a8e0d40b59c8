/*
 * full_train.c -- host orchestration of full IRWLS on the GPU
 * (reference src/full-train.c). The loops, their exit tests, the rand()
 * calls of the working-set permutation and the verbose output stay on the
 * host; every O(l) or larger step runs on the device through irwls_dev.h.
 * Device state lives for one training call; the host reads back a few
 * scalars per inner iteration (the loop tests) and the set sizes per outer
 * iteration.
 */
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "full-train.h"
#include "irwls_dev.h"
#include "irwls_gpu.h"

int *rpermute(int n) {
    int *p = (int *)malloc((n > 0 ? n : 1) * sizeof(int));
    for (int k = 0; k < n; k++) p[k] = k;
    for (int k = n - 1; k > 0; k--) {
        const int j = irwls_rand() % (k + 1);
        const int t = p[j];
        p[j] = p[k];
        p[k] = t;
    }
    return p;
}

/* Inner IRWLS loop on the working set held in ws (src/full-train.c:131-361);
 * the best iterate ends in ws->bbest. */
static int run_sub(irwls_sub_ws *ws, const irwls_dev_set *X, const properties *props) {
    const double C = props->C;
    if (irwls_sub_init(ws, X, C)) return -1;
    if (irwls_dev_d2h(ws->h_stats, ws->stats, sizeof(irwls_sub_stats)) || irwls_dev_sync()) return -1;
    int n1 = ws->h_stats->nS1, n3 = ws->h_stats->nS3;
    int iter = 0, since_best = 0;
    double dW = 1e9, nW = 1.0, best = 1e9, bmax = 0.0, bmin = 0.0;
    while ((iter < 5) || ((bmin < 0.0) || (bmax > C)) && (iter < 1000) && (since_best < 5) && (dW / nW > 1e-6)) {
        iter++;
        /* G13 of the lists left by the previous iteration (zero before the first) */
        if (iter > 1 && irwls_sub_g13(ws, X, n1, n3)) return -1;
        if (irwls_sub_iterate(ws, X, C, n1, n3)) return -1;
        if (irwls_dev_d2h(ws->h_stats, ws->stats, sizeof(irwls_sub_stats)) || irwls_dev_sync()) return -1;
        const irwls_sub_stats *st = ws->h_stats;
        dW = st->dW;
        nW = st->nW;
        bmax = st->bmax;
        bmin = st->bmin;
        if (dW / nW < best) {
            best = dW / nW;
            since_best = 0;
            if (irwls_dev_d2d(ws->bbest, ws->bnew, (size_t)(ws->w + 1) * sizeof(double))) return -1;
        } else {
            since_best += 1;
        }
        n1 = st->nS1;
        n3 = st->nS3;
    }
    return 0;
}

double *subIRWLS(svm_dataset dataset, properties props, double *GIN, double *e, double *beta) {
    irwls_clear_error();
    const int l = dataset.l;
    irwls_dev_set X;
    if (irwls_check_labels(&dataset, l) || irwls_dev_upload(&dataset, l, props.kernelType, props.Kgamma, 0, 0, &X)) return NULL;
    irwls_sub_ws ws;
    double *out = NULL;
    if (irwls_sub_alloc(&ws, l > 0 ? l : 1)) goto done_x;
    ws.w = l;
    {
        int *ident = (int *)malloc((l > 0 ? l : 1) * sizeof(int));
        for (int i = 0; i < l; i++) ident[i] = i;
        int rc = irwls_dev_h2d(ws.map, ident, l * sizeof(int));
        rc |= irwls_dev_h2d(ws.GIN, GIN, (l + 1) * sizeof(double));
        rc |= irwls_dev_h2d(ws.e, e, l * sizeof(double));
        rc |= irwls_dev_h2d(ws.beta, beta, (l + 1) * sizeof(double));
        rc |= irwls_dev_memset(ws.bbest, 0, (l + 1) * sizeof(double));
        rc |= irwls_dev_sync();
        free(ident);
        if (rc) goto done_ws;
    }
    if (run_sub(&ws, &X, &props)) goto done_ws;
    out = (double *)malloc((l + 1) * sizeof(double));
    if (irwls_dev_d2h(out, ws.bbest, (l + 1) * sizeof(double)) || irwls_dev_d2h(e, ws.e, l * sizeof(double)) ||
        irwls_dev_d2h(beta, ws.beta, (l + 1) * sizeof(double)) || irwls_dev_sync()) {
        free(out);
        out = NULL;
    }
done_ws:
    irwls_sub_release(&ws);
done_x:
    irwls_dev_release(&X);
    return out;
}

/* Outer working-set loop on a dataset resident on the GPU
 * (src/full-train.c:373-668); beta_out receives betaNew (l + 1 values). */
int irwls_full_train_dev(const irwls_dev_set *X, int l, properties props, double *beta_out) {
    const int W = props.MaxSize;
    const double C = props.C;
    if (W <= 0) {
        irwls_set_error(-8, "working-set size must be positive (got %d)", W);
        return -8;
    }
    int rc = 0;
    double *e = NULL, *beta = NULL, *bnew = NULL, *cb = NULL, *dbias = NULL, *norms = NULL;
    int *SW = NULL, *SIN = NULL, *SC = NULL, *lst = NULL, *cnt = NULL, *perm_d = NULL;
    irwls_outer_counts *counts = NULL, *h_counts = NULL;
    double *h_norms = NULL;
    irwls_sub_ws ws;
    memset(&ws, 0, sizeof ws);
    const size_t L1 = (size_t)(l + 1);
    /* precision form: the error update of most rows runs on the tensor cores
       from a split copy of the dataset (irwls_tc_kernel_rowsum, about 1e-5
       relative per kernel value); the rows whose errors decide anything --
       support vectors, rows within `band` of the margin, the working set --
       keep FP64 increments (the exact set S), rows entering S are recomputed
       from the support vectors, and every row is recomputed once the
       accumulated error bound of the others reaches band / 5. The working-set
       solves, GIN and the in-set updates are the FP64 form's. */
    void *tcs = NULL;
    if (irwls_get_precision() == IRWLS_PRECISION_MIXED && !(tcs = irwls_tc_set_create(X, l, W))) return -1;
    const double band = 0.05, eps = 2e-5 * (tcs ? irwls_tc_set_kbound(tcs) : 1.0);
    int *xflag = NULL, *xmark = NULL, *xS = NULL, *xSnew = NULL, *svlst = NULL, *svcnt = NULL, *xcnt = NULL,
        *h_xcnt = NULL;
    double *eS = NULL, *svcb = NULL, *h_l1 = NULL;
    int nS = 0;
    double acc = 0.0;
    rc |= irwls_dev_malloc((void **)&e, L1 * sizeof(double));
    rc |= irwls_dev_malloc((void **)&beta, L1 * sizeof(double));
    rc |= irwls_dev_malloc((void **)&bnew, L1 * sizeof(double));
    rc |= irwls_dev_malloc((void **)&cb, L1 * sizeof(double));
    rc |= irwls_dev_malloc((void **)&dbias, 2 * sizeof(double));
    rc |= irwls_dev_malloc((void **)&norms, 2 * sizeof(double));
    rc |= irwls_dev_malloc((void **)&SW, (W + 1) * sizeof(int));
    rc |= irwls_dev_malloc((void **)&SIN, L1 * sizeof(int));
    rc |= irwls_dev_malloc((void **)&SC, L1 * sizeof(int));
    rc |= irwls_dev_malloc((void **)&lst, L1 * sizeof(int));
    rc |= irwls_dev_malloc((void **)&perm_d, L1 * sizeof(int));
    rc |= irwls_dev_malloc((void **)&cnt, 2 * sizeof(int));
    rc |= irwls_dev_malloc((void **)&counts, sizeof(irwls_outer_counts));
    rc |= irwls_dev_host_alloc((void **)&h_counts, sizeof(irwls_outer_counts));
    rc |= irwls_dev_host_alloc((void **)&h_norms, 2 * sizeof(double));
    rc |= irwls_sub_alloc(&ws, W);
    if (tcs) {
        rc |= irwls_dev_malloc((void **)&xflag, L1 * sizeof(int));
        rc |= irwls_dev_malloc((void **)&xmark, L1 * sizeof(int));
        rc |= irwls_dev_malloc((void **)&xS, L1 * sizeof(int));
        rc |= irwls_dev_malloc((void **)&xSnew, L1 * sizeof(int));
        rc |= irwls_dev_malloc((void **)&svlst, L1 * sizeof(int));
        rc |= irwls_dev_malloc((void **)&svcnt, 2 * sizeof(int));
        rc |= irwls_dev_malloc((void **)&xcnt, 2 * sizeof(int));
        rc |= irwls_dev_malloc((void **)&eS, L1 * sizeof(double));
        rc |= irwls_dev_malloc((void **)&svcb, L1 * sizeof(double));
        rc |= irwls_dev_host_alloc((void **)&h_xcnt, 2 * sizeof(int));
        rc |= irwls_dev_host_alloc((void **)&h_l1, sizeof(double));
        if (!rc) {
            rc |= irwls_dev_memset(xflag, 0, L1 * sizeof(int));
            rc |= irwls_dev_memset(xmark, 0, L1 * sizeof(int));
        }
    }
    if (rc) goto done;

    /* initial working set: every tenth sample, up to W (src/full-train.c:411-423) */
    int nSW = 0, nSIN = 0;
    {
        int *hsw = (int *)malloc((W + 1) * sizeof(int));
        int *hsin = (int *)malloc(L1 * sizeof(int));
        for (int i = 0; i < l; i++) {
            if (i % 10 < 1 && nSW < W) hsw[nSW++] = i;
            else hsin[nSIN++] = i;
        }
        rc |= irwls_dev_h2d(SW, hsw, nSW * sizeof(int));
        rc |= irwls_dev_h2d(SIN, hsin, nSIN * sizeof(int));
        rc |= irwls_dev_d2d(e, X->y, l * sizeof(double));
        rc |= irwls_dev_memset(beta, 0, L1 * sizeof(double));
        rc |= irwls_dev_memset(bnew, 0, L1 * sizeof(double));
        rc |= irwls_dev_memset(ws.GIN, 0, (W + 2) * sizeof(double));
        rc |= irwls_dev_sync();
        free(hsw);
        free(hsin);
        if (rc) goto done;
        if (tcs) {
            /* e = y is exact everywhere: S is the first working set */
            rc |= irwls_full_exact_set(e, X->y, bnew, l, SW, nSW, band, 1, xflag, xmark, xS, xSnew, xcnt);
            rc |= irwls_dev_d2h(h_xcnt, xcnt, 2 * sizeof(int));
            rc |= irwls_dev_sync();
            if (rc) goto done;
            nS = h_xcnt[0];
        }
    }

    int stop = 0, since_best = 0;
    double best = 1e20;
    while (stop == 0 && since_best < 300) {
        /* GIN of the inactive set; kept as is when the set is empty (:436-456) */
        if (nSIN > 0 && irwls_full_gin(X, SW, nSW, SIN, nSIN, bnew, lst, cb, cnt, ws.GIN)) goto fail;
        ws.w = nSW;
        ws.map = SW;
        ws.tcs = tcs;
        if (irwls_full_gather_ws(SW, nSW, e, beta, l, ws.e, ws.beta)) goto fail;
        if (irwls_dev_memset(ws.bbest, 0, (size_t)(nSW + 1) * sizeof(double))) goto fail;
        if (run_sub(&ws, X, &props)) goto fail;
        /* betaNew over the working set; e -= K(:, SW) (betaNew - beta) - dbias (:488-510) */
        if (irwls_full_apply_ws(SW, nSW, ws.bbest, beta, l, bnew, lst, cb, cnt, dbias)) goto fail;
        if (tcs) {
            /* FP64 increments of the exact rows, tensor-core update of all
               rows, then the exact values written back */
            if (nS > 0) {
                /* at most nSW changed weights: exact tensor-core dot products
                   where the data allow them, else the FP64 kernels */
                if (irwls_dev_gather(e, xS, nS, eS)) goto fail;
                const int ex = irwls_tc_exact_rowsum(tcs, X, xS, nS, lst, 0, cnt, nSW, cb, NULL, NULL, -1, eS, dbias, eS);
                if (ex < 0 ||
                    (ex == 1 && irwls_dev_kernel_rowsum_n(X, xS, nS, X, lst, cnt, cb, NULL, NULL, -1, eS, dbias, eS)))
                    goto fail;
            }
            if (irwls_tc_kernel_rowsum(tcs, lst, cnt, cb, e, dbias, e)) goto fail;
            if (irwls_dev_scatter(eS, xS, nS, e) || irwls_dev_d2h(h_l1, dbias + 1, sizeof(double))) goto fail;
        } else if (irwls_dev_kernel_rowsum_n(X, NULL, l, X, lst, cnt, cb, NULL, NULL, -1, e, dbias, e)) {
            goto fail;
        }
        if (irwls_full_norms(beta, bnew, l + 1, norms)) goto fail;
        if (irwls_dev_d2h(h_norms, norms, 2 * sizeof(double)) || irwls_dev_sync()) goto fail;
        if (tcs) {
            /* a tensor-core wait that ran out left these errors stale: stop now */
            const int tc = irwls_tc_status();
            if (tc) {
                irwls_set_error(-13, "a tensor-core pipeline wait of the error update ran out (code %d)", tc);
                goto fail;
            }
            acc += eps * h_l1[0];
        }
        const double ratio = h_norms[0] / h_norms[1];
        if (ratio < props.Eta) stop = 1;
        if (irwls_dev_d2d(beta, bnew, L1 * sizeof(double))) goto fail;
        if (ratio < best) {
            best = ratio;
            since_best = 0;
        } else {
            since_best += 1;
        }
        /* classification and the next working set (:540-643) */
        if (irwls_full_classify(bnew, e, X->y, l, C, SW, SC, SIN, counts)) goto fail;
        if (irwls_dev_d2h(h_counts, counts, sizeof(irwls_outer_counts)) || irwls_dev_sync()) goto fail;
        nSW = h_counts->nSW;
        nSIN = h_counts->nSIN;
        const int nSC = h_counts->nSC;
        if (props.verbose == 1) {
            printf("%s", ".");
            fflush(stdout);
        }
        if (nSC < (W - nSW)) {
            if (irwls_full_fill_ws(SW, nSW, SIN, nSIN, SC, nSC, NULL, nSC)) goto fail;
            nSW += nSC;
        } else {
            int *perm = rpermute(nSC);
            const int space = W - nSW;
            int r2 = irwls_dev_h2d(perm_d, perm, nSC * sizeof(int));
            r2 |= irwls_full_fill_ws(SW, nSW, SIN, nSIN, SC, nSC, perm_d, space);
            r2 |= irwls_dev_sync();  /* perm is pageable host memory: finish the copy before freeing it */
            free(perm);
            if (r2) goto fail;
            nSW += space;
            nSIN += nSC - space;
        }
        if (tcs && !stop) {
            /* the exact set of the next update; all rows recomputed when the
               error bound of the others nears the band */
            int all_exact = 0;
            if (acc > band / 5) {
                if (irwls_full_exact_errors(X, l, bnew, svlst, svcb, svcnt, e)) goto fail;
                acc = 0.0;
                all_exact = 1;
            }
            if (irwls_full_exact_set(e, X->y, bnew, l, SW, nSW, band, all_exact, xflag, xmark, xS, xSnew, xcnt) ||
                irwls_dev_d2h(h_xcnt, xcnt, 2 * sizeof(int)) || irwls_dev_sync())
                goto fail;
            nS = h_xcnt[0];
            const int nnew = h_xcnt[1];
            if (nnew > 0) {
                /* rows entering S: e = y - sum over the support vectors - b */
                if (irwls_full_sv_list(bnew, l, svlst, svcb, svcnt) || irwls_dev_gather(X->y, xSnew, nnew, eS) ||
                    irwls_dev_d2h(h_xcnt, svcnt, sizeof(int)) || irwls_dev_sync())
                    goto fail;
                const int nsv = h_xcnt[0];
                const int ex = irwls_tc_exact_rowsum(tcs, X, xSnew, nnew, svlst, nsv, NULL, nsv, svcb, NULL, NULL, -1,
                                                     eS, bnew + l, eS);
                if (ex < 0 || (ex == 1 && irwls_dev_kernel_rowsum_n(X, xSnew, nnew, X, svlst, svcnt, svcb, NULL, NULL,
                                                                    -1, eS, bnew + l, eS)))
                    goto fail;
                if (irwls_dev_scatter(eS, xSnew, nnew, e)) goto fail;
            }
        }
    }
    if (irwls_dev_d2h(beta_out, bnew, L1 * sizeof(double)) || irwls_dev_sync()) goto fail;
    if (tcs) {
        const int tc = irwls_tc_status();
        if (tc) {
            irwls_set_error(-13, "a tensor-core pipeline wait of the error update ran out (code %d)", tc);
            goto fail;
        }
    }
    goto done;
fail:
    rc = -1;
done:
    irwls_sub_release(&ws);
    irwls_tc_set_free(tcs);
    void *xbufs[] = {xflag, xmark, xS, xSnew, svlst, svcnt, xcnt, eS, svcb};
    for (size_t k = 0; k < sizeof xbufs / sizeof xbufs[0]; k++) irwls_dev_free(xbufs[k]);
    irwls_dev_host_free(h_xcnt);
    irwls_dev_host_free(h_l1);
    void *bufs[] = {e, beta, bnew, cb, dbias, norms, SW, SIN, SC, lst, perm_d, cnt, counts};
    for (size_t k = 0; k < sizeof bufs / sizeof bufs[0]; k++) irwls_dev_free(bufs[k]);
    irwls_dev_host_free(h_counts);
    irwls_dev_host_free(h_norms);
    return rc ? -1 : 0;
}

double *trainFULL(svm_dataset dataset, properties props) {
    irwls_clear_error();
    if (props.verbose == 1) printf("\n");
    irwls_dev_set X;
    if (irwls_check_labels(&dataset, dataset.l) || irwls_dev_upload(&dataset, dataset.l, props.kernelType, props.Kgamma, 0, 0, &X)) return NULL;
    double *beta = (double *)malloc((size_t)(dataset.l + 1) * sizeof(double));
    if (irwls_full_train_dev(&X, dataset.l, props, beta)) {
        free(beta);
        beta = NULL;
    }
    irwls_dev_release(&X);
    if (props.verbose == 1) printf("\n");
    return beta;
}

/* Rows with beta != 0 become the model (src/full-train.c:779-839). */
model calculateFULLModel(properties props, svm_dataset dataset, double *beta) {
    model m;
    m.Kgamma = props.Kgamma;
    m.bias = beta[dataset.l];
    m.sparse = dataset.sparse;
    m.maxdim = dataset.maxdim;
    m.kernelType = props.kernelType;
    int nElem = 0, nSVs = 0;
    for (int i = 0; i < dataset.l; i++) {
        if (beta[i] != 0.0) {
            ++nSVs;
            const svm_sample *p = dataset.x[i];
            while (p->index != -1) {
                ++p;
                ++nElem;
            }
            ++nElem;
        }
    }
    m.nSVs = nSVs;
    m.nElem = nElem;
    m.weights = (double *)calloc(nSVs, sizeof(double));
    m.quadratic_value = (double *)calloc(nSVs, sizeof(double));
    m.x = (svm_sample **)calloc(nSVs, sizeof(svm_sample *));
    m.features = (svm_sample *)calloc(nElem, sizeof(svm_sample));
    int sv = 0, f = 0;
    for (int i = 0; i < dataset.l; i++) {
        if (beta[i] != 0.0) {
            m.quadratic_value[sv] = dataset.quadratic_value[i];
            m.weights[sv] = beta[i];
            m.x[sv] = &m.features[f];
            const svm_sample *p = dataset.x[i];
            while (p->index != -1) {
                m.features[f].index = p->index;
                m.features[f].value = p->value;
                ++p;
                ++f;
            }
            m.features[f].index = -1;  /* value stays 0 from calloc */
            ++f;
            ++sv;
        }
    }
    return m;
}
