/*
 * predict.c -- batched prediction on the GPU (reference
 * src/LIBIRWLS-predict.c:56-131). The test rows and the model's support
 * vectors are uploaded into one feature-index space; the decision values are
 * ordered kernel row sums (bias first, then support vectors in model order);
 * in the precision form they come from the tensor-core engine of dev_tc.cu.
 * The accuracy line is computed on the host from the returned values, as the
 * reference does.
 */
#include <stdio.h>
#include <stdlib.h>

#include "LIBIRWLS-predict.h"
#include "irwls_dev.h"
#include "irwls_gpu.h"

/* Linear-kernel fast path (off by default; IRWLS_LINEAR_FAST=1 or
   irwls_set_linear_fast_path(1)): a linear model predicts through its primal
   weights W = sum_j w_j sv_j, which changes the summation order and so the
   last bits of the decision values relative to the reference. */
static int g_linear_fast = -1;

void irwls_set_linear_fast_path(int on) { g_linear_fast = on ? 1 : 0; }

int irwls_get_linear_fast_path(void) {
    if (g_linear_fast < 0) {
        const char *e = getenv("IRWLS_LINEAR_FAST");
        g_linear_fast = (e && e[0] == '1') ? 1 : 0;
    }
    return g_linear_fast;
}

static double *predict(svm_dataset ds, model m, predictProperties props, int hard) {
    irwls_clear_error();
    const int n = ds.l;
    double *out = (double *)malloc((size_t)(n > 0 ? n : 1) * sizeof(double));
    if (n > 0) {
        int w = irwls_feature_width(&ds, n);
        const int wm = irwls_model_feature_width(&m);
        if (wm > w) w = wm;
        irwls_dev_set T, S;
        double *d_w = NULL, *d_out = NULL;
        const int fast = m.kernelType == 0 && irwls_get_linear_fast_path();
        int rc = fast ? irwls_dev_upload_csr(&ds, n, m.kernelType, m.Kgamma, w, &T)
                      : irwls_dev_upload(&ds, n, m.kernelType, m.Kgamma, 1, w, &T);
        if (rc) {
            free(out);
            return NULL;
        }
        rc = irwls_dev_upload_model(&m, w, &S);
        if (rc) {
            irwls_dev_release(&T);
            free(out);
            return NULL;
        }
        double *d_W = NULL;
        rc |= irwls_dev_malloc((void **)&d_w, (size_t)(m.nSVs > 0 ? m.nSVs : 1) * sizeof(double));
        rc |= irwls_dev_malloc((void **)&d_out, (size_t)n * sizeof(double));
        if (fast) rc |= irwls_dev_malloc((void **)&d_W, irwls_predict_linear_scratch(S.width, m.nSVs) * sizeof(double));
        if (!rc) {
            rc |= irwls_dev_h2d(d_w, m.weights, (size_t)m.nSVs * sizeof(double));
            if (fast)
                rc |= irwls_predict_linear(&T, n, &S, m.nSVs, d_w, m.bias, hard, d_W, d_out);
            else if (irwls_get_precision() == IRWLS_PRECISION_MIXED)
                rc |= irwls_tc_predict(&T, n, &S, m.nSVs, d_w, m.bias, hard, d_out);
            else
                rc |= irwls_predict_soft(&T, n, &S, m.nSVs, d_w, m.bias, hard, d_out);
            rc |= irwls_dev_d2h(out, d_out, (size_t)n * sizeof(double));
            rc |= irwls_dev_sync();
        }
        irwls_dev_free(d_w);
        irwls_dev_free(d_out);
        irwls_dev_free(d_W);
        irwls_dev_release(&T);
        irwls_dev_release(&S);
        if (rc) {
            free(out);
            return NULL;
        }
    }
    if (props.Labels == 1) {
        double hits = 0.0;
        for (int i = 0; i < n; i++) {
            if ((out[i] > 0) & (ds.y[i] > 0)) hits++;
            if ((out[i] <= 0) & (ds.y[i] <= 0)) hits++;
        }
        printf("Accuracy: %f\n", hits / (double)n);
    }
    return out;
}

double *softTest(svm_dataset dataset, model mymodel, predictProperties props) {
    return predict(dataset, mymodel, props, 0);
}

double *test(svm_dataset dataset, model mymodel, predictProperties props) {
    return predict(dataset, mymodel, props, 1);
}
