/*
 * gpu_api.c -- entry points that the reference does not have (irwls_gpu.h):
 * error channel, device-resident datasets, the Python module's dataset
 * builders (reference python-package/pythonmodule.c:213-355) and kernel
 * timing.
 */
#include <stdlib.h>
#include <string.h>

#include "budgeted-train.h"
#include "irwls_dev.h"
#include "irwls_gpu.h"

int irwls_last_error(void) { return irwls_get_error(); }
const char *irwls_last_error_message(void) { return irwls_get_error_message(); }
int irwls_gpu_available(void) { return irwls_dev_init() == 0; }

struct irwls_resident {
    irwls_dev_set X;
    svm_dataset ds;
    int kernelType;
};

irwls_resident *irwls_resident_upload(svm_dataset dataset, properties props, int with_mean_rows) {
    irwls_clear_error();
    irwls_resident *r = (irwls_resident *)calloc(1, sizeof *r);
    r->ds = dataset;
    r->kernelType = props.kernelType;
    const int rows = dataset.l + (with_mean_rows ? 2 : 0);
    if (irwls_check_labels(&dataset, dataset.l) || irwls_dev_upload(&dataset, rows, props.kernelType, props.Kgamma, 0, 0, &r->X)) {
        free(r);
        return NULL;
    }
    return r;
}

/* The device rows and the host dataset of a resident set (dev_model.cu). */
const irwls_dev_set *irwls_resident_devset(const irwls_resident *r) { return &r->X; }
const svm_dataset *irwls_resident_dataset(const irwls_resident *r) { return &r->ds; }

void irwls_resident_free(irwls_resident *r) {
    if (!r) return;
    irwls_dev_release(&r->X);
    free(r);
}

static int check_props(irwls_resident *r, properties *props) {
    if (props->kernelType != r->kernelType) {
        irwls_set_error(-10, "kernel type %d differs from the one the dataset was uploaded for (%d)",
                        props->kernelType, r->kernelType);
        return -10;
    }
    r->X.neg_gamma = -props->Kgamma;
    return 0;
}

int irwls_resident_budgeted(irwls_resident *r, properties props, int *centroids, double *weights) {
    irwls_clear_error();
    if (check_props(r, &props)) return -1;
    if (props.algorithm == 0) {
        int *c = randomCentroids(r->ds, props);
        memcpy(centroids, c, (size_t)props.size * sizeof(int));
        free(c);
    } else if (irwls_sgma_dev(&r->X, &r->ds, props, centroids)) {
        return -1;
    }
    return irwls_par_dev(&r->X, r->ds.l, centroids, props, weights) ? -1 : 0;
}

int irwls_resident_full(irwls_resident *r, properties props, double *beta) {
    irwls_clear_error();
    if (check_props(r, &props)) return -1;
    return irwls_full_train_dev(&r->X, r->ds.l, props, beta) ? -1 : 0;
}

/* numpy2dataset: every non-zero value becomes feature j+1; the set is flagged
 * sparse as soon as one value is non-zero (pythonmodule.c:213-263). */
svm_dataset irwls_dataset_from_dense(const double *X, const double *y, int n, int d) {
    svm_dataset ds;
    ds.l = n;
    ds.maxdim = d;
    ds.sparse = 0;
    ds.y = (double *)calloc(n > 0 ? n : 1, sizeof(double));
    ds.quadratic_value = (double *)calloc(n > 0 ? n : 1, sizeof(double));
    ds.x = (svm_sample **)calloc(n > 0 ? n : 1, sizeof(svm_sample *));
    long long elements = n;
    for (long long t = 0; t < (long long)n * d; t++)
        if (X[t] != 0.0) {
            elements++;
            ds.sparse = 1;
        }
    for (int i = 0; i < n; i++) ds.y[i] = y ? y[i] : 0.0;
    ds.features = (svm_sample *)calloc(elements > 0 ? elements : 1, sizeof(svm_sample));
    long long k = 0;
    for (int i = 0; i < n; i++) {
        ds.x[i] = &ds.features[k];
        for (int e = 0; e < d; e++) {
            const double v = X[(size_t)i * d + e];
            if (v != 0.0) {
                ds.quadratic_value[i] += v * v;
                ds.features[k].index = e + 1;
                ds.features[k].value = v;
                k++;
            }
        }
        ds.features[k++].index = -1;
    }
    return ds;
}

/* numpy2datasetWithAverage (pythonmodule.c:277-355). Rows l and l+1 are laid
 * out as the module lays them out: the positive mean row holds every feature
 * 1..d followed by a zero entry of index 0; the negative mean row starts with
 * the terminator, so it is empty; the two "norms" are plain sums of the mean
 * values. These quirks are kept so that results match the module's. */
svm_dataset irwls_dataset_from_dense_with_means(const double *X, const double *y, int n, int d) {
    svm_dataset ds;
    ds.l = n;
    ds.maxdim = d;
    ds.sparse = 0;
    ds.y = (double *)calloc(n + 2, sizeof(double));
    ds.quadratic_value = (double *)calloc(n + 2, sizeof(double));
    ds.x = (svm_sample **)calloc(n + 2, sizeof(svm_sample *));
    long long elements = n;
    int positives = 0, negatives = 0;
    for (int i = 0; i < n; i++) {
        for (int e = 0; e < d; e++)
            if (X[(size_t)i * d + e] != 0.0) {
                elements++;
                ds.sparse = 1;
            }
        ds.y[i] = y[i];
        if (y[i] == 1.0) positives++;
        else negatives++;
    }
    ds.features = (svm_sample *)calloc(elements + 2 * (d + 1), sizeof(svm_sample));
    svm_sample *mp = &ds.features[elements];
    svm_sample *mn = &ds.features[elements + d + 1];
    ds.y[n] = 1.0;
    ds.y[n + 1] = -1.0;
    ds.x[n] = mp;
    ds.x[n + 1] = mn;
    for (int e = 0; e < d; e++) {
        mp[e].index = e + 1;
        mp[e].value = 0.0;
        mn[e].index = e + 1;
        mn[e].value = 0.0;
    }
    ds.features[elements + d + 1].index = -1;
    ds.features[elements + 2 * d + 1].index = -1;
    long long k = 0;
    for (int i = 0; i < n; i++) {
        ds.x[i] = &ds.features[k];
        for (int e = 0; e < d; e++) {
            const double v = X[(size_t)i * d + e];
            if (v != 0.0) {
                ds.quadratic_value[i] += v * v;
                ds.features[k].index = e + 1;
                ds.features[k].value = v;
                if (ds.y[i] == 1.0) mp[e].value += (v / positives);
                else mn[e].value += (v / negatives);
                k++;
            }
        }
        ds.features[k++].index = -1;
    }
    for (int e = 0; e < d; e++) {
        ds.quadratic_value[n] += mp[e].value;
        ds.quadratic_value[n + 1] += mn[e].value;
    }
    return ds;
}

void irwls_profile_enable(int on) { irwls_prof_enable(on); }
void irwls_profile_reset(void) { irwls_prof_reset(); }
void irwls_profile_read(int slot, double *ms, long long *launches) {
    irwls_prof_collect();
    if (slot < 0 || slot >= IRWLS_PROF_SLOTS) {
        *ms = 0.0;
        *launches = 0;
        return;
    }
    irwls_prof_read(slot, ms, launches);
}
long long irwls_kernel_launches(void) { return irwls_launch_count(); }
