/*
 * kernels_scalar.c -- the reference's per-pair kernel API
 * (src/kernels.c:63-183) for external callers. One pair per call on the host;
 * the library's training and prediction never call these (they evaluate
 * kernel tiles on the GPU, dev_tiles.cu).
 */
#include <math.h>

#include "IOStructures.h"
#include "kernels.h"

static double merge_dot(const svm_sample *a, const svm_sample *b) {
    double s = 0.0;
    while (a->index != -1 && b->index != -1) {
        if (a->index == b->index) {
            s += a->value * b->value;
            ++a;
            ++b;
        } else if (a->index > b->index) {
            ++b;
        } else {
            ++a;
        }
    }
    return s;
}

static double merge_distance(double qa, double qb, const svm_sample *a, const svm_sample *b) {
    double s = qa + qb;
    while (a->index != -1 && b->index != -1) {
        if (a->index == b->index) {
            s += -2.0 * a->value * b->value;
            ++a;
            ++b;
        } else if (a->index < b->index) {
            ++a;
        } else {
            ++b;
        }
    }
    return s;
}

double kernelFunction(svm_dataset dataset, int index1, int index2, properties props) {
    const svm_sample *a = dataset.x[index1], *b = dataset.x[index2];
    if (props.kernelType == 0) return merge_dot(a, b);
    double s = 0.0;
    if (dataset.sparse == 0) {
        for (int t = 0; t < dataset.maxdim; t++) {
            const double d = a[t].value - b[t].value;
            s += d * d;
        }
    } else {
        s = merge_distance(dataset.quadratic_value[index1], dataset.quadratic_value[index2], a, b);
    }
    return exp(-(props.Kgamma) * s);
}

double kernelTest(svm_dataset dataset, int index1, model mymodel, int index2) {
    const svm_sample *a = dataset.x[index1], *b = mymodel.x[index2];
    if (mymodel.kernelType == 0) return merge_dot(a, b);
    return exp(-(mymodel.Kgamma) *
               merge_distance(dataset.quadratic_value[index1], mymodel.quadratic_value[index2], a, b));
}
