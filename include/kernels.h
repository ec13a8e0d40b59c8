/*
 * kernels.h -- scalar kernel functions of the drop-in LIBIRWLS library.
 *
 * These two entry points keep the reference's per-pair API for external
 * callers. They are evaluated on the host, one pair per call; none of the
 * library's training or prediction routines calls them (those evaluate whole
 * kernel tiles on the GPU).
 */
#ifndef IRWLS_GB300_KERNELS_H
#define IRWLS_GB300_KERNELS_H

#include "IOStructures.h"

#ifdef __cplusplus
extern "C" {
#endif

/* k(x_index1, x_index2) inside one dataset: linear dot product, or
 * exp(-gamma*d2) with d2 = sum (x-y)^2 over maxdim raw values when
 * dataset.sparse == 0, else d2 = q1 + q2 - 2 x.y.
 * Replaces reference include/kernels.h:55 (src/kernels.c:63-118). */
double kernelFunction(svm_dataset dataset, int index1, int index2, properties props);

/* k(dataset row index1, support vector index2 of mymodel); RBF always uses
 * the norm form q1 + q2 - 2 x.y.
 * Replaces reference include/kernels.h:74 (src/kernels.c:137-183). */
double kernelTest(svm_dataset dataset, int index1, model mymodel, int index2);

#ifdef __cplusplus
}
#endif

#endif
