/*
 * full-train.h -- full (non-budgeted) SVM training by IRWLS on working sets.
 * The training itself runs on the GPU; see irwls_gpu.h for the error channel.
 */
#ifndef IRWLS_GB300_FULL_TRAIN_H
#define IRWLS_GB300_FULL_TRAIN_H

#include "IOStructures.h"

#ifdef __cplusplus
extern "C" {
#endif

/* malloc'd random permutation of 0..n-1 drawn with libc rand()
 * (reference include/full-train.h:51, src/full-train.c:65-77). */
int *rpermute(int n);

/* One inner IRWLS solve on a working set given as its own dataset of
 * dataset.l rows. GIN has l+1 entries, e has l, beta has l+1 (last = bias).
 * e and beta are updated in place; returns a malloc'd copy of the best
 * iterate (l+1 doubles), or NULL on a device error.
 * Replaces reference include/full-train.h:69 (src/full-train.c:96-362). */
double *subIRWLS(svm_dataset dataset, properties props, double *GIN, double *e, double *beta);

/* Full IRWLS training. Returns malloc'd weights beta[0..l-1] (beta_i =
 * alpha_i y_i) followed by the bias beta[l]; NULL on a device error.
 * Replaces reference include/full-train.h:85 (src/full-train.c:373-668). */
double *trainFULL(svm_dataset dataset, properties props);

/* Command-line help of full-train (reference include/full-train.h:94). */
void printFULLInstructions(void);

/* Parses "-g -c -e -t -k -w -s -f -p -v" options and shifts argv
 * (reference include/full-train.h:106, src/full-train.c:708-766). */
properties parseTrainFULLParameters(int *argc, char ***argv);

/* Packs the rows with beta != 0 into a model
 * (reference include/full-train.h:119, src/full-train.c:779-839). */
model calculateFULLModel(properties props, svm_dataset dataset, double *beta);

#ifdef __cplusplus
}
#endif

#endif
