/*
 * budgeted-train.h -- budgeted (semi-parametric) SVM: centroid selection by
 * SGMA or at random, then weighted least squares by IRWLS. Runs on the GPU.
 */
#ifndef IRWLS_GB300_BUDGETED_TRAIN_H
#define IRWLS_GB300_BUDGETED_TRAIN_H

#include "IOStructures.h"

#ifdef __cplusplus
extern "C" {
#endif

/* First props.size entries of a libc-rand() Fisher-Yates permutation of
 * 0..l-1; malloc'd (reference include/budgeted-train.h:47,
 * src/budgeted-train.c:73-100). */
int *randomCentroids(svm_dataset dataset, properties props);

/* Sparse Greedy Matrix Approximation: props.size centroid indices (the two
 * class-mean rows l and l+1 first), malloc'd; NULL on a device error
 * (reference include/budgeted-train.h:58, src/budgeted-train.c:114-309). */
int *SGMA(svm_dataset dataset, properties props);

/* IRWLS weights of the budgeted model over the given centroids; malloc'd
 * props.size doubles, NULL on a device error
 * (reference include/budgeted-train.h:70, src/budgeted-train.c:324-505). */
double *IRWLSpar(svm_dataset dataset, int *indexes, properties props);

/* Command-line help of budgeted-train (reference include/budgeted-train.h:80). */
void printBudgetedInstructions(void);

/* Parses "-g -c -e -k -t -w -s -a -f -p -v" and shifts argv
 * (reference include/budgeted-train.h:92, src/budgeted-train.c:581-642). */
properties parseTrainParameters(int *argc, char ***argv);

/* Packs the centroids and their weights into a model (bias 0)
 * (reference include/budgeted-train.h:106, src/budgeted-train.c:519-570). */
model calculateBudgetedModel(properties props, svm_dataset dataset, int *centroids, double *beta);

#ifdef __cplusplus
}
#endif

#endif
