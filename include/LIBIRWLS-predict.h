/*
 * LIBIRWLS-predict.h -- batched prediction with a trained model on the GPU.
 */
#ifndef IRWLS_GB300_PREDICT_H
#define IRWLS_GB300_PREDICT_H

#include "IOStructures.h"

#ifdef __cplusplus
extern "C" {
#endif

/* Labels (+1 when the decision value is >= 0, else -1) of dataset.l rows,
 * malloc'd; prints "Accuracy: %f" when props.Labels == 1. NULL on a device
 * error. Replaces reference include/LIBIRWLS-predict.h:48
 * (src/LIBIRWLS-predict.c:99-131). */
double *test(svm_dataset dataset, model mymodel, predictProperties props);

/* Decision values bias + sum_j w_j k(x, sv_j), malloc'd. Replaces reference
 * include/LIBIRWLS-predict.h:61 (src/LIBIRWLS-predict.c:56-86). */
double *softTest(svm_dataset dataset, model mymodel, predictProperties props);

/* Command-line help of LIBIRWLS-predict (reference include/LIBIRWLS-predict.h:70). */
void printPredictInstructions(void);

/* Parses "-t -f -p -v -l -s" and shifts argv
 * (reference include/LIBIRWLS-predict.h:82, src/LIBIRWLS-predict.c:170-224). */
predictProperties parsePredictParameters(int *argc, char ***argv);

#ifdef __cplusplus
}
#endif

#endif
