/*
 * IOStructures.h -- data model and libsvm/CSV/model-file I/O of the drop-in
 * LIBIRWLS library (libirwls_gb300.so).
 *
 * The four structs below are ABI-identical to the reference's
 * (include/IOStructures.h:44-122 of RobeDM/LIBIRWLS): same field order, same
 * types, so code compiled against the reference headers links unchanged.
 * Everything here is host C; datasets stay in host memory owned by the caller.
 */
#ifndef IRWLS_GB300_IOSTRUCTURES_H
#define IRWLS_GB300_IOSTRUCTURES_H

#include <stdio.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Training options (reference include/IOStructures.h:44-56). */
typedef struct properties {
    double Kgamma;    /* RBF gamma */
    int kernelType;   /* 0 linear, 1 RBF */
    double C;         /* SVM cost */
    int Threads;      /* host thread count (device work ignores it) */
    int MaxSize;      /* working-set size of full IRWLS */
    int size;         /* budget (number of centroids) of budgeted IRWLS */
    int algorithm;    /* centroid selection: 0 random, 1 SGMA */
    double Eta;       /* stop threshold of full IRWLS */
    int file;         /* 1 libsvm, 0 CSV */
    char *separator;  /* CSV separator */
    int verbose;      /* 1 prints progress on stdout */
} properties;

/* Prediction options (reference include/IOStructures.h:65-72). */
typedef struct predictProperties {
    int Labels;       /* 1 if the test file carries labels (accuracy is printed) */
    int Threads;
    int Soft;         /* 1 returns decision values, 0 returns +-1 */
    int file;
    char *separator;
    int verbose;
} predictProperties;

/* Trained classifier (reference include/IOStructures.h:81-93). */
typedef struct model {
    double Kgamma;
    int kernelType;
    int sparse;
    int nSVs;
    int nElem;                    /* svm_sample entries in features[] incl. -1 terminators */
    double *weights;              /* one weight per support vector / centroid */
    struct svm_sample **x;        /* row pointers into features[] */
    double *quadratic_value;      /* squared L2 norm of every support vector */
    int maxdim;
    double bias;
    struct svm_sample *features;
} model;

/* One (index, value) feature; rows end with index == -1
 * (reference include/IOStructures.h:102-105). */
typedef struct svm_sample {
    int index;
    double value;
} svm_sample;

/* A dataset: l rows; labeled readers append two class-mean rows at l and l+1
 * (reference include/IOStructures.h:114-122). */
typedef struct svm_dataset {
    int l;
    int sparse;                   /* 0: every row shares row 0's index pattern */
    int maxdim;
    double *y;
    struct svm_sample **x;
    double *quadratic_value;
    struct svm_sample *features;
} svm_dataset;

/* reference include/IOStructures.h:131 */
void freeDataset(svm_dataset data);
/* reference include/IOStructures.h:140 */
void freeModel(model modelo);
/* Labeled libsvm reader; appends the class-mean rows
 * (reference include/IOStructures.h:155, src/IOStructures.c:88-275). */
svm_dataset readTrainFile(char filename[]);
/* Labeled CSV reader (reference include/IOStructures.h:171, src/IOStructures.c:293-493). */
svm_dataset readTrainFileCSV(char filename[], char *separator);
/* Unlabeled libsvm reader (reference include/IOStructures.h:187, src/IOStructures.c:510-625). */
svm_dataset readUnlabeledFile(char filename[]);
/* Unlabeled CSV reader (reference include/IOStructures.h:205, src/IOStructures.c:642-762). */
svm_dataset readUnlabeledFileCSV(char filename[], char *separator);
/* Binary model writer (reference include/IOStructures.h:216, src/IOStructures.c:773-788). */
void storeModel(model *mod, FILE *Output);
/* Binary model reader (reference include/IOStructures.h:226, src/IOStructures.c:798-825). */
void readModel(model *mod, FILE *Input);
/* One "%lf" line per prediction (reference include/IOStructures.h:238, src/IOStructures.c:836-848). */
void writeOutput(char fileoutput[], double *predictions, int size);

#ifdef __cplusplus
}
#endif

#endif
