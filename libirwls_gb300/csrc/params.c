/*
 * params.c -- command-line option parsing and help of the three front-ends
 * (reference src/full-train.c:676-766, src/budgeted-train.c:581-673,
 * src/LIBIRWLS-predict.c:140-224). Same option letters, defaults, argv
 * shifting and exit codes as the reference.
 */
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "IOStructures.h"
#include "LIBIRWLS-predict.h"
#include "budgeted-train.h"
#include "full-train.h"

static void common_help(int budgeted) {
    fprintf(stderr, "Options:\n");
    fprintf(stderr, "  -k kernel type (default 1): 0 linear u'v, 1 RBF exp(-gamma |u-v|^2)\n");
    fprintf(stderr, "  -g gamma of the RBF kernel (default 1)\n");
    fprintf(stderr, "  -c cost C (default 1)\n");
    fprintf(stderr, "  -t host threads (default 1; the GPU path ignores it)\n");
    if (budgeted) {
        fprintf(stderr, "  -s budget: number of centroids (default 10)\n");
        fprintf(stderr, "  -a centroid selection (default 1): 0 random, 1 SGMA\n");
    } else {
        fprintf(stderr, "  -w working-set size (default 500)\n");
        fprintf(stderr, "  -e stop threshold (default 0.001)\n");
    }
    fprintf(stderr, "  -f file format (default 1): 0 CSV, 1 libsvm\n");
    fprintf(stderr, "  -p CSV separator (default \",\")\n");
    fprintf(stderr, "  -v verbose (default 1): 0 silent, 1 progress messages\n");
}

void printFULLInstructions(void) {
    fprintf(stderr, "full-train: trains a full SVM by IRWLS on the GPU and writes its model.\n\n");
    fprintf(stderr, "Usage: full-train [options] training_set_file model_file\n\n");
    common_help(0);
}

void printBudgetedInstructions(void) {
    fprintf(stderr, "budgeted-train: trains a budgeted SVM (SGMA + IRWLS) on the GPU and writes its model.\n\n");
    fprintf(stderr, "Usage: budgeted-train [options] training_set_file model_file\n\n");
    common_help(1);
}

void printPredictInstructions(void) {
    fprintf(stderr, "LIBIRWLS-predict: classifies a data set with a model from full-train or budgeted-train.\n\n");
    fprintf(stderr, "Usage: LIBIRWLS-predict [options] data_set_file model_file output_file\n\n");
    fprintf(stderr, "Options:\n");
    fprintf(stderr, "  -t host threads (default 1)\n");
    fprintf(stderr, "  -l 1 if the data set is labeled (prints the accuracy), 0 otherwise (default 0)\n");
    fprintf(stderr, "  -s 1 writes decision values, 0 writes +1/-1 (default 0)\n");
    fprintf(stderr, "  -f file format (default 1): 0 CSV, 1 libsvm\n");
    fprintf(stderr, "  -p CSV separator (default \",\")\n");
    fprintf(stderr, "  -v verbose (default 1)\n");
}

/* Moves the positional arguments that follow the options to argv[1..]. */
static void shift_args(int *argc, char ***argv, int first) {
    int j;
    for (j = 1; first + j - 1 < *argc; ++j) (*argv)[j] = (*argv)[first + j - 1];
    *argc -= first - 1;
}

static properties train_defaults(int algorithm) {
    properties p;
    p.Kgamma = 1.0;
    p.C = 1.0;
    p.Threads = 1;
    p.MaxSize = 500;
    p.Eta = 0.001;
    p.size = 10;
    p.algorithm = algorithm;
    p.kernelType = 1;
    p.file = 1;
    p.separator = ",";
    p.verbose = 1;
    return p;
}

static properties parse_train(int *argc, char ***argv, int budgeted) {
    properties p = train_defaults(1);
    int i;
    for (i = 1; i < *argc; ++i) {
        if ((*argv)[i][0] != '-') break;
        if (++i >= *argc) {
            if (budgeted) printBudgetedInstructions();
            else printFULLInstructions();
            exit(1);
        }
        const char *name = &(*argv)[i - 1][1];
        char *value = (*argv)[i];
        if (strcmp(name, "g") == 0) p.Kgamma = atof(value);
        else if (strcmp(name, "c") == 0) p.C = atof(value);
        else if (strcmp(name, "e") == 0) p.Eta = atof(value);
        else if (strcmp(name, "t") == 0) p.Threads = atoi(value);
        else if (strcmp(name, "k") == 0) p.kernelType = atoi(value);
        else if (strcmp(name, "w") == 0) p.MaxSize = atoi(value);
        else if (strcmp(name, "s") == 0) p.size = atoi(value);
        else if (budgeted && strcmp(name, "a") == 0) p.algorithm = atoi(value);
        else if (strcmp(name, "f") == 0) p.file = atoi(value);
        else if (strcmp(name, "p") == 0) p.separator = value;
        else if (strcmp(name, "v") == 0) p.verbose = atoi(value);
        else {
            fprintf(stderr, "Unknown parameter %s\n", name);
            if (budgeted) printBudgetedInstructions();
            else printFULLInstructions();
            exit(2);
        }
    }
    shift_args(argc, argv, i);
    return p;
}

properties parseTrainFULLParameters(int *argc, char ***argv) { return parse_train(argc, argv, 0); }
properties parseTrainParameters(int *argc, char ***argv) { return parse_train(argc, argv, 1); }

predictProperties parsePredictParameters(int *argc, char ***argv) {
    predictProperties p;
    p.Labels = 0;
    p.Threads = 1;
    p.Soft = 0;
    p.file = 1;
    p.separator = ",";
    p.verbose = 1;
    int i;
    for (i = 1; i < *argc; ++i) {
        if ((*argv)[i][0] != '-') break;
        if (++i >= *argc) {
            printPredictInstructions();
            exit(1);
        }
        const char *name = &(*argv)[i - 1][1];
        char *value = (*argv)[i];
        if (strcmp(name, "t") == 0) p.Threads = (int)atof(value);
        else if (strcmp(name, "f") == 0) p.file = atoi(value);
        else if (strcmp(name, "p") == 0) p.separator = value;
        else if (strcmp(name, "v") == 0) p.verbose = atoi(value);
        else if (strcmp(name, "l") == 0) {
            p.Labels = atoi(value);
            if (p.Labels != 0 && p.Labels != 1) {
                printf("\nInvalid type of test data set:%d\n", p.Labels);
                exit(2);
            }
        } else if (strcmp(name, "s") == 0) {
            p.Soft = atoi(value);
            if (p.Soft != 0 && p.Soft != 1) {
                printf("\nInvalid type of output (-s param):%d\n", p.Soft);
                exit(2);
            }
        } else {
            fprintf(stderr, "Unknown parameter %s\n", name);
            printPredictInstructions();
            exit(2);
        }
    }
    shift_args(argc, argv, i);
    return p;
}
