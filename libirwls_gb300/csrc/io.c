/*
 * io.c -- dataset readers, model file and prediction output of the drop-in
 * library (host C; reference src/IOStructures.c). The in-memory layout, the
 * tokenisation (strtok on the same delimiters, in the same order), the error
 * exits and the binary model format are the reference's, so files read or
 * written here are interchangeable with the reference's.
 */
#include <ctype.h>
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "IOStructures.h"

#define LINE_MAX_CHARS 100000

static void fail(const char *msg) {
    fprintf(stderr, "%s", msg);
    exit(2);
}

static FILE *open_or_exit(const char *filename, const char *mode) {
    if (filename == NULL) fail("File not specified");
    FILE *f = fopen(filename, mode);
    if (f == NULL) {
        fprintf(stderr, "File not found: %s\n", filename);
        exit(2);
    }
    return f;
}

void freeDataset(svm_dataset data) {
    free(data.y);
    free(data.quadratic_value);
    free(data.x);
    free(data.features);
}

void freeModel(model modelo) {
    free(modelo.weights);
    free(modelo.quadratic_value);
    free(modelo.x);
    free(modelo.features);
}

/* Labeled libsvm file (src/IOStructures.c:88-275): two passes; the second
 * builds rows with -1 terminators, norms in file order, the sparse flag, and
 * appends the mean of the +1 rows (row l) and of the other rows (row l+1).
 * The norm of row l+1 divides by the positive count, as the reference does. */
svm_dataset readTrainFileGPU(char filename[]);

svm_dataset readTrainFile(char filename[]) {
    /* IRWLS_DEVICE_PARSER=1: the same dataset parsed on the GPU (dev_parse.cu) */
    const char *dev = getenv("IRWLS_DEVICE_PARSER");
    if (dev && dev[0] == '1') return readTrainFileGPU(filename);
    svm_dataset ds;
    char *line = (char *)malloc(LINE_MAX_CHARS);
    char *end, *tok, *idx, *val;
    FILE *f = open_or_exit(filename, "rb");

    ds.l = 0;
    ds.sparse = 0;
    int elements = 0, maxidx = 0;
    while (fgets(line, LINE_MAX_CHARS, f) != NULL) {
        strtok(line, " \t");
        for (;;) {
            idx = strtok(NULL, ":");
            tok = strtok(NULL, " \t");
            if (tok == NULL || *tok == '\n') break;
            int k = (int)strtol(idx, &end, 10);
            if (k > maxidx) maxidx = k;
            ++elements;
        }
        ++elements;
        ++ds.l;
    }
    elements += 2 * (maxidx + 2);
    double *sum_pos = (double *)calloc(maxidx + 1, sizeof(double));
    double *sum_neg = (double *)calloc(maxidx + 1, sizeof(double));
    double n_pos = 0.0, n_neg = 0.0;
    rewind(f);

    ds.y = (double *)calloc(ds.l + 2, sizeof(double));
    ds.quadratic_value = (double *)calloc(ds.l + 2, sizeof(double));
    ds.x = (svm_sample **)calloc(ds.l + 2, sizeof(svm_sample *));
    ds.features = (svm_sample *)calloc(elements, sizeof(svm_sample));
    ds.maxdim = 0;

    int max_index = 0, j = 0;
    for (int i = 0; i < ds.l; i++) {
        int row_max = -1;
        if (fgets(line, LINE_MAX_CHARS, f) == NULL) fail("Error reading data file\n");
        ds.x[i] = &ds.features[j];
        char *label = strtok(line, " \t\n");
        if (label == NULL) fail("Wrong file format\n");
        ds.y[i] = strtod(label, &end);
        if (ds.y[i] == 1.0) n_pos = n_pos + 1;
        else n_neg = n_neg + 1;
        if (end == label || *end != '\0') fail("Wrong file format\n");
        int dm = 0;
        for (;;) {
            idx = strtok(NULL, ":");
            val = strtok(NULL, " \t");
            if (val == NULL) break;
            ds.features[j].index = (int)strtol(idx, &end, 10);
            if (end == idx || *end != '\0' || ds.features[j].index <= row_max) fail("Wrong file format\n");
            row_max = ds.features[j].index;
            if (ds.features[dm].index != ds.features[j].index) ds.sparse = 1;
            ds.features[j].value = strtod(val, &end);
            if (ds.y[i] == 1.0) sum_pos[ds.features[j].index] += ds.features[j].value;
            else sum_neg[ds.features[j].index] += ds.features[j].value;
            const double v = strtod(val, &end);
            ds.quadratic_value[i] += v * v;
            if (end == val || (*end != '\0' && !isspace((unsigned char)*end))) fail("Wrong file format\n");
            ++dm;
            ++j;
        }
        if (row_max > max_index) max_index = row_max;
        ds.features[j++].index = -1;
    }

    ds.y[ds.l] = 1.0;
    ds.x[ds.l] = &ds.features[j];
    for (int k = 0; k <= maxidx; k++) {
        if (sum_pos[k] != 0.0) {
            ds.features[j].index = k;
            ds.features[j].value = sum_pos[k] / n_pos;
            const double v = sum_pos[k] / n_pos;
            ds.quadratic_value[ds.l] += v * v;
            ++j;
        }
    }
    ds.features[j++].index = -1;
    ds.y[ds.l + 1] = -1.0;
    ds.x[ds.l + 1] = &ds.features[j];
    for (int k = 0; k <= maxidx; k++) {
        if (sum_neg[k] != 0.0) {
            ds.features[j].index = k;
            ds.features[j].value = sum_neg[k] / n_neg;
            const double v = sum_neg[k] / n_pos;
            ds.quadratic_value[ds.l + 1] += v * v;
            ++j;
        }
    }
    ds.features[j++].index = -1;
    ds.maxdim = max_index;
    fclose(f);
    free(sum_pos);
    free(sum_neg);
    free(line);
    return ds;
}

/* The dataset of readTrainFile from rows parsed elsewhere (the device reader,
 * dev_parse.cu): rows[] holds the l rows in file order, each ended by a -1
 * entry (row i from row_start[i]); y and q are the labels and row norms. The
 * class-mean rows l and l + 1 are formed here exactly as readTrainFile forms
 * them (sums in row order, the negative mean's norm divided by the positive
 * count), over the pass-1 index range 0 ... maxidx.
 *
 * In two steps for a caller that copies the rows itself:
 * irwls_dataset_alloc allocates the arrays (features sized as readTrainFile
 * sizes them, zeroed), the caller writes the rows to features[0,
 * row_entries), and irwls_dataset_finish sets the row pointers, labels and
 * norms and appends the class-mean rows. Either step frees what it holds on
 * failure and returns -3; irwls_dataset_assemble is the two with a copy of
 * rows[] between them. */
int irwls_dataset_alloc(svm_dataset *ds, int l, long long pass1_elements, int maxidx, long long row_entries) {
    long long elements = pass1_elements > row_entries ? pass1_elements : row_entries;
    elements += 2 * ((long long)maxidx + 2);
    ds->l = l;
    ds->y = (double *)calloc((size_t)l + 2, sizeof(double));
    ds->quadratic_value = (double *)calloc((size_t)l + 2, sizeof(double));
    ds->x = (svm_sample **)calloc((size_t)l + 2, sizeof(svm_sample *));
    ds->features = (svm_sample *)calloc((size_t)elements, sizeof(svm_sample));
    if (!ds->y || !ds->quadratic_value || !ds->x || !ds->features) {
        freeDataset(*ds);
        memset(ds, 0, sizeof *ds);
        irwls_set_error(-3, "host allocation failed while assembling the dataset");
        return -3;
    }
    return 0;
}

int irwls_dataset_finish(svm_dataset *ds, int l, int maxidx, int max_index, int sparse, long long row_entries,
                         const long long *row_start, const double *y, const double *q) {
    const int top = maxidx > max_index ? maxidx : max_index;
    double *sum_pos = (double *)calloc((size_t)top + 1, sizeof(double));
    double *sum_neg = (double *)calloc((size_t)top + 1, sizeof(double));
    if (!sum_pos || !sum_neg) {
        free(sum_pos);
        free(sum_neg);
        freeDataset(*ds);
        memset(ds, 0, sizeof *ds);
        irwls_set_error(-3, "host allocation failed while assembling the dataset");
        return -3;
    }
    ds->sparse = sparse;
    double n_pos = 0.0, n_neg = 0.0;
    for (int i = 0; i < l; i++) {
        ds->x[i] = &ds->features[row_start[i]];
        ds->y[i] = y[i];
        ds->quadratic_value[i] = q[i];
        if (y[i] == 1.0) n_pos = n_pos + 1;
        else n_neg = n_neg + 1;
        for (const svm_sample *p = ds->x[i]; p->index != -1; ++p) {
            if (y[i] == 1.0) sum_pos[p->index] += p->value;
            else sum_neg[p->index] += p->value;
        }
    }
    long long j = row_entries;
    ds->y[l] = 1.0;
    ds->x[l] = &ds->features[j];
    for (int k = 0; k <= maxidx; k++) {
        if (sum_pos[k] != 0.0) {
            ds->features[j].index = k;
            ds->features[j].value = sum_pos[k] / n_pos;
            const double v = sum_pos[k] / n_pos;
            ds->quadratic_value[l] += v * v;
            ++j;
        }
    }
    ds->features[j++].index = -1;
    ds->y[l + 1] = -1.0;
    ds->x[l + 1] = &ds->features[j];
    for (int k = 0; k <= maxidx; k++) {
        if (sum_neg[k] != 0.0) {
            ds->features[j].index = k;
            ds->features[j].value = sum_neg[k] / n_neg;
            const double v = sum_neg[k] / n_pos;
            ds->quadratic_value[l + 1] += v * v;
            ++j;
        }
    }
    ds->features[j++].index = -1;
    ds->maxdim = max_index;
    free(sum_pos);
    free(sum_neg);
    return 0;
}

int irwls_dataset_assemble(svm_dataset *ds, int l, long long pass1_elements, int maxidx, int max_index, int sparse,
                           const svm_sample *rows, long long row_entries, const long long *row_start,
                           const double *y, const double *q) {
    int rc = irwls_dataset_alloc(ds, l, pass1_elements, maxidx, row_entries);
    if (rc) return rc;
    if (row_entries > 0) memcpy(ds->features, rows, (size_t)row_entries * sizeof(svm_sample));
    return irwls_dataset_finish(ds, l, maxidx, max_index, sparse, row_entries, row_start, y, q);
}

/* Labeled CSV file (src/IOStructures.c:293-493): label first, the k-th value
 * becomes feature k, zero values are not stored, class-mean rows appended as
 * for libsvm files. The format check of a stored value looks at the end
 * pointer of the previous number parsed on the line, as the reference does. */
svm_dataset readTrainFileCSV(char filename[], char *separator) {
    svm_dataset ds;
    char *line = (char *)malloc(LINE_MAX_CHARS);
    char *end = NULL, *prev_end = NULL, *tok;
    FILE *f = open_or_exit(filename, "rb");
    ds.l = 0;
    ds.sparse = 0;
    int elements = 0, maxidx = 0;
    while (fgets(line, LINE_MAX_CHARS, f) != NULL) {
        strtok(line, separator);
        int k = 0;
        for (;;) {
            k++;
            tok = strtok(NULL, separator);
            if (tok == NULL || *tok == '\n') break;
            if (k > maxidx) maxidx = k;
            if (strtod(tok, &end) != 0.0) ++elements;
        }
        ++elements;
        ++ds.l;
    }
    elements += 2 * (maxidx + 2);
    double *sum_pos = (double *)calloc(maxidx + 1, sizeof(double));
    double *sum_neg = (double *)calloc(maxidx + 1, sizeof(double));
    double n_pos = 0.0, n_neg = 0.0;
    rewind(f);
    ds.y = (double *)calloc(ds.l + 2, sizeof(double));
    ds.quadratic_value = (double *)calloc(ds.l + 2, sizeof(double));
    ds.x = (svm_sample **)calloc(ds.l + 2, sizeof(svm_sample *));
    ds.features = (svm_sample *)calloc(elements, sizeof(svm_sample));
    int max_index = 0, j = 0;
    for (int i = 0; i < ds.l; i++) {
        int row_max = -1;
        if (fgets(line, LINE_MAX_CHARS, f) == NULL) fail("Error reading data file\n");
        ds.x[i] = &ds.features[j];
        char *label = strtok(line, separator);
        if (label == NULL) fail("Wrong file format\n");
        ds.y[i] = strtod(label, &prev_end);
        if (ds.y[i] == 1.0) n_pos = n_pos + 1;
        else n_neg = n_neg + 1;
        if (prev_end == label || *prev_end != '\0') fail("Wrong file format\n");
        int k = 0, dm = 0;
        for (;;) {
            k++;
            tok = strtok(NULL, separator);
            if (tok == NULL) break;
            const double v = strtod(tok, &end);
            if (v != 0.0) {
                ds.features[j].index = k;
                if (*prev_end != '\0' || k <= row_max) fail("Wrong file format\n");
                row_max = k;
                if (ds.features[dm].index != k) ds.sparse = 1;
                ds.features[j].value = strtod(tok, &prev_end);
                if (ds.y[i] == 1.0) sum_pos[k] += ds.features[j].value;
                else sum_neg[k] += ds.features[j].value;
                const double w = strtod(tok, &prev_end);
                ds.quadratic_value[i] += w * w;
                if (prev_end == tok || (*prev_end != '\0' && !isspace((unsigned char)*prev_end)))
                    fail("Wrong file format\n");
                ++dm;
                ++j;
            }
        }
        if (row_max > max_index) max_index = row_max;
        ds.features[j++].index = -1;
    }
    ds.y[ds.l] = 1.0;
    ds.x[ds.l] = &ds.features[j];
    for (int k = 0; k <= maxidx; k++)
        if (sum_pos[k] != 0.0) {
            ds.features[j].index = k;
            ds.features[j].value = sum_pos[k] / n_pos;
            const double v = sum_pos[k] / n_pos;
            ds.quadratic_value[ds.l] += v * v;
            ++j;
        }
    ds.features[j++].index = -1;
    ds.y[ds.l + 1] = -1.0;
    ds.x[ds.l + 1] = &ds.features[j];
    for (int k = 0; k <= maxidx; k++)
        if (sum_neg[k] != 0.0) {
            ds.features[j].index = k;
            ds.features[j].value = sum_neg[k] / n_neg;
            const double v = sum_neg[k] / n_pos;
            ds.quadratic_value[ds.l + 1] += v * v;
            ++j;
        }
    ds.features[j++].index = -1;
    ds.maxdim = max_index;
    fclose(f);
    free(sum_pos);
    free(sum_neg);
    free(line);
    return ds;
}

/* Unlabeled libsvm file (src/IOStructures.c:510-625). */
svm_dataset readUnlabeledFile(char filename[]) {
    svm_dataset ds;
    char *line = (char *)malloc(LINE_MAX_CHARS);
    char *end, *idx, *val;
    FILE *f = open_or_exit(filename, "r");
    ds.l = 0;
    ds.sparse = 0;
    int elements = 0;
    while (fgets(line, LINE_MAX_CHARS, f) != NULL) {
        strtok(line, " \t");
        ++elements;
        for (;;) {
            char *p = strtok(NULL, " \t");
            if (p == NULL || *p == '\n') break;
            ++elements;
        }
        ++elements;
        ++ds.l;
    }
    rewind(f);
    ds.y = (double *)calloc(ds.l, sizeof(double));
    ds.quadratic_value = (double *)calloc(ds.l, sizeof(double));
    ds.x = (svm_sample **)calloc(ds.l, sizeof(svm_sample *));
    ds.features = (svm_sample *)calloc(elements, sizeof(svm_sample));
    int max_index = 0, j = 0;
    for (int i = 0; i < ds.l; i++) {
        int row_max = -1;
        if (fgets(line, LINE_MAX_CHARS, f) == NULL) fail("Error reading data file\n");
        ds.x[i] = &ds.features[j];
        ds.y[i] = 0;
        int dm = 0;
        idx = strtok(line, ":");
        val = strtok(NULL, " \t");
        while (val != NULL) {
            ds.features[j].index = (int)strtol(idx, &end, 10);
            if (end == idx || *end != '\0' || ds.features[j].index <= row_max) fail("Wrong file format\n");
            row_max = ds.features[j].index;
            if (ds.features[dm].index != ds.features[j].index) ds.sparse = 1;
            ds.features[j].value = strtod(val, &end);
            const double v = strtod(val, &end);
            ds.quadratic_value[i] += v * v;
            if (end == val || (*end != '\0' && !isspace((unsigned char)*end))) fail("Wrong file format\n");
            idx = strtok(NULL, ":");
            val = strtok(NULL, " \t");
            ++dm;
            ++j;
        }
        if (row_max > max_index) max_index = row_max;
        ds.features[j++].index = -1;
    }
    ds.maxdim = max_index;
    fclose(f);
    free(line);
    return ds;
}

/* Unlabeled CSV file (src/IOStructures.c:642-762). The reference starts every
 * row with strtok(NULL, ...), i.e. it continues the tokeniser state left by
 * the previous call instead of starting on the new line; this reader makes
 * the same calls, so it returns the same rows on the same C library. */
svm_dataset readUnlabeledFileCSV(char filename[], char *separator) {
    svm_dataset ds;
    char *line = (char *)malloc(LINE_MAX_CHARS);
    char *end, *tok;
    FILE *f = open_or_exit(filename, "r");
    ds.l = 0;
    ds.sparse = 0;
    int elements = 0;
    while (fgets(line, LINE_MAX_CHARS, f) != NULL) {
        tok = strtok(line, separator);
        if (strtod(tok, &end) != 0.0) ++elements;
        for (;;) {
            tok = strtok(NULL, separator);
            if (tok == NULL || *tok == '\n') break;
            if (strtod(tok, &end) != 0.0) ++elements;
        }
        ++elements;
        ++ds.l;
    }
    printf("Num Elements %d\n", elements);
    rewind(f);
    ds.y = (double *)calloc(ds.l, sizeof(double));
    ds.quadratic_value = (double *)calloc(ds.l, sizeof(double));
    ds.x = (svm_sample **)calloc(ds.l, sizeof(svm_sample *));
    ds.features = (svm_sample *)calloc(elements, sizeof(svm_sample));
    int max_index = 0, j = 0;
    for (int i = 0; i < ds.l; i++) {
        int row_max = -1;
        if (fgets(line, LINE_MAX_CHARS, f) == NULL) fail("Error reading data file\n");
        ds.x[i] = &ds.features[j];
        ds.y[i] = 0;
        tok = strtok(NULL, separator);
        int k = 0;
        for (;;) {
            ++k;
            if (tok == NULL) break;
            const double v = strtod(tok, &end);
            if (v != 0.0) {
                ds.features[j].index = k;
                if (*end != '\0' || k <= row_max) fail("Wrong file format\n");
                row_max = k;
                ds.features[j].value = v;
                ds.quadratic_value[i] += v * v;
                if (end == tok || (*end != '\0' && !isspace((unsigned char)*end))) fail("Wrong file format\n");
                ++j;
            }
            tok = strtok(NULL, separator);
        }
        if (row_max > max_index) max_index = row_max;
        ds.features[j++].index = -1;
    }
    ds.maxdim = max_index;
    fclose(f);
    free(line);
    return ds;
}

/* Binary model: gamma, bias (doubles), maxdim, kernelType, sparse, nSVs,
 * nElem (ints), weights[nSVs], norms[nSVs], features[nElem] as 16-byte
 * (index, value) records (src/IOStructures.c:773-788). */
void storeModel(model *mod, FILE *Output) {
    size_t n = 0;
    n += fwrite(&mod->Kgamma, sizeof(double), 1, Output);
    n += fwrite(&mod->bias, sizeof(double), 1, Output);
    n += fwrite(&mod->maxdim, sizeof(int), 1, Output);
    n += fwrite(&mod->kernelType, sizeof(int), 1, Output);
    n += fwrite(&mod->sparse, sizeof(int), 1, Output);
    n += fwrite(&mod->nSVs, sizeof(int), 1, Output);
    n += fwrite(&mod->nElem, sizeof(int), 1, Output);
    n += fwrite(mod->weights, sizeof(double), mod->nSVs, Output);
    n += fwrite(mod->quadratic_value, (mod->nSVs) * sizeof(double), 1, Output);
    n += fwrite(mod->x[0], (mod->nElem) * sizeof(svm_sample), 1, Output);
    (void)n;
    fflush(Output);
}

/* Reads the format above; row pointers start after every -1 terminator
 * (src/IOStructures.c:798-825). */
void readModel(model *mod, FILE *Input) {
    size_t n = 0;
    n += fread(&mod->Kgamma, sizeof(double), 1, Input);
    n += fread(&mod->bias, sizeof(double), 1, Input);
    n += fread(&mod->maxdim, sizeof(int), 1, Input);
    n += fread(&mod->kernelType, sizeof(int), 1, Input);
    n += fread(&mod->sparse, sizeof(int), 1, Input);
    n += fread(&mod->nSVs, sizeof(int), 1, Input);
    n += fread(&mod->nElem, sizeof(int), 1, Input);
    mod->weights = (double *)malloc((mod->nSVs) * sizeof(double));
    mod->quadratic_value = (double *)malloc((mod->nSVs) * sizeof(double));
    n += fread(mod->weights, sizeof(double), mod->nSVs, Input);
    n += fread(mod->quadratic_value, (mod->nSVs) * sizeof(double), 1, Input);
    mod->x = (svm_sample **)malloc((mod->nSVs) * sizeof(svm_sample *));
    mod->features = (svm_sample *)calloc((mod->nElem), sizeof(svm_sample));
    n += fread(mod->features, (mod->nElem) * sizeof(svm_sample), 1, Input);
    (void)n;
    mod->x[0] = &mod->features[0];
    int sv = 1;
    for (int k = 0; k < mod->nElem; k++) {
        if (mod->features[k].index == -1) {
            if (sv < mod->nSVs) mod->x[sv] = &mod->features[k + 1];
            ++sv;
        }
    }
}

void writeOutput(char fileoutput[], double *predictions, int size) {
    FILE *out = fopen(fileoutput, "w+");
    if (out != NULL) {
        for (int i = 0; i < size; i++) fprintf(out, "%lf\n", predictions[i]);
        fclose(out);
    }
}
