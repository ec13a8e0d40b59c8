/*
 * irwls_gpu.h -- entry points of libirwls_gb300.so that the reference does not
 * have: the error channel (the reference's training API has none), device
 * residency for callers that train repeatedly on one dataset, dataset
 * builders for the Python module, and kernel timing for benchmarks.
 */
#ifndef IRWLS_GB300_GPU_H
#define IRWLS_GB300_GPU_H

#include "IOStructures.h"

#ifdef __cplusplus
extern "C" {
#endif

/* Status of the last call that can fail on the device: 0 = success, < 0 =
 * an error, > 0 = a warning. Training and prediction functions return NULL
 * after an error and set this; a warning leaves the result in place.
 * Errors: -1 no device, -2 CUDA error, -3 allocation failed, -4 invalid
 * dataset (negative feature index, non-finite value or label, too many
 * entries) or arguments, -5 width/file limits, -6 solve limits, -7 to -12
 * limits of particular paths (see the message), -13 a tensor-core pipeline
 * wait ran out, -14 a CUDA error was already pending (allocation-free solve),
 * -20 to -22 the device libsvm reader. Warnings: IRWLS_WARN_PIVOT. */
int irwls_last_error(void);
const char *irwls_last_error_message(void);
/* ParallelLinearSystem / ParallelChol met a pivot that is not positive. The
 * reference (LAPACK dpotrf) reports it in an info value it ignores; this
 * library factors on as the reference's solve does and reports it here. */
enum { IRWLS_WARN_PIVOT = 1 };
/* Test hook, no counterpart in the reference: arms an injected failure of the
 * n-th device or pinned-host allocation the library makes from now on (n <= 0
 * disarms). The call that meets it fails with -3, as when the runtime refuses
 * memory, and the library stays usable. */
void irwls_debug_fail_alloc(long long n);
/* Test hook, no counterpart in the reference: the poll limit of every bounded
 * wait of the precision form's full-IRWLS error-update kernel (<= 0: the
 * default, 2^26 polls) and a stall switch with which that kernel's MMA thread
 * issues no MMA and never completes an accumulator, so that the epilogue's
 * wait runs out with no copy or MMA in flight. The training then fails with
 * -13 and the next one runs normally. */
void irwls_debug_tc_wait(long long limit, int stall);
/* Operand pieces (1 or 3) the last precision-form full-IRWLS training used:
 * 1 when every value of the set is exactly a bf16 after a scale of 1 or 255
 * (binary and 8-bit data; the products are then exact), else 3 (hi + mid +
 * lo of the FP32 value). */
int irwls_last_tc_pieces(void);
/* Kernel row sums of precision-form full IRWLS done in the exact-integer
 * mode since the last reset: on data whose values are integers after the
 * operand scale (8-bit values / 255, binary) with squared row norms below
 * 2^24 in those units, the exact rows' updates, the working-set updates and
 * G13 take their dot products exactly from the tensor cores (bf16 integer
 * products, FP32 sums below 2^24) and the exp and sums in FP64. */
long long irwls_tc_exact_calls(int reset);
/* Working-set solves of precision-form full IRWLS since the last reset:
 * those done by the FP32-factor + FP64-refinement cluster solve, and those
 * whose order fitted it but which went to the FP64 factorization (an FP32
 * pivot that was not positive, or a refinement that did not converge). */
void irwls_ws_mixed_counts(long long *solves, long long *fallbacks, int reset);
/* The precision form's solve of a full-IRWLS working-set system, device
 * pointers: the bordered matrix [H y; y^T 0] of src/full-train.c:165-186
 * with H's lower triangle in d_H (n1 x n1, column-major, leading dimension
 * ld >= n1 + 1) and y in row n1 of the same array, right-hand side d_rhs
 * (n1 + 1 values); d_x (n1 + 1 values) receives the solution that the
 * reference's dpotrf/dpotrs call (src/ParallelAlgorithms.c:361-388) gives,
 * whose last pivot fails by construction: with u = H^-1 y, v = H^-1 r and
 * s = y^T u, x_n = (r_n - y^T v) / s^2 and x = v - u x_n. H is factored in
 * FP32 inside one 16-CTA thread-block cluster and the two solves are refined
 * with FP64 residuals until they reach FP64 accuracy. Runs on the library's
 * stream and synchronizes it; d_H is not modified. Returns 0 when solved, 1
 * when the system must be solved in FP64 instead (n1 < 1, n1 above
 * irwls_ws_mixed_max(), an FP32 pivot that was not positive, or a
 * refinement that did not converge; d_x is then not a solution), or a
 * negative error code. irwls_ws_mixed_max() is 512, or 0 when the device
 * cannot run a 16-CTA cluster. */
int irwls_ws_solve_mixed(const double *d_H, int n1, int ld, const double *d_rhs, double *d_x);
int irwls_ws_mixed_max(void);
/* 1 when a CUDA device is usable. The library has no CPU path: without a
 * device every training or prediction call fails with an error. */
int irwls_gpu_available(void);

/* Arithmetic of the training paths:
 * IRWLS_PRECISION_FP64 (default): FP64 throughout, reference parity;
 * IRWLS_PRECISION_MIXED: the precision form -- SGMA candidate scores from
 * tensor-core products of three bf16 pieces per value (FP32 accuracy) on
 * the Nystrom features of the current centroids, with the K_mm
 * factorization and its solves in FP64 (it can pick a different centroid
 * where two candidates score within about 1e-7 of each other); the IRWLSpar Gram from exact
 * integer digit products on the tensor cores (about 2^-45 of the column
 * scales per row), its Cholesky, solves, residual and stop test in FP64;
 * in full IRWLS, the error updates of rows away from the margin on the
 * tensor cores. The environment variable IRWLS_PRECISION=mixed selects it
 * at start-up. */
enum { IRWLS_PRECISION_FP64 = 0, IRWLS_PRECISION_MIXED = 1 };
void irwls_set_precision(int mode);
int irwls_get_precision(void);

/* The libsvm reader on the GPU: the same svm_dataset as readTrainFile
 * (reference src/IOStructures.c:88-275) -- rows, labels, norms, the sparse
 * flag, maxdim and the class-mean rows -- with the text tokenised and every
 * number converted on the device (exactly as the C library's strtod/strtol).
 * irwls_parse_libsvm parses len bytes of file content and returns 0, -20 (the
 * reference's "Wrong file format"), -21 (a hexadecimal number, a NaN payload
 * or a decimal of more than 19 digits too close to a rounding boundary:
 * converted by the host reader, not by this one) or -22 (a line longer than
 * the reference's 99999-byte line buffer), the line in the message.
 * readTrainFileGPU reads a file, and exits with the reference's message and
 * status 2 on an error, as readTrainFile does. IRWLS_DEVICE_PARSER=1 makes
 * readTrainFile itself use the device reader. */
int irwls_parse_libsvm(const char *buf, size_t len, svm_dataset *ds);
svm_dataset readTrainFileGPU(char filename[]);
/* Numbers one per line through the device's strtod (out[i]; status[i]: 0
 * whole line, 1 trailing text, -1 no number, 2 not converted). Returns the
 * line count or a negative error. */
long long irwls_parse_doubles(const char *buf, size_t len, double *out, int *status, long long cap);

/* Linear-kernel prediction fast path (off by default): test()/softTest() of
 * a model with kernelType 0 evaluate b + x . W with W = sum_j w_j sv_j formed
 * once on the device, instead of the reference's per-support-vector kernel
 * sum (src/LIBIRWLS-predict.c:56-131); decision values then differ from the
 * reference's in the last bits (summation order). The environment variable
 * IRWLS_LINEAR_FAST=1 turns it on at start-up. */
void irwls_set_linear_fast_path(int on);
int irwls_get_linear_fast_path(void);

/* A training set uploaded to the GPU once (rows l + 2 when the class-mean
 * rows exist), for repeated training without host-to-device traffic. */
typedef struct irwls_resident irwls_resident;
irwls_resident *irwls_resident_upload(svm_dataset dataset, properties props, int with_mean_rows);
void irwls_resident_free(irwls_resident *r);
/* Budgeted training (SGMA or random centroids, then IRWLS) on a resident set;
 * fills centroids[props.size] and weights[props.size]. 0 on success. */
int irwls_resident_budgeted(irwls_resident *r, properties props, int *centroids, double *weights);
/* Full IRWLS on a resident set; fills beta[l + 1]. 0 on success. */
int irwls_resident_full(irwls_resident *r, properties props, double *beta);

/* Models on the GPU (reference calculateFULLModel / calculateBudgetedModel,
 * src/full-train.c:779-839, src/budgeted-train.c:519-570; storeModel /
 * readModel, src/IOStructures.c:773-825): the support vectors are packed,
 * read, stored and used for prediction on the device, without host
 * svm_sample arrays. irwls_dmodel_full packs the rows with beta != 0 of a
 * resident dataset (beta: l + 1 weights, the last one the bias),
 * irwls_dmodel_budgeted the given centroids (the resident set needs its
 * class-mean rows when a centroid is one of them); irwls_dmodel_store writes
 * the bytes storeModel writes for the same model; irwls_dmodel_read reads
 * that format; irwls_dmodel_predict is test (soft = 0) or softTest (soft = 1)
 * with the device model, printing the accuracy line when props.Labels == 1.
 * NULL / a nonzero return on an error (irwls_last_error_message). */
typedef struct irwls_dmodel irwls_dmodel;
irwls_dmodel *irwls_dmodel_full(const irwls_resident *r, properties props, const double *beta);
irwls_dmodel *irwls_dmodel_budgeted(const irwls_resident *r, properties props, const int *centroids,
                                    const double *weights);
irwls_dmodel *irwls_dmodel_read(const char *path);
int irwls_dmodel_store(const irwls_dmodel *m, const char *path);
double *irwls_dmodel_predict(const irwls_dmodel *m, svm_dataset ds, predictProperties props, int soft);
void irwls_dmodel_info(const irwls_dmodel *m, int *nSVs, int *nElem, double *bias);
void irwls_dmodel_free(irwls_dmodel *m);

/* Python-module dataset builders (reference python-package/pythonmodule.c):
 * dense row-major n x d doubles, every non-zero stored as feature j+1,
 * sparse = 1 when any value is non-zero (:213-263). The _with_means variant
 * appends the two class-mean rows as the module builds them (:277-355).
 * Free with freeDataset. */
svm_dataset irwls_dataset_from_dense(const double *X, const double *y, int n, int d);
svm_dataset irwls_dataset_from_dense_with_means(const double *X, const double *y, int n, int d);

/* Kernel timing with CUDA events on the library's stream. */
void irwls_profile_enable(int on);
void irwls_profile_reset(void);
/* slot: 0 SGMA score GEMM, 1 Gram update, 2 kernel row sums, 3 Cholesky
 * solve, 4 prediction, 5 SGMA candidate rows and solves, 6 SGMA selection
 * and factor/column update, 7 digit slicing of the precision form's Gram,
 * 8 the device libsvm reader's kernels.
 * Total milliseconds and launches since the reset. */
void irwls_profile_read(int slot, double *ms, long long *launches);
/* Kernel launches issued by the library since it was loaded. */
long long irwls_kernel_launches(void);
/* Iterations and final active-row count of the last IRWLSpar run. */
void irwls_last_run_info(int *par_iterations, int *active_rows);
/* Algorithmic flops of the last IRWLSpar run's Gram updates: the sum over
 * iterations of active_rows * (m + 1) * m (lower triangle and K2 row). */
double irwls_last_gram_flops(void);
/* bf16 tensor-core flops issued by the precision form's Gram kernel since
 * the last call with reset != 0 (28 digit-pair products per tile step). */
double irwls_gram_tc_flops(int reset);
/* Host-to-device and device-to-host bytes copied since the library was loaded. */
void irwls_transfer_bytes(long long *h2d, long long *d2h);
/* Overwrites a device buffer of `bytes` bytes (allocated on first use) so
 * that the next timed step starts with a cold L2. */
int irwls_l2_flush(size_t bytes);
/* CUDA-event timer on the library's stream: start, then stop returns ms. */
int irwls_timer_start(void);
double irwls_timer_stop(void);
/* FP64 FMA throughput of the device (TFLOP/s), measured by a DFMA-chain
 * kernel: the roofline denominator of the FP64 kernels. */
double irwls_fp64_peak_tflops(int reps);
/* Batching form: `count` independent trainings run concurrently, `workers`
 * at a time (<= 0: the autotuned count, 16 before any tuning), each on its
 * own CUDA stream with its own random generator. SVM i draws the sequence
 * srand(seeds[i]) would give (seeds NULL: 1 for every SVM), so its result
 * equals trainFULL(datasets[i], props[i]) -- or SGMA / randomCentroids then
 * IRWLSpar -- called after srand(seeds[i]). Outputs are malloc'd arrays
 * (betas[i]: l_i + 1 values; centroids[i] / weights[i]: props[i].size
 * values) that the caller frees; NULL for an SVM that failed. Returns 0 or
 * the first error. These have no counterpart in the reference. */
int irwls_full_train_batch(const svm_dataset *datasets, const properties *props, const unsigned *seeds, int count,
                           int workers, double **betas);
int irwls_budgeted_train_batch(const svm_dataset *datasets, const properties *props, const unsigned *seeds,
                               int count, int workers, int **centroids, double **weights);
/* Times full trainings of the `sample` largest SVMs of the batch at 4 to 48
 * concurrent workers, keeps the fastest count for later batches and returns
 * it (-1 on error). */
int irwls_batch_autotune(const svm_dataset *datasets, const properties *props, int count, int sample);
/* Fixes the worker count used when a batch is called with workers <= 0. */
void irwls_batch_set_workers(int workers);
/* n numbers of the library's equivalent of libc's srand(seed); rand(). */
void irwls_rand_sequence(unsigned seed, int n, int *out);
/* Learned-proposal form of SGMA (precision form, RBF kernels): a network of
 * 8 candidate features -> 128 -> 128 -> 1 (ReLU), parameters in the order W1
 * [128][8], b1, W2 [128][128], b2, W3 [1][128], b3 (FP32), trained on the GPU
 * by the library's own kernels. With a proposer set, every SGMA step scores
 * `pool` random candidates (half of each label) with it and sends its best 24
 * of each label, with 8 random ones of each label, to the exact score instead
 * of 64 random ones; NULL restores the reference's random candidates. None of
 * this has a counterpart in the reference. */
void *irwls_mlp_create(unsigned seed);
void irwls_mlp_free(void *mlp);
int irwls_mlp_param_count(void);
int irwls_mlp_feature_count(void);
int irwls_mlp_get_params(void *mlp, float *out);
int irwls_mlp_set_params(void *mlp, const float *in);
/* Mean squared error of the predictions of n rows X [n][8] against T and its
 * gradient (parameter layout); < 0 on error. */
double irwls_mlp_loss_grad(void *mlp, const float *X, const float *T, int n, float *grad);
int irwls_mlp_predict_host(void *mlp, const float *X, int n, float *out);
/* Adam on minibatches, `epochs` passes over a seeded shuffle; returns the mean
 * loss of the last pass. */
double irwls_mlp_train(void *mlp, const float *X, const float *T, int n, int epochs, int batch, float lr,
                       unsigned seed);
/* Features ((size - 2) x 64 x 8) and exact scores ((size - 2) x 64) of the
 * candidates of one precision-form SGMA run: random ones, or the installed
 * proposer's (on-policy traces). */
int irwls_sgma_traces(svm_dataset dataset, properties props, float *feat, float *score);
void irwls_set_sgma_proposer(void *mlp, int pool);
/* trace(K - K_nm K_mm^-1 K_mn) over the training rows after the last
 * precision-form SGMA run (RBF), or -1. */
double irwls_last_nystrom_residual(void);
/* FP32 FMA throughput of the device (TFLOP/s, one FMA = 2 flops), measured
 * the same way. */
double irwls_fp32_peak_tflops(int reps);

/* Cholesky factorization and solve of one system on the GPU that allocates
 * no memory; no counterpart in the reference. For callers that cannot let a
 * library allocate device memory mid-run: processes that gave the device's
 * memory to their own pool allocator at start-up, or latency-sensitive code
 * that must not run cudaMalloc/cudaFree (they can synchronize the device).
 *
 * d_M: column-major n x n matrix in device memory, leading dimension
 * ld >= n + 1 (row n holds the right-hand side); overwritten by its lower
 * Cholesky factor (a non-positive pivot is stored as LAPACK dpotrf leaves it).
 * Row n is scratch: its contents on return are unspecified.
 * d_b: right-hand side (n doubles, device) copied into row n, or NULL if row n
 * already holds it. d_x: solution (n doubles, device), or NULL to factor only.
 * d_info: NULL, or a device int that receives the first failed pivot
 * (1-based, 0 if none). stream: a cudaStream_t, or NULL for the default
 * stream; the call only enqueues work on it.
 *
 * Limit: n <= 4096; larger orders are rejected (-11, see
 * irwls_last_error_message). A CUDA error already pending in the calling
 * thread when the call starts is left in place and the call returns -14
 * without enqueueing anything. Scratch: one array of about 1.06 MiB in the library's
 * device memory, held by every GPU that loads the library until the process
 * exits. All calls share it and it keeps the last call's contents, so calls
 * that overlap on the GPU (on different streams) race; serialize them. The
 * first call on each device looks up the array's device address (with that
 * device current); make that first call before any stream capture.
 * Returns 0 on success. */
int irwls_chol_solve_noalloc(double *d_M, int n, int ld, const double *d_b, double *d_x, int *d_info,
                             void *stream);
/* CTAs of the cooperative backward sweep that a solve of order n uses on the
 * current device (0: the single-CTA sweep); no counterpart in the reference. */
int irwls_chol_sweep_ctas(int n);
/* Test hook, no counterpart in the reference: which Cholesky factorization
 * the solves use. 0 (default): one cooperative launch scheduled by data flow
 * where the device allows it, else the multi-launch panel sequence; 1: the
 * multi-launch sequence; 2: the data-flow launch only. Both give the same
 * bits. */
void irwls_debug_chol_path(int mode);

#ifdef __cplusplus
}
#endif

#endif
