/*
 * irwls_dev.h -- the thin C-ABI between the host-C orchestration of the
 * IRWLS solvers and the CUDA kernels (sm_103a). Plain C types only; pointers
 * named d_* are device addresses. Every call is asynchronous on the library's
 * single CUDA stream unless it says otherwise, and returns 0 on success or a
 * negative status (the message is kept for irwls_last_error_message()).
 */
#ifndef IRWLS_DEV_H
#define IRWLS_DEV_H

#include <stddef.h>

#include "IOStructures.h"

#ifdef __cplusplus
extern "C" {
#endif

/* ---- errors (implemented in dev_context.cu) ---------------------------- */
void irwls_set_error(int code, const char *fmt, ...);
int irwls_get_error(void);
const char *irwls_get_error_message(void);
void irwls_clear_error(void);
/* A warning (positive code): recorded unless an error or a warning already is. */
void irwls_set_warning(int code, const char *fmt, ...);
/* First failed pivot (1-based) of the last Cholesky on the current context's
 * stream, 0 if none; synchronizes the stream. Returns 0 or an error. */
int irwls_dev_pivot_status(int *info);
/* -4 (and the error set) when one of the first n_rows labels is not finite. */
int irwls_check_labels(const svm_dataset *ds, int n_rows);

/* ---- context ------------------------------------------------------------ */
int irwls_dev_init(void);                     /* idempotent; creates the stream */
int irwls_dev_sync(void);                     /* waits for the stream, checks device flags */
/* Execution contexts (dev_context.cu): a worker thread binds a context of its
 * own (stream, status words, errors, scratch, random generator); NULL binds
 * the default context of the main thread. */
void *irwls_ctx_create(void);
void irwls_ctx_bind(void *h);
void irwls_ctx_destroy(void *h);
int irwls_ctx_error(void *h, char *msg, int cap);
void *irwls_ctx_scratch(int slot, size_t bytes);   /* grow-only, slots 0..3 */
/* The context's random numbers: libc srand/rand in the default context, a
 * generator that reproduces them exactly in worker contexts. */
void irwls_srand(unsigned seed);
int irwls_rand(void);
int irwls_dev_malloc(void **p, size_t bytes);
int irwls_dev_free(void *p);
int irwls_dev_h2d(void *d_dst, const void *h_src, size_t bytes);   /* async */
int irwls_dev_d2h(void *h_dst, const void *d_src, size_t bytes);   /* async */
int irwls_dev_d2d(void *d_dst, const void *d_src, size_t bytes);   /* async */
int irwls_dev_memset(void *d_dst, int byte, size_t bytes);         /* async */
int irwls_dev_workspace(size_t bytes, void **d_ws);   /* grow-only scratch */
void irwls_dev_release_workspace(void);
int irwls_dev_host_alloc(void **p, size_t bytes);      /* pinned host memory */
void irwls_dev_host_free(void *p);

/* ---- datasets resident on the GPU --------------------------------------- */
/* Kernel-evaluation modes (reference src/kernels.c:63-183). */
enum { IRWLS_K_RAW_RBF = 0,   /* sparse == 0: sum over maxdim raw values of (a-b)^2 */
       IRWLS_K_NORM_RBF = 1,  /* q_a + q_b - 2 a.b over shared feature indices */
       IRWLS_K_LINEAR = 2 };  /* a.b over shared feature indices */

typedef struct irwls_dev_set {
    int n_rows;       /* rows uploaded */
    int width;        /* dense row width: maxdim (raw mode) or max feature index + 1 */
    int ld;           /* leading dimension of X (>= width, even) */
    int mode;
    double neg_gamma; /* -gamma */
    double *X;        /* n_rows x ld dense rows (raw values or values by feature index) */
    int *rp;          /* CSR row pointers (n_rows + 1) of the by-index values */
    int *ci;          /* CSR column = feature index */
    double *cv;       /* CSR values */
    double *q;        /* quadratic_value per row */
    double *y;        /* labels per row */
    long long nnz;
} irwls_dev_set;

/* Uploads rows 0..n_rows-1 of `ds`. kernelType/gamma pick the mode as the
 * reference's kernelFunction does; force_norm selects the norm form for RBF
 * whatever ds.sparse says (kernelTest always uses it). width_hint widens the
 * by-index layout (so two sets share one column space). */
int irwls_dev_upload(const svm_dataset *ds, int n_rows, int kernelType, double gamma, int force_norm,
                     int width_hint, irwls_dev_set *out);
/* The same rows as CSR only (X holds no dense copy): for the linear
 * prediction path. */
int irwls_dev_upload_csr(const svm_dataset *ds, int n_rows, int kernelType, double gamma, int width_hint,
                         irwls_dev_set *out);
/* Same upload from the rows of a model. */
int irwls_dev_upload_model(const model *m, int width_hint, irwls_dev_set *out);
void irwls_dev_release(irwls_dev_set *s);
int irwls_feature_width(const svm_dataset *ds, int n_rows);   /* max index + 1 over rows */
int irwls_model_feature_width(const model *m);

/* ---- kernel tiles (dev_tiles.cu) ----------------------------------------- */
/* out[i*ld_out + j] = k(A[ia_i], B[ib_j]) for i < nA, j < nB. ia/ib may be
 * NULL (identity). A and B are the same dataset (training) or two datasets
 * with one column space (prediction). */
int irwls_dev_kernel_block(const irwls_dev_set *A, const int *d_ia, int nA, const irwls_dev_set *B,
                           const int *d_ib, int nB, double *d_out, int ld_out);

/* Ordered kernel row sums, the reference's accumulation order exactly:
 *   acc_i = init_i; for j in 0..nB-1: acc_i = acc_i OP term(i, j); out_i = acc_i
 * with term(i, j) = ((cb_j * k(A_i, B_j)) * sa_i) * sb_j  (sa/sb optional,
 * multiplication by +-1 labels is exact), OP = +1 add / -1 subtract, and
 * term = k * cb_j when `k_first` (the reference writes k*coef in its error
 * updates). tail (if non-NULL) is then subtracted: out_i = acc_i - tail[0]. */
int irwls_dev_kernel_rowsum(const irwls_dev_set *A, const int *d_ia, int nA, const irwls_dev_set *B,
                            const int *d_ib, int nB, const double *d_cb, const double *d_sa,
                            const double *d_sb, int k_first, int op, const double *d_init,
                            const double *d_tail, double *d_out);
/* Same with the B count read from device memory (*d_nB). */
int irwls_dev_kernel_rowsum_n(const irwls_dev_set *A, const int *d_ia, int nA, const irwls_dev_set *B,
                              const int *d_ib, const int *d_nB, const double *d_cb, const double *d_sa,
                              const double *d_sb, int op, const double *d_init, const double *d_tail,
                              double *d_out);
/* Block with optional transposed store: out[j*ld_out + i] when trans. */
int irwls_dev_kernel_block_t(const irwls_dev_set *A, const int *d_ia, int nA, const irwls_dev_set *B,
                             const int *d_ib, int nB, double *d_out, long long ld_out, int trans);

/* ---- linear algebra (dev_chol.cu) --------------------------------------- */
/* In-place lower Cholesky of the n x n matrix M (column-major, leading
 * dimension ld >= n + 1) with LAPACK's failed-pivot behaviour. When d_x is
 * non-NULL the right-hand side is row n of M (copied there from d_b when d_b
 * is non-NULL) and the solution of L L^T x = b is written to d_x. */
int irwls_dev_chol_solve(double *d_M, int n, int ld, const double *d_b, double *d_x);
/* The first failed pivot (1-based, 0 if none) of the last factorization in
 * *info; synchronous. */
int irwls_dev_chol_info(int *info);
int irwls_dev_zero_upper(double *d_M, int n, int ld);
/* out = A v (trans 0) or A^T v (trans 1), A column-major size x size. */
int irwls_dev_gemv(const double *d_A, const double *d_v, double *d_out, int size, int trans);

/* ---- full IRWLS steps (dev_full.cu) -------------------------------------- */
typedef struct irwls_sub_stats {
    double dW, nW, bmax, bmin;
    int nS1, nS3, pad0, pad1;
} irwls_sub_stats;

/* The inner-IRWLS device state on a working set of w rows; map[i] is the
 * row of `X` that working-set row i refers to. */
typedef struct irwls_sub_ws {
    int w;
    int cap;
    int *map;             /* device, w entries (points at mapbuf or a caller list) */
    double *a, *e, *beta, *bnew, *bsol, *bbest, *G13, *rhs, *GIN, *y, *dlt, *scal, *H;
    int *grp, *S1, *S3, *lst, *gl1, *gl3, *cnt, *mapbuf;
    irwls_sub_stats *stats;   /* device */
    irwls_sub_stats *h_stats; /* pinned host mirror */
    int ldH;
    void *tcs;                /* precision form: the training's tensor-core set (NULL: FP64 throughout) */
} irwls_sub_ws;

int irwls_sub_alloc(irwls_sub_ws *ws, int cap);
void irwls_sub_release(irwls_sub_ws *ws);
/* a_i and the groups at entry (src/full-train.c:131-155); e, beta and map
 * must be set; stats->nS1/nS3 filled. */
int irwls_sub_init(irwls_sub_ws *ws, const irwls_dev_set *X, double C);
/* G13 of the current S1/S3 lists (src/full-train.c:327-344). */
int irwls_sub_g13(irwls_sub_ws *ws, const irwls_dev_set *X, int n1, int n3);
/* One inner iteration: H and rhs, solve, weights, working-set error update,
 * a_i and groups (src/full-train.c:160-307). */
int irwls_sub_iterate(irwls_sub_ws *ws, const irwls_dev_set *X, double C, int n1, int n3);

/* Outer-loop steps (src/full-train.c:436-643). d_lst/d_cb/d_cnt are scratch
 * lists of at least l entries. */
typedef struct irwls_outer_counts {
    int nSW, nSIN, nSC, pad;
} irwls_outer_counts;
int irwls_full_gin(const irwls_dev_set *X, const int *d_SW, int nSW, const int *d_SIN, int nSIN,
                   const double *d_bnew, int *d_lst, double *d_cb, int *d_cnt, double *d_GIN);
int irwls_full_gather_ws(const int *d_SW, int nSW, const double *d_e, const double *d_beta, int l,
                         double *d_esub, double *d_bsub);
int irwls_full_apply_ws(const int *d_SW, int nSW, const double *d_bt, const double *d_beta, int l,
                        double *d_bnew, int *d_lst, double *d_cb, int *d_cnt, double *d_dbias);
int irwls_full_norms(const double *d_beta, const double *d_bnew, int n, double *d_out2);
int irwls_full_classify(const double *d_bnew, const double *d_e, const double *d_y, int l, double C,
                        int *d_SW, int *d_SC, int *d_SIN, irwls_outer_counts *d_counts);
int irwls_full_fill_ws(int *d_SW, int nSW, int *d_SIN, int nSIN, const int *d_SC, int nSC,
                       const int *d_perm, int space);

/* ---- budgeted IRWLS steps (dev_budget.cu) -------------------------------- */
/* SGMA: d_cent[0] must hold row l; L is row-major (ldL), KSC column-major
 * (l rows per centroid column). */
int irwls_sgma_first(const irwls_dev_set *X, int l, int *d_cent, double *d_L, int ldL, double *d_KSC);
int irwls_sgma_score(const irwls_dev_set *X, int l, const int *d_cand, int ncand, const int *d_cent, int s,
                     const double *d_L, int ldL, const double *d_KSC, double *d_W, double *d_Z, double *d_KN,
                     int ldz, double *d_eta, double *d_part);
int irwls_sgma_partials(int l);   /* rows of d_part (x 64) that a score step writes */
int irwls_sgma_select(const double *d_part, int l, const double *d_eta, const int *d_cand, int s, int *d_cent,
                      int *d_best, double *d_bestval);
int irwls_sgma_extend(const irwls_dev_set *X, int l, int s, const int *d_cent, const int *d_best,
                      const double *d_W, int ldz, double *d_L, int ldL, double *d_KSC);
/* IRWLSpar: KC row-major m x m, KSC row-major l x m. */
int irwls_par_build(const irwls_dev_set *X, int l, const int *d_idx, int m, double *d_KC, double *d_KSC);
int irwls_par_first(const double *d_y, int l, double M, int *d_act, double *d_sd, double *d_day);
size_t irwls_par_gram_part_bytes(int m, int P);
int irwls_par_gram(const double *d_KSC, int m, const int *d_act, int nact, const double *d_sd,
                   const double *d_day, const double *d_KC, double *d_K1, int ldK1, double *d_part, int P);
/* Precision form of the Gram on the tensor cores (dev_gram_tc.cu): A' as
   exact base-128 integer digits per column scale, digit-pair products summed
   exactly in FP32 tensor memory and drained into 96-bit integers; d_ws holds
   irwls_par_gram_tc_bytes(l, m) bytes for up to l active rows. */
size_t irwls_par_gram_tc_bytes(int l, int m);
/* Reads and clears device flag word 1: 0, or the code a tensor-core kernel
   left when one of its bounded waits ran out. */
int irwls_tc_status(void);
int irwls_par_gram_tc(const double *d_KSC, int m, const int *d_act, int nact, const double *d_sd,
                      const double *d_day, const double *d_KC, double *d_K1, int ldK1, double *d_part, int P,
                      void *d_ws);
int irwls_par_gram_reduce(const double *d_part, int P, int m, const double *d_KC, double *d_K1, int ldK1);
int irwls_par_residual(const double *d_KSC, int l, int m, const double *d_beta, const double *d_y, double C,
                       double M, double *d_e, double *d_Da);
int irwls_par_weights(const double *d_Da, const double *d_y, int l, int *d_act, double *d_sd, double *d_day,
                      int *d_nact);
int irwls_par_delta(const double *d_bnew, double *d_beta, int m, double *d_out2);

/* Precision form of full IRWLS (dev_tc.cu): split-BF16 copy of a set and the
 * tensor-core error update out_i = (init_i - sum_j cb_j k(x_i, x_{idx_j})) -
 * tail[0] over all of its rows, j < *d_n <= wmax. */
void *irwls_tc_set_create(const irwls_dev_set *X, int rows, int wmax);
/* e = y - K(:, SV) beta_SV - beta[l] in FP64 (dev_full.cu); lst/cb/cnt are scratch of l entries. */
int irwls_full_exact_errors(const irwls_dev_set *X, int l, const double *d_beta, int *d_lst, double *d_cb, int *d_cnt,
                            double *d_e);
/* The exact-error row set of the precision form (dev_full.cu): S = support
 * vectors, rows with |e y| < band, and SW; Snew = rows of S not flagged
 * before (none when all_exact); counts = {|S|, |Snew|}. */
int irwls_full_exact_set(const double *d_e, const double *d_y, const double *d_beta, int l, const int *d_SW, int nSW,
                         double band, int all_exact, int *d_flag, int *d_mark, int *d_S, int *d_Snew, int *d_counts);
int irwls_full_sv_list(const double *d_beta, int l, int *d_lst, double *d_cb, int *d_cnt);   /* beta != 0, i < l */
int irwls_dev_gather(const double *d_src, const int *d_idx, int n, double *d_dst);    /* dst[k] = src[idx[k]] */
int irwls_dev_scatter(const double *d_src, const int *d_idx, int n, double *d_dst);   /* dst[idx[k]] = src[k] */
/* Bound on |k(x_i, x_j)| over the set (1 for RBF, max q for linear). */
double irwls_tc_set_kbound(void *h);
void irwls_tc_set_free(void *h);
/* Exact-integer mode (dev_tc.cu): FP64 kernel row sums over the rows d_ia
 * (nA) against the list d_ib (nB entries, or *d_nB <= nbmax when d_nB is
 * given) with the dot products exact on the tensor cores:
 *   out_i = (init_i OP sum_j ((cb_j k(ia_i, ib_j)) sa_{ia_i}) sb_{ib_j}) - tail[0]
 * (the irwls_dev_kernel_rowsum arguments; cb, sa, sb, init, tail optional).
 * Returns 1 when the set does not allow it (values not integers after the
 * set's scale, norms too large for exact FP32 sums, raw RBF mode) or the
 * list may be longer than the set's gather room; the caller then uses the
 * FP64 kernels. */
int irwls_tc_exact_rowsum(void *h, const irwls_dev_set *X, const int *d_ia, int nA, const int *d_ib, int nB,
                          const int *d_nB, int nbmax, const double *d_cb, const double *d_sa, const double *d_sb,
                          int op, const double *d_init, const double *d_tail, double *d_out);
int irwls_tc_set_exact(void *h);
/* The same mode writing the kernel block: out[j * ldo + i] =
 * (k(ia_i, ib_j) sa_{ia_i}) sb_{ib_j} for i < nA, j < nB (only the blocks
 * touching the lower triangle when `lower`); 1 when not applicable. */
int irwls_tc_exact_block(void *h, const irwls_dev_set *X, const int *d_ia, int nA, const int *d_ib, int nB,
                         const double *d_sa, const double *d_sb, double *d_out, long long ldo, int lower);
int irwls_tc_kernel_rowsum(void *h, const int *d_idx, const int *d_n, const double *d_cb, const double *d_init,
                           const double *d_tail, double *d_out);
/* Precision-form prediction: d_out = b + sum_j w_j k(t_i, s_j) (or its sign)
 * from the tensor-core products; T and S share the feature width. */
int irwls_tc_predict(const irwls_dev_set *T, int n, const irwls_dev_set *S, int nSV, const double *d_w, double bias,
                     int hard, double *d_out);

/* Resident-dataset drivers (full_train.c, budgeted_train.c). */
int irwls_full_train_dev(const irwls_dev_set *X, int l, properties props, double *beta_out);
int irwls_sgma_dev(const irwls_dev_set *X, const svm_dataset *ds, properties props, int *cent_out);
int irwls_par_dev(const irwls_dev_set *X, int l, const int *idx, properties props, double *weights_out);

/* ---- prediction (dev_predict.cu) ----------------------------------------- */
int irwls_predict_soft(const irwls_dev_set *T, int n, const irwls_dev_set *S, int nSV, const double *d_w,
                       double bias, int hard, double *d_out);
size_t irwls_predict_linear_scratch(int width, int nsv);
int irwls_predict_linear(const irwls_dev_set *T, int n, const irwls_dev_set *S, int nSV, const double *d_w,
                         double bias, int hard, double *d_W, double *d_out);

/* ---- timing of the dominant kernels ------------------------------------- */
void irwls_prof_enable(int on);
int irwls_prof_on(void);
void irwls_prof_begin(int slot);
void irwls_prof_end(int slot);
int irwls_prof_collect(void);
void irwls_prof_read(int slot, double *ms, long long *launches);
void irwls_prof_reset(void);
enum { IRWLS_PROF_SGMA_GEMM = 0, IRWLS_PROF_GRAM = 1, IRWLS_PROF_ROWSUM = 2, IRWLS_PROF_CHOL = 3,
       IRWLS_PROF_PREDICT = 4, IRWLS_PROF_SGMA_CAND = 5, IRWLS_PROF_SGMA_UPDATE = 6, IRWLS_PROF_GRAM_SLICE = 7,
       IRWLS_PROF_PARSE = 8, IRWLS_PROF_SLOTS = 9 };
long long irwls_launch_count(void);
void irwls_count_launch(int n);

#ifdef __cplusplus
}
#endif

#endif
