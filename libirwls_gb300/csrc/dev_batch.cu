// dev_batch.cu -- batching form: many independent SVM trainings (a C x gamma
// grid, one-vs-rest splits, subsets of uneven size) run concurrently on one
// GPU.
//
// Each training of the reference is a chain of small, mostly latency-bound
// kernels with a host decision between iterations, so one training occupies
// a few SMs at a time. The batch driver runs `workers` trainings at once:
// every worker thread binds an execution context of its own (CUDA stream,
// status words, scratch, and a random generator that reproduces libc's
// srand/rand sequence), takes the next SVM from a queue ordered by
// decreasing size, uploads its dataset on its stream and trains it with the
// same host orchestration as trainFULL / SGMA + IRWLSpar. SVM i's random
// draws start from seeds[i], so its result is exactly what the single-call
// API gives after srand(seeds[i]). The worker count is either given or taken
// from the autotuner, which times the largest SVMs of a batch at a few
// concurrency levels and keeps the fastest.
#include <stdlib.h>
#include <string.h>

#include <algorithm>
#include <atomic>
#include <chrono>
#include <mutex>
#include <numeric>
#include <string>
#include <thread>
#include <vector>

#include "dev_common.cuh"

extern "C" int irwls_full_train_dev(const irwls_dev_set *X, int l, properties props, double *beta_out);
extern "C" int irwls_sgma_dev(const irwls_dev_set *X, const svm_dataset *ds, properties props, int *cent_out);
extern "C" int irwls_par_dev(const irwls_dev_set *X, int l, const int *idx, properties props, double *weights_out);
extern "C" int *randomCentroids(svm_dataset dataset, properties props);

namespace {

int g_tuned_workers = 0;  // 0: not tuned

int default_workers() { return g_tuned_workers > 0 ? g_tuned_workers : 16; }

// One full-IRWLS SVM in the calling thread's context.
int train_full_one(const svm_dataset &ds, const properties &p, unsigned seed, double **beta) {
    irwls_dev_set X;
    if (irwls_check_labels(&ds, ds.l) || irwls_dev_upload(&ds, ds.l, p.kernelType, p.Kgamma, 0, 0, &X)) return -1;
    double *b = (double *)malloc((size_t)(ds.l + 1) * sizeof(double));
    irwls_srand(seed);
    const int rc = b ? irwls_full_train_dev(&X, ds.l, p, b) : -3;
    irwls_dev_release(&X);
    if (rc) {
        free(b);
        b = nullptr;
    }
    *beta = b;
    return rc ? -1 : 0;
}

// Rows of a budgeted training: the class-mean rows l and l+1 are uploaded
// with the data.
int train_budgeted_one(const svm_dataset &ds, const properties &p, unsigned seed, int **cent, double **w) {
    *cent = nullptr;
    *w = nullptr;
    irwls_srand(seed);
    irwls_dev_set X;
    if (irwls_check_labels(&ds, ds.l) || irwls_dev_upload(&ds, ds.l + 2, p.kernelType, p.Kgamma, 0, 0, &X)) return -1;
    const int m = p.size > 0 ? p.size : 1;
    int *c = nullptr;
    int rc = 0;
    if (p.algorithm == 1) {
        c = (int *)malloc((size_t)m * sizeof(int));
        rc = irwls_sgma_dev(&X, &ds, p, c);
    } else {
        c = randomCentroids(ds, p);
    }
    double *ww = (double *)malloc((size_t)m * sizeof(double));
    if (!rc) rc = irwls_par_dev(&X, ds.l, c, p, ww);
    irwls_dev_release(&X);
    if (rc) {
        free(c);
        free(ww);
        return -1;
    }
    *cent = c;
    *w = ww;
    return 0;
}

// Runs job(i) for i in `order` on `workers` threads, each in its own context.
// Returns 0 or the first error (its message copied into the caller's context).
template <class Job>
int run_pool(const std::vector<int> &order, int workers, Job job) {
    if (irwls_dev_init()) return -1;
    workers = std::max(1, std::min<int>(workers, (int)order.size()));
    std::atomic<int> next{0};
    std::mutex mu;
    int first_err = 0;
    std::string first_msg;
    std::vector<std::thread> threads;
    for (int w = 0; w < workers; ++w) {
        threads.emplace_back([&]() {
            void *ctx = irwls_ctx_create();
            if (!ctx) {
                std::lock_guard<std::mutex> g(mu);
                if (!first_err) {
                    first_err = -2;
                    first_msg = "cannot create a worker context";
                }
                return;
            }
            irwls_ctx_bind(ctx);
            for (int k; (k = next++) < (int)order.size();) {
                if (job(order[k]) != 0) {
                    char msg[512];
                    const int e = irwls_ctx_error(ctx, msg, sizeof msg);
                    std::lock_guard<std::mutex> g(mu);
                    if (!first_err) {
                        first_err = e ? e : -1;
                        first_msg = msg;
                    }
                    irwls_clear_error();
                }
            }
            irwls_ctx_bind(nullptr);
            irwls_ctx_destroy(ctx);
        });
    }
    for (auto &t : threads) t.join();
    if (first_err) irwls_set_error(first_err, "batch: %s", first_msg.c_str());
    return first_err;
}

std::vector<int> by_size(const svm_dataset *ds, int count) {
    std::vector<int> order(count);
    std::iota(order.begin(), order.end(), 0);
    std::stable_sort(order.begin(), order.end(), [&](int a, int b) { return ds[a].l > ds[b].l; });
    return order;
}

}  // namespace

extern "C" int irwls_full_train_batch(const svm_dataset *datasets, const properties *props, const unsigned *seeds,
                                      int count, int workers, double **betas) {
    irwls_clear_error();
    for (int i = 0; i < count; ++i) betas[i] = nullptr;
    if (count <= 0) return 0;
    return run_pool(by_size(datasets, count), workers > 0 ? workers : default_workers(), [&](int i) {
        return train_full_one(datasets[i], props[i], seeds ? seeds[i] : 1u, &betas[i]);
    });
}

extern "C" int irwls_budgeted_train_batch(const svm_dataset *datasets, const properties *props,
                                          const unsigned *seeds, int count, int workers, int **centroids,
                                          double **weights) {
    irwls_clear_error();
    for (int i = 0; i < count; ++i) {
        centroids[i] = nullptr;
        weights[i] = nullptr;
    }
    if (count <= 0) return 0;
    return run_pool(by_size(datasets, count), workers > 0 ? workers : default_workers(), [&](int i) {
        return train_budgeted_one(datasets[i], props[i], seeds ? seeds[i] : 1u, &centroids[i], &weights[i]);
    });
}

// Times full-IRWLS trainings of the largest `sample` SVMs of the batch at
// each candidate worker count (each candidate runs `sample` trainings, the
// sample repeated as needed so that every worker has one), keeps the count
// with the highest rows-per-second and returns it; later batches called with
// workers <= 0 use it.
extern "C" int irwls_batch_autotune(const svm_dataset *datasets, const properties *props, int count, int sample) {
    if (count <= 0) return default_workers();
    const std::vector<int> order = by_size(datasets, count);
    const int cand[] = {4, 8, 16, 24, 32, 48};
    double best_rate = -1.0;
    int best = default_workers();
    for (int w : cand) {
        const int jobs = std::max(sample, w);
        std::vector<int> sub(jobs);
        for (int k = 0; k < jobs; ++k) sub[k] = order[k % std::min(sample, count)];
        double rows = 0.0;
        for (int i : sub) rows += datasets[i].l;
        const auto t0 = std::chrono::steady_clock::now();
        std::atomic<int> slot{0};
        std::vector<double *> betas(jobs, nullptr);
        const int rc = run_pool(sub, w, [&](int i) {
            const int k = slot++;
            return train_full_one(datasets[i], props[i], 1u, &betas[k]);
        });
        const double dt = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
        for (double *b : betas) free(b);
        if (rc) return -1;
        const double rate = rows / dt;
        if (rate > best_rate) {
            best_rate = rate;
            best = w;
        }
    }
    g_tuned_workers = best;
    return best;
}

extern "C" void irwls_batch_set_workers(int workers) { g_tuned_workers = workers > 0 ? workers : 0; }
