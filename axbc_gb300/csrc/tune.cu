// Autotuner: picks the forward direction-switch factors (batched and plain)
// and the batch width by timing trial passes on the context's own graph.
#include <algorithm>
#include <vector>

#include "common.cuh"

static int timed(axbc_ctx *c, float *ms, int (*fn)(axbc_ctx *, void *), void *arg)
{
    cudaEvent_t a, b;
    CU(cudaEventCreate(&a));
    CU(cudaEventCreate(&b));
    CU(cudaEventRecord(a, c->stream));
    int rc = fn(c, arg);
    CU(cudaEventRecord(b, c->stream));
    CU(cudaEventSynchronize(b));
    CU(cudaEventElapsedTime(ms, a, b));
    cudaEventDestroy(a);
    cudaEventDestroy(b);
    return rc;
}

struct Trial {
    const uint32_t *v0;
    const double *p;
    int k, H;
    uint64_t te;
    int w;  // batch width (batched trials)
};

// the trial pivots in batches of t->w (t->k pivots in all)
static int run_batch_trial(axbc_ctx *c, void *arg)
{
    Trial *t = (Trial *)arg;
    t->te = 0;
    for (int off = 0; off < t->k; off += t->w) {
        const int k = std::min(t->w, t->k - off);
        std::vector<axbc_pivot_stats> st(k);
        TRY(axbc_run_batch(c, t->v0 + off, t->p + off, k, t->H, st.data()));
        for (auto &x : st) t->te += x.te;
    }
    return AXBC_OK;
}

// best (shortest) of `reps` timed runs after one untimed run
static int best_of(axbc_ctx *c, int reps, int (*fn)(axbc_ctx *, void *), void *arg, float *best)
{
    float ms = 0;
    TRY(timed(c, &ms, fn, arg));
    *best = 1e30f;
    for (int r = 0; r < reps; r++) {
        TRY(timed(c, &ms, fn, arg));
        *best = std::min(*best, ms);
    }
    return AXBC_OK;
}

static int run_plain_trial(axbc_ctx *c, void *arg)
{
    Trial *t = (Trial *)arg;
    t->te = 0;
    for (int i = 0; i < t->k; i++) {
        axbc_pivot_stats st;
        TRY(axbc_run_pivot(c, t->v0[i], t->p[i], t->H, &st));
        t->te += st.te;
    }
    return AXBC_OK;
}

static int tune_trials(axbc_ctx *c, const uint32_t *pivots, int npivots, int H, axbc_tuning *out);

extern "C" int axbc_autotune(axbc_ctx *c, const uint32_t *pivots, int npivots, int H,
                             axbc_tuning *out)
{
    CHECK_ARG(c && pivots && out, "axbc_autotune: null argument");
    CHECK_ARG(npivots >= 1, "axbc_autotune: need at least one trial pivot");
    for (int i = 0; i < npivots; i++) CHECK_ARG(pivots[i] < c->g->n, "axbc_autotune: pivot >= n");
    // the trial passes add into bc: the context's bc and last dependency vector
    // are set aside first and put back at the end, so tuning leaves its results
    // as they were
    const uint64_t n = c->g->n;
    DBuf keep;
    TRY(keep.alloc(2 * n * 4));
    CU(cudaMemcpyAsync(keep.as<float>(), c->bc, n * 4, cudaMemcpyDeviceToDevice, c->stream));
    CU(cudaMemcpyAsync(keep.as<float>() + n, c->delta_last, n * 4, cudaMemcpyDeviceToDevice, c->stream));
    const bool dl_valid = c->delta_last_valid;
    const double f_batch0 = c->push_factor_batch, f_single0 = c->push_factor_single;
    int rc = tune_trials(c, pivots, npivots, H, out);
    if (rc != AXBC_OK) {
        c->push_factor_batch = f_batch0;
        c->push_factor_single = f_single0;
    }
    cudaError_t e = cudaMemcpyAsync(c->bc, keep.as<float>(), n * 4, cudaMemcpyDeviceToDevice, c->stream);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(c->delta_last, keep.as<float>() + n, n * 4, cudaMemcpyDeviceToDevice, c->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
    c->delta_last_valid = dl_valid;
    if (rc == AXBC_OK && e != cudaSuccess) return axbc_cuda_fail(e, "autotune restore", __FILE__, __LINE__);
    return rc;
}

// the timed trials of axbc_autotune; leaves the chosen factors in the context
static int tune_trials(axbc_ctx *c, const uint32_t *pivots, int npivots, int H, axbc_tuning *out)
{
    // all trial pivots (up to 4 batches), each candidate timed as the best of 2
    const int kb = std::min(npivots, 4 * AXBC_MAX_BATCH);
    std::vector<double> p(kb, 1.0 / (double)c->g->n);
    const double cand[] = {0.03125, 0.125, 0.5, 1.0, 2.0, 4.0, 8.0, 16.0, 32.0};
    // batched: direction factor at full width, then the width
    double best_f = c->push_factor_batch, best_rate = -1;
    const int wfull = std::min(kb, AXBC_MAX_BATCH);
    for (double f : cand) {
        c->push_factor_batch = f;
        Trial t{pivots, p.data(), kb, H, 0, wfull};
        float ms = 0;
        TRY(best_of(c, 2, run_batch_trial, &t, &ms));
        const double rate = t.te / (ms * 1e-3);
        if (rate > best_rate) {
            best_rate = rate;
            best_f = f;
        }
    }
    c->push_factor_batch = best_f;
    int best_w = wfull;
    double best_wrate = best_rate;
    for (int w = 8; w < wfull; w *= 2) {
        Trial t{pivots, p.data(), kb, H, 0, w};
        float ms = 0;
        TRY(best_of(c, 2, run_batch_trial, &t, &ms));
        const double rate = t.te / (ms * 1e-3);
        if (rate > best_wrate * 1.02) {
            best_wrate = rate;
            best_w = w;
        }
    }
    // plain form: direction factor on up to 4 pivots
    const int kp = std::min(npivots, 4);
    double best_fs = c->push_factor_single, best_srate = -1;
    for (double f : cand) {
        c->push_factor_single = f;
        Trial t{pivots, p.data(), kp, H, 0, 1};
        float ms = 0;
        TRY(timed(c, &ms, run_plain_trial, &t));
        const double rate = t.te / (ms * 1e-3);
        if (rate > best_srate) {
            best_srate = rate;
            best_fs = f;
        }
    }
    c->push_factor_single = best_fs;
    out->push_factor_single = best_fs;
    out->push_factor_batch = best_f;
    out->batch_width = best_w;
    out->pad = 0;
    out->batch_te_per_s = best_wrate;
    out->plain_te_per_s = best_srate;
    return AXBC_OK;
}
