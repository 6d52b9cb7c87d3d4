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
};

static int run_batch_trial(axbc_ctx *c, void *arg)
{
    Trial *t = (Trial *)arg;
    std::vector<axbc_pivot_stats> st(t->k);
    TRY(axbc_run_batch(c, t->v0, t->p, t->k, t->H, st.data()));
    t->te = 0;
    for (auto &x : st) t->te += x.te;
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

extern "C" int axbc_autotune(axbc_ctx *c, const uint32_t *pivots, int npivots, int H,
                             axbc_tuning *out)
{
    CHECK_ARG(c && pivots && out, "axbc_autotune: null argument");
    CHECK_ARG(npivots >= 1, "axbc_autotune: need at least one trial pivot");
    for (int i = 0; i < npivots; i++) CHECK_ARG(pivots[i] < c->g->n, "axbc_autotune: pivot >= n");
    const int kb = std::min(npivots, AXBC_MAX_BATCH);
    std::vector<double> p(kb, 1.0 / (double)c->g->n);
    const double cand[] = {0.03125, 0.125, 0.5, 1.0, 2.0, 8.0, 32.0};
    // batched: direction factor at full width, then the width
    double best_f = c->push_factor_batch, best_rate = -1;
    for (double f : cand) {
        c->push_factor_batch = f;
        Trial t{pivots, p.data(), kb, H, 0};
        float ms = 0;
        TRY(timed(c, &ms, run_batch_trial, &t));  // warm
        TRY(timed(c, &ms, run_batch_trial, &t));
        const double rate = t.te / (ms * 1e-3);
        if (rate > best_rate) {
            best_rate = rate;
            best_f = f;
        }
    }
    c->push_factor_batch = best_f;
    int best_w = kb;
    double best_wrate = best_rate;
    for (int w = 8; w < kb; w *= 2) {
        Trial t{pivots, p.data(), w, H, 0};
        float ms = 0;
        TRY(timed(c, &ms, run_batch_trial, &t));
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
        Trial t{pivots, p.data(), kp, H, 0};
        float ms = 0;
        TRY(timed(c, &ms, run_plain_trial, &t));
        const double rate = t.te / (ms * 1e-3);
        if (rate > best_srate) {
            best_srate = rate;
            best_fs = f;
        }
    }
    c->push_factor_single = best_fs;
    TRY(axbc_ctx_reset(c));
    out->push_factor_single = best_fs;
    out->push_factor_batch = best_f;
    out->batch_width = best_w;
    out->pad = 0;
    out->batch_te_per_s = best_wrate;
    out->plain_te_per_s = best_srate;
    return AXBC_OK;
}
