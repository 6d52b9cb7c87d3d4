// Device state of one sampled run (the reference's main loop for one job) and
// the steps that drive it; shared by axbc_run_sampled and the request server.
#pragma once
#include <vector>

#include "common.cuh"

struct SampledRun {
    axbc_run_params prm;
    SamplerState *ss;
    SamplerState *ss_host;  // pinned mirror, valid after the stream syncs
    float *bc, *delta_last;
    uint8_t *used;
    uint32_t *checks;
    float *checkval;
    double *dyn_local, *dyn_csum, *dyn_local2, *dyn_csum2;
    uint32_t *hist_v;
    double *hist_p;
    uint64_t hist_cap;
    int batches;
};

// device bytes of a run with its own buffers
uint64_t sr_bytes(uint64_t n, const axbc_run_params *prm);
int sr_check_params(const axbc_graph *g, const axbc_run_params *prm, int max_width);
int sr_alloc(axbc_graph *g, const axbc_run_params *prm, SampledRun *r);
void sr_free(SampledRun *r);
int sr_begin(axbc_ctx *c, SampledRun *r);
int sr_draw(axbc_ctx *c, SampledRun *r);
int sr_nb(const SampledRun *r);
bool sr_done(const SampledRun *r);  // ss_host's done flag
bool sr_finished(const SampledRun *r);
// a pass of the drawn pivots [off, off + cnt) of the run's round in lanes
// lane0.. (cnt is capped by the round and the lanes left)
int sr_load(axbc_ctx *c, SampledRun *r, int off, int lane0, int cnt = AXBC_WMAX);
int sr_post(axbc_ctx *c, SampledRun *r, int off, int lane0, int cnt = AXBC_WMAX);
// Bader's test between two passes of a round (before its next pivot); the
// result reaches ss_host->done once the stream has synchronised
int sr_stop_test(axbc_ctx *c, SampledRun *r);
int sr_result(axbc_ctx *c, SampledRun *r, axbc_run_result *res, std::vector<uint32_t> *piv,
              std::vector<double> *probs, std::vector<uint32_t> *checks);
