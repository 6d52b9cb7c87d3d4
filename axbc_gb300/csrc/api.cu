// Contexts, results, errors: the handle-based part of the C ABI.
#include <cstdarg>
#include <cstdio>
#include <cstring>

#include "common.cuh"

static thread_local char g_err[512] = "";

void axbc_set_error(const char *fmt, ...)
{
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(g_err, sizeof g_err, fmt, ap);
    va_end(ap);
}

int axbc_cuda_fail(cudaError_t e, const char *what, const char *file, int line)
{
    const char *base = strrchr(file, '/');
    axbc_set_error("CUDA error %d (%s) in %s at %s:%d", (int)e, cudaGetErrorString(e), what,
                   base ? base + 1 : file, line);
    if (e == cudaErrorMemoryAllocation) {
        (void)cudaGetLastError();
        return AXBC_ERR_NOMEM;
    }
    return AXBC_ERR_CUDA;
}

extern "C" const char *axbc_last_error(void) { return g_err; }

extern "C" const char *axbc_version(void) { return "axbc_gb300 0.1 (sm_103a)"; }

extern "C" const char *axbc_status_str(int st)
{
    switch (st) {
    case AXBC_OK: return "ok";
    case AXBC_ERR_INVALID: return "invalid argument";
    case AXBC_ERR_CUDA: return "CUDA error";
    case AXBC_ERR_NOMEM: return "out of memory";
    case AXBC_ERR_TIMEOUT: return "device wait timed out";
    case AXBC_ERR_RANGE: return "size beyond a limit";
    case AXBC_ERR_STATE: return "call out of order";
    case AXBC_ERR_BUSY: return "admission refused";
    default: return "unknown status";
    }
}

int axbc_grid_for(const axbc_ctx *c, int tpb, int blocks_per_sm)
{
    (void)tpb;
    return (c->num_sms > 0 ? c->num_sms : 152) * blocks_per_sm;
}

static cudaEvent_t pool_get(axbc_ctx *c)
{
    if (!c->ev_pool.empty()) {
        cudaEvent_t e = c->ev_pool.back();
        c->ev_pool.pop_back();
        return e;
    }
    cudaEvent_t e = nullptr;
    if (cudaEventCreate(&e) != cudaSuccess) return nullptr;
    return e;
}

void axbc_prof_start(axbc_ctx *c, int kind, double bytes)
{
    c->launches++;
    if (!c->prof_on) return;
    ProfRec r{kind, bytes, pool_get(c), pool_get(c), -1};
    if (r.a) cudaEventRecord(r.a, c->stream);
    c->prof.push_back(r);
}

void axbc_prof_stop(axbc_ctx *c)
{
    if (!c->prof_on || c->prof.empty()) return;
    ProfRec &r = c->prof.back();
    if (r.b) cudaEventRecord(r.b, c->stream);
}

static void prof_clear(axbc_ctx *c)
{
    for (ProfRec &r : c->prof) {
        if (r.a) c->ev_pool.push_back(r.a);
        if (r.b) c->ev_pool.push_back(r.b);
    }
    c->prof.clear();
}

extern "C" int axbc_ctx_profile(axbc_ctx *c, int enable)
{
    CHECK_ARG(c, "axbc_ctx_profile: null context");
    CU(cudaStreamSynchronize(c->stream));
    prof_clear(c);
    c->prof_on = enable != 0;
    return AXBC_OK;
}

extern "C" int axbc_ctx_profile_read(axbc_ctx *c, double *ms, uint64_t *count, double *bytes,
                                     int nkinds)
{
    CHECK_ARG(c && ms && count && bytes, "axbc_ctx_profile_read: null argument");
    CU(cudaStreamSynchronize(c->stream));
    for (int k = 0; k < nkinds; k++) {
        ms[k] = 0;
        count[k] = 0;
        bytes[k] = 0;
    }
    for (const ProfRec &r : c->prof) {
        if (r.kind >= nkinds || !r.a || !r.b) continue;
        float t = 0;
        CU(cudaEventElapsedTime(&t, r.a, r.b));
        ms[r.kind] += t;
        count[r.kind] += 1;
        bytes[r.kind] += r.bytes;
    }
    prof_clear(c);
    return AXBC_OK;
}

// Every timed launch since profiling was enabled (or the last read), in
// launch order: kind, forward level (-1: none), milliseconds, model bytes.
// Reads up to cap records into the arrays (NULL: skip); *count = all records;
// the records are kept (axbc_ctx_profile_read clears them).
extern "C" int axbc_ctx_profile_records(axbc_ctx *c, int32_t *kinds, int32_t *tags, float *ms,
                                        double *bytes, uint64_t cap, uint64_t *count)
{
    CHECK_ARG(c && count, "axbc_ctx_profile_records: null argument");
    CU(cudaStreamSynchronize(c->stream));
    uint64_t i = 0;
    for (const ProfRec &r : c->prof) {
        if (!r.a || !r.b) continue;
        if (i < cap) {
            float t = 0;
            CU(cudaEventElapsedTime(&t, r.a, r.b));
            if (kinds) kinds[i] = r.kind;
            if (tags) tags[i] = r.tag;
            if (ms) ms[i] = t;
            if (bytes) bytes[i] = r.bytes;
        }
        i++;
    }
    *count = i;
    return AXBC_OK;
}

extern "C" int axbc_ctx_count(axbc_ctx *c, int enable)
{
    CHECK_ARG(c, "axbc_ctx_count: null context");
    CU(cudaStreamSynchronize(c->stream));
    if (enable && !c->wcount) {
        TRY(axbc_dalloc((void **)&c->wcount, KP_NKINDS * WC_NFIELDS * 8, &c->bytes));
        CU(cudaMemset(c->wcount, 0, KP_NKINDS * WC_NFIELDS * 8));
    }
    c->count_on = enable != 0;
    return AXBC_OK;
}

extern "C" int axbc_ctx_count_read(axbc_ctx *c, uint64_t *counts, int nkinds)
{
    CHECK_ARG(c && counts, "axbc_ctx_count_read: null argument");
    CHECK_ARG(nkinds >= 0 && nkinds <= KP_NKINDS, "axbc_ctx_count_read: nkinds out of range");
    for (int i = 0; i < nkinds * WC_NFIELDS; i++) counts[i] = 0;
    if (!c->wcount) return AXBC_OK;
    CU(cudaStreamSynchronize(c->stream));
    unsigned long long h[KP_NKINDS * WC_NFIELDS];
    CU(cudaMemcpy(h, c->wcount, sizeof(h), cudaMemcpyDeviceToHost));
    CU(cudaMemset(c->wcount, 0, sizeof(h)));
    for (int i = 0; i < nkinds * WC_NFIELDS; i++) counts[i] = h[i];
    return AXBC_OK;
}

extern "C" int axbc_ctx_launches(const axbc_ctx *c, uint64_t *launches)
{
    CHECK_ARG(c && launches, "axbc_ctx_launches: null argument");
    *launches = c->launches;
    return AXBC_OK;
}

extern "C" int axbc_ctx_create(axbc_graph *g, void *stream, axbc_ctx **out)
{
    CHECK_ARG(g && out, "axbc_ctx_create: null argument");
    axbc_ctx *c = new axbc_ctx();
    c->g = g;
    int dev = 0;
    CU(cudaGetDevice(&dev));
    CU(cudaDeviceGetAttribute(&c->num_sms, cudaDevAttrMultiProcessorCount, dev));
    if (stream) {
        c->stream = (cudaStream_t)stream;
    } else {
        CU(cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking));
        c->own_stream = true;
    }
    int rc = axbc_dalloc((void **)&c->bc, g->n * 4, &c->bytes);
    if (!rc) rc = axbc_dalloc((void **)&c->delta_last, g->n * 4, &c->bytes);
    if (rc) {
        axbc_ctx_destroy(c);
        return rc;
    }
    CU(cudaMemsetAsync(c->bc, 0, g->n * 4, c->stream));
    CU(cudaMemsetAsync(c->delta_last, 0, g->n * 4, c->stream));
    CU(cudaStreamSynchronize(c->stream));
    *out = c;
    return AXBC_OK;
}

extern "C" int axbc_ctx_destroy(axbc_ctx *c)
{
    if (!c) return AXBC_OK;
    if (c->stream) cudaStreamSynchronize(c->stream);
    axbc_dfree(c->bc);
    axbc_dfree(c->delta_last);
    axbc_dfree(c->wcount);
    axbc_dfree(c->gsync);
    axbc_dfree(c->lvl);
    axbc_dfree(c->sigma);
    axbc_dfree(c->delta);
    axbc_dfree(c->queue);
    axbc_dfree(c->partial);
    axbc_dfree(c->pc);
    if (c->pc_host) cudaFreeHost(c->pc_host);
    axbc_dfree(c->seen);
    for (uint32_t *p : c->fmask) axbc_dfree(p);
    axbc_dfree(c->msigma);
    axbc_dfree(c->mdelta);
    axbc_dfree(c->mq);
    axbc_dfree(c->task_ctr);
    axbc_dfree(c->fmtab);
    axbc_dfree(c->ctrs);
    axbc_dfree(c->d_level_te);
    axbc_dfree(c->d_level_cnt);
    axbc_dfree(c->d_level_mode);
    axbc_dfree(c->lpool);
    axbc_dfree(c->lstart);
    axbc_dfree(c->lcount);
    axbc_dfree(c->lcap);
    axbc_dfree(c->lheavy);
    for (int i = 0; i < 2; i++) {
        if (c->fwd_step_exec[i]) cudaGraphExecDestroy(c->fwd_step_exec[i]);
        if (c->bwd_step_exec[i]) cudaGraphExecDestroy(c->bwd_step_exec[i]);
    }
    axbc_dfree(c->mpartial);
    axbc_dfree(c->bi);
    if (c->bi_host) cudaFreeHost(c->bi_host);
    axbc_dfree(c->ss);
    if (c->ss_host) cudaFreeHost(c->ss_host);
    axbc_dfree(c->used);
    axbc_dfree(c->checks);
    axbc_dfree(c->checkval);
    axbc_dfree(c->dyn_local);
    axbc_dfree(c->dyn_csum);
    axbc_dfree(c->dyn_local2);
    axbc_dfree(c->dyn_csum2);
    axbc_dfree(c->wtmp);
    prof_clear(c);
    for (cudaEvent_t e : c->ev_pool) cudaEventDestroy(e);
    if (c->rb_ev) cudaEventDestroy(c->rb_ev);
    if (c->own_stream && c->stream) cudaStreamDestroy(c->stream);
    delete c;
    return AXBC_OK;
}

extern "C" int axbc_ctx_reset(axbc_ctx *c)
{
    CHECK_ARG(c, "axbc_ctx_reset: null context");
    CU(cudaMemsetAsync(c->bc, 0, c->g->n * 4, c->stream));
    CU(cudaMemsetAsync(c->delta_last, 0, c->g->n * 4, c->stream));
    CU(cudaStreamSynchronize(c->stream));
    c->delta_last_valid = true;
    c->run_pivots.clear();
    c->run_probs.clear();
    return AXBC_OK;
}

extern "C" int axbc_ctx_bytes(const axbc_ctx *c, uint64_t *bytes)
{
    CHECK_ARG(c && bytes, "axbc_ctx_bytes: null argument");
    *bytes = c->bytes;
    return AXBC_OK;
}

extern "C" int axbc_ctx_set_tuning(axbc_ctx *c, double pf_single, double pf_batch)
{
    CHECK_ARG(c, "axbc_ctx_set_tuning: null context");
    CHECK_ARG(pf_single >= 0 && pf_batch >= 0, "axbc_ctx_set_tuning: factors must be >= 0");
    c->push_factor_single = pf_single;
    c->push_factor_batch = pf_batch;
    return AXBC_OK;
}

extern "C" int axbc_get_bc(axbc_ctx *c, float *bc_host)
{
    CHECK_ARG(c && bc_host, "axbc_get_bc: null argument");
    CU(cudaMemcpyAsync(bc_host, c->bc, c->g->n * 4, cudaMemcpyDeviceToHost, c->stream));
    CU(cudaStreamSynchronize(c->stream));
    return AXBC_OK;
}

extern "C" int axbc_get_delta(axbc_ctx *c, float *delta_host)
{
    CHECK_ARG(c && delta_host, "axbc_get_delta: null argument");
    const float *src = c->delta_last_valid || !c->delta ? c->delta_last : c->delta;
    CU(cudaMemcpyAsync(delta_host, src, c->g->n * 4, cudaMemcpyDeviceToHost, c->stream));
    CU(cudaStreamSynchronize(c->stream));
    return AXBC_OK;
}

extern "C" int axbc_get_sigma(axbc_ctx *c, uint32_t *sigma_host)
{
    CHECK_ARG(c && sigma_host, "axbc_get_sigma: null argument");
    CHECK_ARG(c->sigma, "axbc_get_sigma: no plain pivot has run");
    CU(cudaMemcpyAsync(sigma_host, c->sigma, c->g->n * 4, cudaMemcpyDeviceToHost, c->stream));
    CU(cudaStreamSynchronize(c->stream));
    return AXBC_OK;
}

extern "C" int axbc_get_levels(axbc_ctx *c, int32_t *lvl_host)
{
    CHECK_ARG(c && lvl_host, "axbc_get_levels: null argument");
    CHECK_ARG(c->lvl, "axbc_get_levels: no plain pivot has run");
    CU(cudaMemcpyAsync(lvl_host, c->lvl, c->g->n * 4, cudaMemcpyDeviceToHost, c->stream));
    CU(cudaStreamSynchronize(c->stream));
    return AXBC_OK;
}

extern "C" int axbc_bc_device_ptr(axbc_ctx *c, float **bc_dev)
{
    CHECK_ARG(c && bc_dev, "axbc_bc_device_ptr: null argument");
    *bc_dev = c->bc;
    return AXBC_OK;
}

extern "C" int axbc_ctx_sync(axbc_ctx *c)
{
    CHECK_ARG(c, "axbc_ctx_sync: null context");
    CU(cudaStreamSynchronize(c->stream));
    return AXBC_OK;
}
