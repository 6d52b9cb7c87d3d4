// Request server: many sampled runs over resident graphs, batched across
// requests.  The reference runs one job per process (src/axbc2d.c:2729-3156);
// here every admitted request keeps its own sampler, bc, last delta and check
// vertices on the device, and each resident graph has a worker thread and a
// stream that pack the drawn rounds of the graph's requests into the lanes of
// a shared multi-source pass (continuous batching); passes on different graphs
// overlap on the device.  A request's lanes are contiguous and in its pivot
// order, its update goes to its own bc vector, and its Bader replay reads only
// its own lanes, so every request gets the bits it would get alone.
//
// Admission: a request's device bytes (sr_bytes) must fit in what the budget
// has left; requests wait in arrival order, and a smaller later one may pass
// a larger one that does not fit yet.  On a graph, the rounds that have
// waited longest go first into the next pass.
#include <algorithm>
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <map>
#include <memory>
#include <mutex>
#include <string>
#include <thread>
#include <vector>

#include "common.cuh"
#include "sampled.cuh"

// pivots per round of the requests whose width does not change their bits
#ifndef AXBC_SERVE_STATIC_WIDTH
#define AXBC_SERVE_STATIC_WIDTH AXBC_WMAX
#endif

namespace {

uint64_t now_ns()
{
    return (uint64_t)std::chrono::duration_cast<std::chrono::nanoseconds>(
               std::chrono::steady_clock::now().time_since_epoch())
        .count();
}



struct Request;

struct ServeGraph {
    axbc_graph *g = nullptr;
    int H = 0;
    axbc_ctx *ctx = nullptr;  // the shared multi-source buffers of this graph
    cudaStream_t stream = nullptr;
    std::thread worker;             // drives this graph's passes on its own stream
    std::vector<Request *> active;  // admitted requests; touched by this worker only
    uint64_t passes = 0, lanes = 0, busy_ns = 0;  // worker's account (read under the mutex)
};

struct Request {
    uint64_t id = 0;
    int graph = 0;
    ServeGraph *G = nullptr;  // the graph's entry (stable; graphs are never removed)
    axbc_run_params prm{};
    int state = AXBC_REQ_QUEUED;
    int status = AXBC_OK;
    std::string err;
    uint64_t bytes = 0;
    SampledRun run{};
    bool allocated = false;
    bool need_draw = false;  // worker: the next round is not drawn yet
    uint64_t drawn_at = 0;   // worker: pass count when the pending round was drawn
    int off = 0;             // worker: first pivot of the drawn round not yet traversed
    int want = AXBC_WMAX;    // worker: how many of them the next pass takes
    bool test_pending = false;  // worker: the stop test between two passes is in flight
    bool worker_ref = false; // in the worker's active list (guarded by the mutex)
    bool released = false;   // released while the worker still held it
    axbc_run_result res{};
    std::vector<float> bc;
    std::vector<uint32_t> pivots;
    std::vector<double> probs;
    uint64_t t_submit = 0, t_start = 0, t_finish = 0;
};

}  // namespace

struct axbc_server {
    int device = 0;
    uint64_t budget = 0, in_use = 0;
    std::vector<std::unique_ptr<ServeGraph>> graphs;  // stable addresses for the workers
    std::mutex mu;
    std::condition_variable work_cv, done_cv;
    std::deque<uint64_t> queue;  // submitted, not admitted, in arrival order
    std::map<uint64_t, std::unique_ptr<Request>> reqs;
    bool stop = false;
    uint64_t next_id = 1;
    uint64_t passes = 0, lanes = 0, admitted = 0, completed = 0;
};

static void req_fail(axbc_server *S, Request *r, int st)
{
    std::lock_guard<std::mutex> lk(S->mu);
    r->state = AXBC_REQ_FAILED;
    r->status = st;
    r->err = axbc_last_error();
    r->t_finish = now_ns();
    S->done_cv.notify_all();
}

// result to host memory, device state freed, budget returned
static void req_finish(axbc_server *S, Request *r)
{
    axbc_ctx *c = r->G->ctx;
    int st = sr_result(c, &r->run, &r->res, &r->pivots, &r->probs, nullptr);
    if (st == AXBC_OK) {
        r->bc.resize(r->G->g->n);
        if (cudaMemcpy(r->bc.data(), r->run.bc, r->bc.size() * 4, cudaMemcpyDeviceToHost) != cudaSuccess)
            st = axbc_cuda_fail(cudaGetLastError(), "request result", __FILE__, __LINE__);
    }
    sr_free(&r->run);
    r->allocated = false;
    std::lock_guard<std::mutex> lk(S->mu);
    S->in_use -= r->bytes;
    if (st == AXBC_OK) {
        r->state = AXBC_REQ_DONE;
        S->completed++;
    } else {
        r->state = AXBC_REQ_FAILED;
        r->status = st;
        r->err = axbc_last_error();
    }
    r->t_finish = now_ns();
    S->done_cv.notify_all();
}

// One pass over graph gi: draw the rounds of its requests that need one,
// then pack drawn rounds into the lanes of one multi-source pass.  The first
// round of a request with Bader's stop goes into passes 1, 1, 2, 4, ...
// pivots at a time with the stop tested between them, as axbc_run_sampled
// does, so a request whose stop comes early holds no lanes past it.
static int serve_pass(axbc_server *S, ServeGraph &G, std::vector<Request *> &runs)
{
    axbc_ctx *c = G.ctx;
    bool pending = false;
    for (Request *r : runs) pending |= r->test_pending;
    if (pending) {
        CU(cudaStreamSynchronize(c->stream));
        for (Request *r : runs)
            if (r->test_pending) {
                r->test_pending = false;
                // stopped between two passes: the next draw ends the run
                if (sr_done(&r->run)) r->need_draw = true;
            }
    }
    bool drew = false;
    for (Request *r : runs)
        if (r->need_draw) {
            TRY(sr_draw(c, &r->run));
            drew = true;
        }
    if (drew) CU(cudaStreamSynchronize(c->stream));
    std::vector<Request *> ready;
    for (Request *r : runs) {
        if (r->need_draw) {
            r->need_draw = false;
            r->drawn_at = G.passes;
            r->off = 0;
            r->want = r->prm.bader_c > 0 && r->run.batches == 0 ? 1 : AXBC_WMAX;
            if (sr_finished(&r->run)) {
                req_finish(S, r);
                continue;
            }
            if (sr_nb(&r->run) == 0) {
                // only degree-0 draws before the round limit: account them
                TRY(sr_post(c, &r->run, 0, 0));
                r->need_draw = true;
                continue;
            }
        }
        if (r->state == AXBC_REQ_RUNNING) ready.push_back(r);
    }
    // rounds that have waited longest first, so that no request starves
    std::stable_sort(ready.begin(), ready.end(),
                     [](const Request *a, const Request *b) { return a->drawn_at < b->drawn_at; });
    struct Seg {
        Request *r;
        int lane0, cnt;
    };
    std::vector<Seg> segs;
    int lane = 0;
    for (Request *r : ready) {
        const int cnt = std::min(sr_nb(&r->run) - r->off, r->want);
        if (lane + cnt > AXBC_WMAX) continue;  // its drawn round waits for the next pass
        segs.push_back({r, lane, cnt});
        lane += cnt;
    }
    if (segs.empty()) return AXBC_OK;
    for (auto &sg : segs) TRY(sr_load(c, &sg.r->run, sg.r->off, sg.lane0, sg.cnt));
    TRY(axbc_batch_traverse(c, lane, G.H));
    float *tg[AXBC_WMAX];
    for (int i = 0; i < AXBC_WMAX; i++) tg[i] = segs[0].r->run.bc;
    std::vector<float *> dout;
    std::vector<int> lo, hi;
    for (auto &sg : segs) {
        for (int l = sg.lane0; l < sg.lane0 + sg.cnt; l++) tg[l] = sg.r->run.bc;
        dout.push_back(sg.r->run.delta_last);
        lo.push_back(sg.lane0);
        hi.push_back(sg.lane0 + sg.cnt);
    }
    TRY(axbc_batch_set_targets(c, tg));
    for (auto &sg : segs) TRY(sr_post(c, &sg.r->run, sg.r->off, sg.lane0, sg.cnt));
    TRY(axbc_batch_apply_lanes(c, dout.data(), lo.data(), hi.data(), (int)segs.size()));
    for (auto &sg : segs) {
        Request *r = sg.r;
        r->run.batches++;
        r->off += sg.cnt;
        if (r->off >= sr_nb(&r->run)) {
            r->need_draw = true;
        } else {
            // the rest of the round goes on only if Bader's test holds off
            TRY(sr_stop_test(c, &r->run));
            r->test_pending = true;
            if (r->off > 1) r->want = std::min(2 * r->want, AXBC_WMAX);
        }
    }
    std::lock_guard<std::mutex> lk(S->mu);
    S->passes++;
    S->lanes += lane;
    G.lanes += lane;
    return AXBC_OK;
}

// The worker of graph gi: admits queued requests for its graph while the
// budget allows, then runs passes over them on the graph's own stream, so
// passes on different graphs overlap on the device.
static void serve_graph_loop(axbc_server *S, int gi)
{
    cudaSetDevice(S->device);
    ServeGraph *Gp;
    {
        std::lock_guard<std::mutex> lk(S->mu);
        Gp = S->graphs[gi].get();
    }
    ServeGraph &G = *Gp;
    for (;;) {
        std::vector<Request *> admit;
        {
            std::unique_lock<std::mutex> lk(S->mu);
            for (;;) {
                // admission in arrival order while the budget allows
                for (auto it = S->queue.begin(); it != S->queue.end();) {
                    Request *r = S->reqs[*it].get();
                    if (r->graph == gi && S->in_use + r->bytes <= S->budget) {
                        S->in_use += r->bytes;
                        r->state = AXBC_REQ_RUNNING;
                        r->t_start = now_ns();
                        r->worker_ref = true;
                        S->admitted++;
                        admit.push_back(r);
                        it = S->queue.erase(it);
                    } else {
                        ++it;
                    }
                }
                if (!admit.empty() || !G.active.empty()) break;
                if (S->stop) return;
                S->work_cv.wait(lk);
            }
        }
        for (Request *r : admit) {
            // static heuristics (-z 0..2) draw from distributions no pivot
            // changes, so without Bader's stop (whose round counter depends on
            // where a round ends) the width only sets how many pivots share a
            // pass: run them 64 wide (same pivots, bits and counters)
            axbc_run_params prm = r->prm;
            if (prm.z <= 2 && prm.bader_c == 0) prm.batch_width = AXBC_SERVE_STATIC_WIDTH;
            int st = sr_alloc(G.g, &prm, &r->run);
            if (st == AXBC_OK) {
                r->allocated = true;
                st = sr_begin(G.ctx, &r->run);
            }
            if (st != AXBC_OK) {
                if (r->allocated) sr_free(&r->run);
                r->allocated = false;
                {
                    std::lock_guard<std::mutex> lk(S->mu);
                    S->in_use -= r->bytes;
                }
                req_fail(S, r, st);
            }
            r->need_draw = true;
            G.active.push_back(r);
        }
        const uint64_t t0 = now_ns();
        uint64_t lanes0;
        {
            std::lock_guard<std::mutex> lk(S->mu);
            lanes0 = G.lanes;
        }
        std::vector<Request *> runs;
        for (Request *r : G.active)
            if (r->state == AXBC_REQ_RUNNING) runs.push_back(r);
        const int st = runs.empty() ? AXBC_OK : serve_pass(S, G, runs);
        {
            std::lock_guard<std::mutex> lk(S->mu);
            G.busy_ns += now_ns() - t0;
            if (G.lanes != lanes0) G.passes++;
        }
        if (st != AXBC_OK) {
            // a failed pass fails the requests that were in it
            for (Request *r : runs) {
                if (r->state != AXBC_REQ_RUNNING) continue;
                if (r->allocated) sr_free(&r->run);
                r->allocated = false;
                {
                    std::lock_guard<std::mutex> lk(S->mu);
                    S->in_use -= r->bytes;
                }
                req_fail(S, r, st);
            }
        }
        std::lock_guard<std::mutex> lk(S->mu);
        std::vector<Request *> keep;
        for (Request *r : G.active) {
            if (r->state == AXBC_REQ_RUNNING) {
                keep.push_back(r);
                continue;
            }
            r->worker_ref = false;
            if (r->released) S->reqs.erase(r->id);
        }
        G.active.swap(keep);
        // room freed: the other graphs' workers may admit now
        S->work_cv.notify_all();
    }
}

extern "C" int axbc_server_create(uint64_t hbm_budget, axbc_server **out)
{
    CHECK_ARG(out, "axbc_server_create: null argument");
    auto S = std::make_unique<axbc_server>();
    CU(cudaGetDevice(&S->device));
    if (hbm_budget == 0) {
        size_t fr = 0, tot = 0;
        CU(cudaMemGetInfo(&fr, &tot));
        hbm_budget = (uint64_t)(fr * 0.8);
    }
    S->budget = hbm_budget;
    *out = S.release();
    return AXBC_OK;
}

extern "C" int axbc_server_add_graph(axbc_server *S, axbc_graph *g, int H, int *graph_id)
{
    CHECK_ARG(S && g && graph_id, "axbc_server_add_graph: null argument");
    CHECK_ARG(H == 0 || H == 1, "axbc_server_add_graph: H must be 0 or 1");
    auto G = std::make_unique<ServeGraph>();
    G->g = g;
    G->H = H;
    CU(cudaStreamCreateWithFlags(&G->stream, cudaStreamNonBlocking));
    int st = axbc_ctx_create(g, G->stream, &G->ctx);
    if (st == AXBC_OK) st = axbc_ensure_batch(G->ctx);
    // the static sampling distributions (degrees, LCC) of the resident graph
    // are built now, not by the first request that needs them: their
    // triangle count can hold the device for a while on a large graph
    if (st == AXBC_OK) st = axbc_build_deg_dist(g, G->stream);
    if (st == AXBC_OK) st = axbc_build_lcc(g, G->stream);
    if (st == AXBC_OK && cudaStreamSynchronize(G->stream) != cudaSuccess)
        st = axbc_cuda_fail(cudaGetLastError(), "server graph set-up", __FILE__, __LINE__);
    if (st != AXBC_OK) {
        if (G->ctx) axbc_ctx_destroy(G->ctx);
        cudaStreamDestroy(G->stream);
        return st;
    }
    std::lock_guard<std::mutex> lk(S->mu);
    S->graphs.push_back(std::move(G));
    const int gi = (int)S->graphs.size() - 1;
    S->graphs[gi]->worker = std::thread(serve_graph_loop, S, gi);
    *graph_id = gi;
    return AXBC_OK;
}

extern "C" int axbc_request_submit(axbc_server *S, int graph_id, const axbc_run_params *prm,
                                   uint64_t *request_id)
{
    CHECK_ARG(S && prm && request_id, "axbc_request_submit: null argument");
    ServeGraph *Gp = nullptr;
    {
        std::lock_guard<std::mutex> lk(S->mu);
        CHECK_ARG(graph_id >= 0 && graph_id < (int)S->graphs.size(), "axbc_request_submit: no such graph");
        Gp = S->graphs[graph_id].get();
    }
    const ServeGraph &G = *Gp;
    TRY(sr_check_params(G.g, prm, AXBC_WMAX));
    CHECK_ARG(prm->H == G.H, "axbc_request_submit: H differs from the graph's");
    auto r = std::make_unique<Request>();
    r->graph = graph_id;
    r->G = Gp;
    r->prm = *prm;
    r->bytes = sr_bytes(G.g->n, prm);
    r->t_submit = now_ns();
    std::lock_guard<std::mutex> lk(S->mu);
    if (r->bytes > S->budget) {
        axbc_set_error("axbc_request_submit: the request needs %llu device bytes, the budget is %llu",
                       (unsigned long long)r->bytes, (unsigned long long)S->budget);
        return AXBC_ERR_BUSY;
    }
    r->id = S->next_id++;
    *request_id = r->id;
    S->queue.push_back(r->id);
    S->reqs[r->id] = std::move(r);
    S->work_cv.notify_all();
    return AXBC_OK;
}

static void fill_info(const Request *r, axbc_request_info *info)
{
    memset(info, 0, sizeof(*info));
    info->state = r->state;
    info->status = r->status;
    info->result = r->res;
    info->bytes = r->bytes;
    info->submit_ns = r->t_submit;
    info->start_ns = r->t_start;
    info->finish_ns = r->t_finish;
    snprintf(info->error, sizeof(info->error), "%s", r->err.c_str());
}

extern "C" int axbc_request_poll(axbc_server *S, uint64_t id, axbc_request_info *info)
{
    CHECK_ARG(S && info, "axbc_request_poll: null argument");
    std::lock_guard<std::mutex> lk(S->mu);
    auto it = S->reqs.find(id);
    CHECK_ARG(it != S->reqs.end(), "axbc_request_poll: no such request");
    fill_info(it->second.get(), info);
    return AXBC_OK;
}

extern "C" int axbc_request_wait(axbc_server *S, uint64_t id, int64_t timeout_ms,
                                 axbc_request_info *info)
{
    CHECK_ARG(S, "axbc_request_wait: null argument");
    std::unique_lock<std::mutex> lk(S->mu);
    auto it = S->reqs.find(id);
    CHECK_ARG(it != S->reqs.end(), "axbc_request_wait: no such request");
    Request *r = it->second.get();
    auto done = [r] { return r->state == AXBC_REQ_DONE || r->state == AXBC_REQ_FAILED; };
    if (timeout_ms < 0) {
        S->done_cv.wait(lk, done);
    } else if (!S->done_cv.wait_for(lk, std::chrono::milliseconds(timeout_ms), done)) {
        if (info) fill_info(r, info);
        axbc_set_error("axbc_request_wait: request %llu not finished after %lld ms",
                       (unsigned long long)id, (long long)timeout_ms);
        return AXBC_ERR_TIMEOUT;
    }
    if (info) fill_info(r, info);
    return AXBC_OK;
}

extern "C" int axbc_request_result(axbc_server *S, uint64_t id, float *bc_host, uint32_t *pivots,
                                   double *probs, uint64_t cap, uint64_t *count)
{
    CHECK_ARG(S, "axbc_request_result: null argument");
    std::lock_guard<std::mutex> lk(S->mu);
    auto it = S->reqs.find(id);
    CHECK_ARG(it != S->reqs.end(), "axbc_request_result: no such request");
    const Request *r = it->second.get();
    if (r->state != AXBC_REQ_DONE) {
        axbc_set_error("axbc_request_result: request %llu is not done", (unsigned long long)id);
        return AXBC_ERR_STATE;
    }
    if (bc_host) memcpy(bc_host, r->bc.data(), r->bc.size() * 4);
    const uint64_t k = std::min<uint64_t>(cap, r->pivots.size());
    if (pivots) memcpy(pivots, r->pivots.data(), k * 4);
    if (probs) memcpy(probs, r->probs.data(), k * 8);
    if (count) *count = r->pivots.size();
    return AXBC_OK;
}

extern "C" int axbc_request_release(axbc_server *S, uint64_t id)
{
    CHECK_ARG(S, "axbc_request_release: null argument");
    std::lock_guard<std::mutex> lk(S->mu);
    auto it = S->reqs.find(id);
    CHECK_ARG(it != S->reqs.end(), "axbc_request_release: no such request");
    Request *r = it->second.get();
    if (r->state == AXBC_REQ_QUEUED) {
        S->queue.erase(std::find(S->queue.begin(), S->queue.end(), id));
    } else if (r->state == AXBC_REQ_RUNNING) {
        axbc_set_error("axbc_request_release: request %llu is running", (unsigned long long)id);
        return AXBC_ERR_STATE;
    }
    if (r->worker_ref) {
        r->released = true;  // the worker forgets it when it lets go
        return AXBC_OK;
    }
    S->reqs.erase(it);
    return AXBC_OK;
}

extern "C" int axbc_server_stats(axbc_server *S, axbc_server_stats_t *st)
{
    CHECK_ARG(S && st, "axbc_server_stats: null argument");
    std::lock_guard<std::mutex> lk(S->mu);
    memset(st, 0, sizeof(*st));
    st->budget = S->budget;
    st->in_use = S->in_use;
    st->queued = S->queue.size();
    st->admitted = S->admitted;
    st->completed = S->completed;
    st->passes = S->passes;
    st->lanes = S->lanes;
    return AXBC_OK;
}

extern "C" int axbc_server_graph_stats(axbc_server *S, int graph_id, uint64_t *passes, uint64_t *lanes,
                                       uint64_t *busy_ns)
{
    CHECK_ARG(S, "axbc_server_graph_stats: null argument");
    std::lock_guard<std::mutex> lk(S->mu);
    CHECK_ARG(graph_id >= 0 && graph_id < (int)S->graphs.size(), "axbc_server_graph_stats: no such graph");
    const ServeGraph &G = *S->graphs[graph_id];  // under the mutex
    if (passes) *passes = G.passes;
    if (lanes) *lanes = G.lanes;
    if (busy_ns) *busy_ns = G.busy_ns;
    return AXBC_OK;
}

extern "C" int axbc_server_destroy(axbc_server *S)
{
    if (!S) return AXBC_OK;
    {
        std::lock_guard<std::mutex> lk(S->mu);
        S->stop = true;
        S->queue.clear();  // queued requests are dropped; admitted ones finish
        S->work_cv.notify_all();
    }
    for (auto &G : S->graphs)
        if (G->worker.joinable()) G->worker.join();
    for (auto &kv : S->reqs)
        if (kv.second->allocated) sr_free(&kv.second->run);
    for (auto &G : S->graphs) {
        axbc_ctx_destroy(G->ctx);
        cudaStreamDestroy(G->stream);
    }
    delete S;
    return AXBC_OK;
}
