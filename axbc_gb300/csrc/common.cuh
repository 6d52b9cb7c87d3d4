// Internal declarations shared by the axbc_gb300 CUDA sources.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <string>
#include <vector>

#include "../../include/axbc.h"

// ---------------------------------------------------------------- constants
// Canonical accumulation order of one vertex's dependency sum (identical in
// the plain and the batched kernels): successor terms in adjacency order,
// CHUNK positions summed as a balanced binary tree, chunk sums added left to
// right inside SPAN positions, span sums added left to right onto reach[v].
// Vertices with more than SPAN neighbours are "heavy": their spans are
// separate work items whose partial sums are combined in span order.
#define AXBC_CHUNK 32
#define AXBC_SPAN 1024
#define AXBC_SAMPLE_BLOCK 1024
#define AXBC_W 32     // lanes of a warp, pivots per mask word
#define AXBC_WMAX 64  // pivots of one multi-source pass (two mask words per vertex)
#define FULL_MASK 0xffffffffu

// ---------------------------------------------------------------- errors
void axbc_set_error(const char *fmt, ...);
int axbc_cuda_fail(cudaError_t e, const char *what, const char *file, int line);

#define CU(call)                                                                  \
    do {                                                                          \
        cudaError_t _e = (call);                                                  \
        if (_e != cudaSuccess) return axbc_cuda_fail(_e, #call, __FILE__, __LINE__); \
    } while (0)

#define CU_LAUNCH(what)                                                           \
    do {                                                                          \
        cudaError_t _e = cudaGetLastError();                                      \
        if (_e != cudaSuccess) return axbc_cuda_fail(_e, what, __FILE__, __LINE__); \
    } while (0)

#define CHECK_ARG(cond, msg)                                                      \
    do {                                                                          \
        if (!(cond)) {                                                            \
            axbc_set_error("%s", msg);                                            \
            return AXBC_ERR_INVALID;                                              \
        }                                                                         \
    } while (0)

#define TRY(call)                                                                 \
    do {                                                                          \
        int _rc = (call);                                                         \
        if (_rc != AXBC_OK) return _rc;                                           \
    } while (0)

// ---------------------------------------------------------------- graph
// One direction of adjacency on the device.  `fwd` is the reference's CSC
// (column c lists the r of edges (r,c)); `rev` is its transpose, used when a
// forward level pulls into unvisited vertices.  For a symmetric graph rev
// aliases fwd.
struct Adj {
    uint64_t n = 0, m = 0;
    uint32_t *col = nullptr;  // n+1
    uint32_t *row = nullptr;  // m
    // heavy vertices (degree > SPAN): one work item per span
    uint32_t n_heavy = 0;
    uint64_t n_heavy_items = 0;
    uint32_t *heavy_v = nullptr;      // n_heavy vertex ids
    uint32_t *heavy_first = nullptr;  // n_heavy first item index
    uint32_t *hitem_v = nullptr;      // n_heavy_items
    uint32_t *hitem_k = nullptr;      // span index of the item
    // vertices by degree, descending (heavy ones first), and the light-vertex
    // tasks: order[ltask[i] .. ltask[i+1]) holds at most 32 vertices whose
    // degrees sum to about one span; dynamic kernels take heavy span items
    // first, then these tasks, so the largest work is handed out first
    uint32_t *order = nullptr;        // n
    uint32_t *ltask = nullptr;        // n_ltask + 1 offsets into order
    uint64_t n_ltask = 0;
    bool owns = true;
};

struct axbc_graph {
    int device = 0;
    uint64_t n = 0, m = 0;
    int symmetric = 1;
    Adj fwd, rev;
    uint32_t *reach = nullptr;  // n
    // The batched passes' view of the graph.  On graphs with a vertex of more
    // than AXBC_RENUMBER_MIN_DEG neighbours the vertices are renumbered by
    // descending degree (ties by id), so that the hubs' level-mask words and
    // per-pivot rows share sectors and lines; every adjacency list keeps its
    // own order (the canonical dependency sums run over the same positions).
    // Otherwise the view is the graph itself (aliases, null maps).
    bool renumbered = false;
    Adj bfwd, brev;
    uint32_t *breach = nullptr;     // reach in view numbering
    uint32_t *to_view = nullptr;    // n: view id of each vertex (null: identity)
    uint32_t *from_view = nullptr;  // n: vertex of each view id (null: identity)
    uint64_t bytes = 0;
    uint32_t max_deg = 0;
    // static pivot distributions, built on first use
    bool have_deg_dist = false;
    uint32_t *deg2p = nullptr;    // uint32 prefix of (uint32)deg^2 (wraps)
    uint32_t *sdn = nullptr;      // neighbour degree sums
    uint32_t *seg_end = nullptr;  // ends of the non-decreasing runs of deg2p
    uint32_t n_seg = 0;
    uint32_t sum_deg = 0;
    bool have_lcc = false;
    float *lcc = nullptr;
    double *lcc_local = nullptr;
    double *lcc_csum = nullptr;
    double S_lcc = 0;
};

// graph helpers (graph.cu)
int axbc_graph_build_device(axbc_graph *g, const uint32_t *d_col, const uint32_t *d_row,
                            const uint32_t *d_reach, cudaStream_t s);
int axbc_build_deg_dist(axbc_graph *g, cudaStream_t s);
int axbc_build_lcc(axbc_graph *g, cudaStream_t s);
// hierarchical prefix of n float weights (sampler.cu)
int axbc_hprefix_launch(const float *w, uint64_t n, double *local, double *csum, cudaStream_t s);

// ---------------------------------------------------------------- context
struct PivotCounters {  // device, single-source
    uint32_t qtail;
    uint32_t pad;
    unsigned long long newdeg;  // degree sum of vertices discovered this level
    unsigned long long reach_sum;
    unsigned long long visited_rdeg;  // in-degree sum of visited vertices
};

struct BatchInfo {  // device, one multi-source batch of up to AXBC_WMAX pivots
    uint32_t nsrc;
    uint32_t pad0;
    unsigned long long applymask;   // sources whose update is applied (Bader replay)
    unsigned long long srcmask;
    unsigned long long depth0mask;  // sources whose BFS ended at level 2
    uint32_t root[AXBC_WMAX];
    double p[AXBC_WMAX];
    // per-source totals accumulated by the level-stats kernel
    unsigned long long nvis[AXBC_WMAX];
    unsigned long long rsum[AXBC_WMAX];
    unsigned long long te[AXBC_WMAX];
    // per-level scratch read back by the host
    unsigned long long lvl_new[AXBC_WMAX];
    unsigned long long front_deg;
    unsigned long long unvis_deg;   // in-degree sum of vertices some pivot has not seen
    unsigned long long unvis_dec;   // this level's decrease of unvis_deg
    unsigned long long lvl_te;  // degree sum over the level's new (vertex, pivot) pairs
    uint32_t any_new;
    uint32_t task_ctr[4];
    int32_t H;
    // device-driven level loop: the step kernels read their level and
    // direction here, the advance kernels move them on
    int32_t cur;        // last completed forward level
    int32_t alive;      // 1 while the last completed level discovered vertices
    int32_t lend;       // first level that discovered nothing (once alive == 0)
    int32_t dmax;       // deepest depth = lend - 1
    int32_t bd;         // next backward depth (counts down to -1)
    int32_t push_next;  // 1: the next forward level pushes from the frontier
    double push_factor;
    unsigned long long push_min;  // frontier degree sums below this always push
    int32_t Ls[AXBC_WMAX];  // per pivot: first level that discovered nothing
    int32_t pool_short;  // a level's list was capped by the pool's size
    int32_t pad_;
    float *lane_bc[AXBC_WMAX];  // per pivot: the bc vector its update goes to
};

// the bc vector of each lane, for a pass whose lanes belong to several runs
struct LaneTargets {
    float *bc[AXBC_WMAX];
};

// capacity of the per-level tables of a context (levels of one traversal)
#define AXBC_MAX_LEVELS (1 << 16)

struct SamplerState;  // sampler.cu

// Grid barrier of a cooperative launch (batch.cu): arrival count, generation,
// and the failure record of a wait that ran out of its budget.
struct GridSync {
    unsigned int count;
    unsigned int gen;
    int err;   // nonzero: the site of the barrier whose wait ran out
    int need;  // the persistent forward loop reached the levels allocated
};
// batches of at most AXBC_PERSIST_AUTO_WIDTH pivots on graphs whose last batch
// was deeper than AXBC_PERSIST_AUTO_LEVELS run their levels in one persistent
// launch
// graphs whose largest degree exceeds this are renumbered for the batched
// passes (meshes and road-like graphs keep their own, already local, order)
#ifndef AXBC_RENUMBER_MIN_DEG
#define AXBC_RENUMBER_MIN_DEG 64
#endif
#ifndef AXBC_PERSIST_AUTO_LEVELS
#define AXBC_PERSIST_AUTO_LEVELS 64
#endif
#ifndef AXBC_PERSIST_AUTO_WIDTH
#define AXBC_PERSIST_AUTO_WIDTH 8
#endif

// Kernel kinds timed by the profiling hooks (axbc_ctx_profile).
enum {
    KP_FWD_PUSH = 0,   // batched forward, push
    KP_FWD_PULL,       // batched forward, pull
    KP_LEVEL_STATS,    // batched level bookkeeping
    KP_BWD,            // batched backward
    KP_BWD_COMBINE,    // batched heavy-vertex combine
    KP_UPDATE,         // batched bc update + delta extraction
    KP_SAMPLER,        // sampler, Bader replay, prefix sums
    KP_PLAIN_FWD,      // plain forward level
    KP_PLAIN_BWD,      // plain backward level (+ combine)
    KP_PLAIN_OTHER,    // plain reset / root / reach sum / update
    KP_PERSIST,        // batched traversal as one persistent cooperative launch
    KP_NKINDS
};

struct ProfRec {
    int kind;
    double bytes;  // algorithmic bytes of the launch
    cudaEvent_t a, b;
    int tag;       // forward level of a device-driven step (-1: none)
};

struct axbc_ctx {
    axbc_graph *g = nullptr;
    cudaStream_t stream = nullptr;
    bool own_stream = false;
    // lazily allocated state is complete (a failed allocation leaves it false,
    // and the next call allocates what is still missing)
    bool single_ready = false, batch_ready = false, tables_ready = false, sampler_ready = false;
    size_t fmtab_synced = 0;  // level-mask pointers copied into the device table
    float *bc = nullptr;
    float *delta_last = nullptr;
    bool delta_last_valid = false;
    // plain single-source state
    int32_t *lvl = nullptr;
    uint32_t *sigma = nullptr;
    float *delta = nullptr;
    uint32_t *queue = nullptr;
    float *partial = nullptr;  // heavy span partials (fwd heavy items)
    PivotCounters *pc = nullptr;
    PivotCounters *pc_host = nullptr;  // pinned
    std::vector<uint64_t> levstart;
    uint64_t s_front_deg = 0, s_prev_newdeg = 0, s_visited_rdeg = 0;  // direction choice
    // multi-source batch state
    uint32_t *seen = nullptr;
    std::vector<uint32_t *> fmask;  // one n-word mask array per level
    uint32_t *msigma = nullptr;     // n*32
    float *mdelta = nullptr;        // n*32
    float *mq = nullptr;            // n*32: (delta + 1) / sigma, per pivot
    uint32_t *task_ctr = nullptr;   // work counters of the dynamic kernels
    float *mpartial = nullptr;      // heavy items * 32
    BatchInfo *bi = nullptr;
    BatchInfo *bi_host = nullptr;  // pinned
    uint32_t **fmtab = nullptr;               // device copy of the fmask pointers
    uint32_t *ctrs = nullptr;                 // per-level work counters (2 per level)
    unsigned long long *d_level_te = nullptr;   // per level: degree sum of new pairs
    unsigned long long *d_level_cnt = nullptr;  // per level: new (vertex, pivot) pairs
    int32_t *d_level_mode = nullptr;            // per level: 1 push, 0 pull
    uint32_t *lpool = nullptr;                  // per-level vertex lists
    uint32_t *lstart = nullptr, *lcount = nullptr, *lcap = nullptr, *lheavy = nullptr;
    uint32_t lpool_cap = 0;
    bool pool_short = false;  // the last batch ran out of list space
    int prev_lend = 0;        // levels of the last batch whose masks need clearing
    // captured forward / backward level steps, per width (index K - 1)
    cudaGraphExec_t fwd_step_exec[2] = {nullptr, nullptr};
    cudaGraphExec_t bwd_step_exec[2] = {nullptr, nullptr};
    int last_batch_levels = 0;
    int last_batch_nsrc = 0;
    int last_batch_k = 1;  // mask words per vertex of the last batch (1: <= 32 pivots, 2: <= 64)
    int last_Ls[AXBC_WMAX] = {0};  // first empty level of each pivot of the last batch
    // the last batch's per-pivot level counts and list-pool flag are read back
    // without waiting; rb_ev marks their arrival (axbc_batch_settle)
    cudaEvent_t rb_ev = nullptr;
    bool rb_pending = false;
    // sampler
    SamplerState *ss = nullptr;
    SamplerState *ss_host = nullptr;  // pinned
    uint8_t *used = nullptr;          // n: pivot already drawn
    uint32_t *checks = nullptr;
    float *checkval = nullptr;  // Bader replay scratch, one per check vertex
    uint32_t nchecks_cap = 0;
    double *dyn_local = nullptr;
    double *dyn_csum = nullptr;
    double *dyn_local2 = nullptr;
    double *dyn_csum2 = nullptr;
    float *wtmp = nullptr;
    std::vector<uint32_t> run_pivots;
    std::vector<double> run_probs;
    std::vector<uint32_t> run_checks;
    // profiling: launch count always, event pairs when prof_on
    uint64_t launches = 0;
    bool prof_on = false;
    std::vector<ProfRec> prof;
    // work counting: the traversal kernels' counting builds run instead of the
    // captured level steps, accumulating into wcount[kind][field]
    bool count_on = false;
    unsigned long long *wcount = nullptr;  // KP_NKINDS * WC_NFIELDS
    // persistent level loop: -1 never, 0 when the last batch was deeper than
    // AXBC_PERSIST_AUTO_LEVELS, 1 always; blocks per SM of its cooperative grid
    int persist_mode = 0;
    int persist_blocks_per_sm = 4;
    struct GridSync *gsync = nullptr;  // its barrier state (device)
    std::vector<cudaEvent_t> ev_pool;
    double level_te_prev = 0;  // degree sum of the previous level's new vertices
    std::vector<double> level_te;
    // tuning
    double push_factor_single = 8.0;  // defaults: see axbc_ctx_set_tuning
    double push_factor_batch = 8.0;
    uint64_t bytes = 0;
    int num_sms = 0;
    // resident blocks per SM, per width (index K - 1)
    int dyn_blocks_per_sm[2] = {0, 0};   // forward push
    int upd_blocks_per_sm[2] = {0, 0};   // batched bc update
    int pull_blocks_per_sm[2] = {0, 0};  // forward pull
    int bwd_blocks_per_sm[2] = {0, 0};   // backward
};

// graph.cu: sort adjacency keys ((column << 32) | row, all-ones = none), drop
// duplicates and self-loops (norm_graph), optionally reduce degree-1
// vertices, and build the graph; kron.cu: the Graph500 generator's edges on the
// device as (source << 32 | target), stage 0 split, 1 permuted, 2 scrambled
int axbc_keys_to_graph(uint64_t *d_keys, uint64_t nk, uint64_t n, int symmetric, int H, axbc_graph **out);
int axbc_kron_device(int scale, int edgefactor, uint64_t seed1, uint64_t seed2, const double *initiator,
                     int stage, uint64_t **d_edges, uint64_t *m_out);

// allocation with byte accounting
int axbc_dalloc(void **p, size_t bytes, uint64_t *acct);
void axbc_dfree(void *p);

// allocate a lazily created member unless an earlier, partly failed call did
#define ALLOC_MISSING(ptr, bytes, acct)                                               \
    do {                                                                              \
        if (!(ptr)) TRY(axbc_dalloc((void **)&(ptr), (bytes), (acct)));               \
    } while (0)

// a scratch device buffer freed when it goes out of scope (error paths included)
struct DBuf {
    void *p = nullptr;
    DBuf() = default;
    DBuf(const DBuf &) = delete;
    DBuf &operator=(const DBuf &) = delete;
    ~DBuf() { axbc_dfree(p); }
    int alloc(size_t bytes) { return axbc_dalloc(&p, bytes, nullptr); }
    void release()
    {
        axbc_dfree(p);
        p = nullptr;
    }
    template <class T> T *as() const { return (T *)p; }
};

// single.cu / batch.cu
int axbc_ensure_single(axbc_ctx *c);
int axbc_single_reset(axbc_ctx *c);
int axbc_single_set_root(axbc_ctx *c, uint32_t v0, int level, uint32_t sig);
int axbc_single_forward_level(axbc_ctx *c, uint32_t qs, uint32_t nf, int level, uint64_t *nfrt);
int axbc_single_backward_level(axbc_ctx *c, uint32_t ls, uint32_t nseg, int d);
int axbc_single_reach_sum(axbc_ctx *c);
int axbc_single_update(axbc_ctx *c, uint32_t v0, double p, const uint32_t *reach_v0_dev,
                       uint64_t nvt_base, int add_all, int add_sum);
int axbc_ensure_batch(axbc_ctx *c);
int axbc_batch_traverse(axbc_ctx *c, int nsrc, int H);
int axbc_batch_settle(axbc_ctx *c);
int axbc_batch_apply(axbc_ctx *c);
int axbc_batch_apply_lanes(axbc_ctx *c, float *const *delta_out, const int *lane_lo,
                           const int *lane_hi, int nseg);
int axbc_batch_set_targets(axbc_ctx *c, float *const *bc_of_lane);
int axbc_batch_levels_alloc(axbc_ctx *c, int levels);

// grid sizing
int axbc_grid_for(const axbc_ctx *c, int threads_per_block, int blocks_per_sm);

// profiling hooks around one kernel launch on c->stream
void axbc_prof_start(axbc_ctx *c, int kind, double bytes);
void axbc_prof_stop(axbc_ctx *c);
struct ProfScope {
    axbc_ctx *c;
    ProfScope(axbc_ctx *cc, int kind, double bytes) : c(cc) { axbc_prof_start(c, kind, bytes); }
    ~ProfScope() { axbc_prof_stop(c); }
};

// ---------------------------------------------------------------- device helpers
__device__ __forceinline__ unsigned lane_id() { return threadIdx.x & 31u; }

// Work counts of the traversal kernels, kept only in their counting builds
// (axbc_ctx_count): per launch kind the bytes the launch has to move at least
// (each 4-byte word it must read or write once, sectors not counted),
// adjacency entries scanned, (edge, pivot) gathers and (vertex, pivot) results
// written.  The plain builds carry an empty counter that compiles away.
enum { WC_BYTES = 0, WC_ENTRIES, WC_GATHERS, WC_PAIRS, WC_NFIELDS };
template <bool ON> struct WorkCount {
    __device__ __forceinline__ void add(int, unsigned long long) {}
    __device__ __forceinline__ void flush(unsigned long long *) {}
};
template <> struct WorkCount<true> {
    unsigned long long f[WC_NFIELDS] = {0, 0, 0, 0};
    __device__ __forceinline__ void add(int i, unsigned long long x) { f[i] += x; }
    // every lane of the warp calls this once, at the end of the kernel
    __device__ __forceinline__ void flush(unsigned long long *w)
    {
#pragma unroll
        for (int i = 0; i < WC_NFIELDS; i++) {
            unsigned long long x = f[i];
            for (int o = 16; o; o >>= 1) x += __shfl_xor_sync(0xffffffffu, x, o);
            if (lane_id() == 0 && x) atomicAdd(&w[i], x);
        }
    }
};

// One successor's share of a dependency, in the reference's operation order
// (scan_frt_mono: (delta[r] + 1) / sigma[r] * sigma[c]), rounded op by op.
__device__ __forceinline__ float dep_term(float delta_r, uint32_t sigma_r, float sigma_c)
{
    return __fmul_rn(__fdiv_rn(__fadd_rn(delta_r, 1.0f), __uint2float_rn(sigma_r)), sigma_c);
}

// Balanced binary tree over the 32 lanes (pairs differing in bit 0 first).
__device__ __forceinline__ float warp_tree_sum(float v)
{
#pragma unroll
    for (int w = 1; w < 32; w <<= 1) v = __fadd_rn(v, __shfl_xor_sync(FULL_MASK, v, w));
    return v;
}

// The bc increment of one pivot for a non-root vertex (update_bc,
// src/cuda_kernels.cu:284): float(double(delta * (float)(reach_v0 + 1)) / p).
__device__ __forceinline__ float bc_term(float delta_v, uint32_t reach_v0, double p)
{
    return __double2float_rn(__ddiv_rn((double)__fmul_rn(delta_v, __uint2float_rn(reach_v0 + 1u)), p));
}
// float(double(x) / p) for x >= 0 without the double divide in the common
// case.  With 1/p split into float hi + lo (1/p computed once per pivot), x*hi
// is formed exactly as a + e by Dekker's two-product (an FMA gives e), then
// b = x*lo + e, so a + b approximates x/p to about 2^-46 relative.  s =
// RN_float(a + b) equals the correctly rounded result unless x/p lies near the
// midpoint between two floats; Knuth's TwoSum gives the exact residual of
// s, and if it is within 2^-40 (relative) of half an ulp -- or s is a power of
// two, tiny, huge or not finite -- the exact double divide decides.
struct InvSplit {
    float hi, lo;
    int ok;  // 1: fast path usable for this p
};
__host__ __device__ __forceinline__ InvSplit inv_split(double p)
{
    InvSplit r{0.0f, 0.0f, 0};
    if (!(p > 0.0) || p > 1e30 || p < 1e-30) return r;
    const double inv = 1.0 / p;
    r.hi = (float)inv;
    r.lo = (float)(inv - (double)r.hi);
    r.ok = 1;
    return r;
}
__device__ __forceinline__ float div_to_float_hl(float x, double p, float hi, float lo, bool ok)
{
    if (ok && x > 0.0f && x < 3.0e38f) {
        const float a = __fmul_rn(x, hi);
        const float e = __fmaf_rn(x, hi, -a);
        const float b = __fmaf_rn(x, lo, e);
        const float s = __fadd_rn(a, b);
        const float bb = __fsub_rn(s, a);
        const float err = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
        const uint32_t bits = __float_as_uint(s);
        const uint32_t ex = (bits >> 23) & 0xffu;
        if (ex >= 40u && ex <= 210u) {
            // the rounding boundary on err's side: half an ulp of s, or a
            // quarter below a power of two (the spacing halves there)
            const uint32_t sh = ((bits & 0x7fffffu) == 0u && err < 0.0f) ? 25u : 24u;
            const float tie = __uint_as_float((ex - sh) << 23);
            const float dist = fabsf(__fsub_rn(fabsf(err), tie));
            if (dist > __fmul_rn(s, 9.094947e-13f /* 2^-40 */)) return s;
        }
    }
    return __double2float_rn(__ddiv_rn((double)x, p));
}
__device__ __forceinline__ float div_to_float(float x, double p, InvSplit iv)
{
    return div_to_float_hl(x, p, iv.hi, iv.lo, iv.ok != 0);
}
__device__ __forceinline__ float bc_term_fast(float delta_v, uint32_t reach_v0, double p, InvSplit iv)
{
    return div_to_float(__fmul_rn(delta_v, __uint2float_rn(reach_v0 + 1u)), p, iv);
}

// The root's increment (:277): reach_v0 * (nvisited - 2) converted to float.
__device__ __forceinline__ float bc_root_term(uint32_t reach_v0, unsigned long long nvis_total)
{
    return __ull2float_rn((unsigned long long)reach_v0 * (nvis_total - 2ull));
}
