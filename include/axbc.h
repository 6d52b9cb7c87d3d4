/*
 * axbc_gb300 -- GB300-native sampled-Brandes betweenness centrality.
 *
 * C ABI of libaxbc_gb300.so.  Plain pointers and sizes only; every call
 * returns an axbc status (0 = AXBC_OK) and never exits the process.  Host
 * buffers belong to the caller, device buffers to the library.  A graph and
 * the contexts built on it live on the CUDA device that was current when the
 * graph was created.  Calls on different contexts may come from different
 * host threads; calls on one context must be serialised by the caller.
 *
 * Reference: fvella/axbc, whose host driver (src/axbc2d.c) calls its CUDA
 * file (src/cuda_kernels.cu) through the extern "C" table of src/bc2d.h:
 * 136-190.  Each entry point below names the reference interface it replaces.
 * The reference's own names and signatures are also exported, unchanged, by
 * the compatibility layer declared in axbc_compat.h.
 */
#ifndef AXBC_H
#define AXBC_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

enum {
    AXBC_OK = 0,
    AXBC_ERR_INVALID = 1,    /* bad argument (null pointer, vertex >= n, ...) */
    AXBC_ERR_CUDA = 2,       /* a CUDA runtime call failed */
    AXBC_ERR_NOMEM = 3,      /* device or host allocation failed */
    AXBC_ERR_TIMEOUT = 4,    /* a bounded device-side wait gave up */
    AXBC_ERR_RANGE = 5,      /* a size exceeds a documented limit */
    AXBC_ERR_STATE = 6,      /* call out of order (e.g. no batch pending) */
    AXBC_ERR_BUSY = 7        /* serving: admission refused for lack of memory */
};

/* Pivots of one multi-source pass: a 32-bit mask per vertex per level up to
 * 32 pivots, a 64-bit mask up to 64 (a warp lane owns two pivots). */
#define AXBC_MAX_BATCH 64
/* largest sampling width of a sampled run: a round draws up to 64 pivots from
 * one snapshot and traverses them as one pass */
#define AXBC_MAX_WIDTH 64

typedef struct axbc_graph axbc_graph;
typedef struct axbc_ctx axbc_ctx;

const char *axbc_status_str(int status);
/* Text of the last error raised on the calling host thread. */
const char *axbc_last_error(void);
/* Library version string. */
const char *axbc_version(void);

/* ---------------------------------------------------------------- graphs */

/* Edge list (pairs of uint64 vertex ids < n) -> the reference's CSC, on the
 * host: mirror if `undirected`, then norm_graph, degree_reduction when H == 1,
 * norm_graph, build_csc.  Replaces read_graph/gen_graph's post-processing in
 * src/axbc2d.c:333-351, 695-907, 2551-2622.  The returned arrays are
 * allocated by the library; release them with axbc_host_free.
 * *col: n+1 offsets; *row: *m neighbour ids; *reach: n removed-leaf counts. */
int axbc_edges_to_csc(const uint64_t *edges, uint64_t nedges, uint64_t n, int undirected,
                      int H, uint32_t **col, uint32_t **row, uint64_t *m, uint32_t **reach,
                      uint64_t *removed_leaves);
void axbc_host_free(void *p);

/* Read an edge-list text file the way read_graph (src/axbc2d.c:356-445)
 * does: '#' lines are comments, other lines "u v".  Returns the edges (uint64
 * pairs, library-allocated) without mirroring. */
int axbc_read_edge_file(const char *path, uint64_t n, uint64_t **edges, uint64_t *nedges);

/* Upload a CSC graph (reference layout: column c lists the rows r of the
 * edges (r,c), ascending) to the current device.  `reach` may be NULL (all
 * zero).  Replaces initcuda + init_bc_1degree_device (src/cuda_kernels.cu:
 * 1558-1600, 1515-1519). */
int axbc_graph_create(const uint32_t *col, const uint32_t *row, uint64_t n, uint64_t m,
                      const uint32_t *reach, axbc_graph **g);

/* The reference's ingest pipeline on the device: upload a host edge list
 * (uint64 pairs, vertices < n), mirror it when `undirected` (mirror,
 * src/axbc2d.c:333-351), sort, drop repeats and self-loops except a self-loop
 * that sorts first (norm_graph, 818-841), with H == 1 remove degree-1
 * vertices into reach (degree_reduction + init_bc_1degree, 695-807, 866-876;
 * undirected graphs only), and build the CSC (build_csc, 883-907).  Same
 * result as axbc_edges_to_csc + axbc_graph_create. */
int axbc_graph_from_edges(const uint64_t *edges, uint64_t nedges, uint64_t n, int undirected, int H,
                          axbc_graph **g);

/* Synthetic inputs generated and built on the device: an R-MAT graph of
 * 2^scale vertices and edgefactor*2^scale generated edges (initiator
 * A,B,C = .57,.19,.19), vertex ids scrambled, self-loops and duplicates
 * removed, mirrored unless `directed`.  H == 1 applies the one-degree
 * reduction.  (The reference generates with the Graph500 generator,
 * src/axbc2d.c:518-527; this generator is the library's own.) */
int axbc_graph_generate_rmat(int scale, int edgefactor, uint64_t seed, int directed, int H,
                             axbc_graph **g);
/* The reference's own synthetic input, generated on the device: the Graph500
 * Kronecker generator's edge list (gen_graph, src/axbc2d.c:518-527, calling
 * make_graph, generator/make_graph.c:35-105), element for element, for
 * 2^scale vertices, edgefactor * 2^scale edges, seeds seed1/seed2 (the
 * reference passes 23 and 24) and a 2x2 initiator (NULL: .57/.19/.19/.05).
 * At most 10^9 edges.
 *   axbc_kron_edges: the edges as int64 (source, target) pairs into
 *     edges_host (2 * edgefactor * 2^scale values).  stage 2 is make_graph's
 *     output; stage 1 the same edges before the edge scramble; stage 0 before
 *     the vertex permutation.
 *   axbc_graph_generate_kronecker: the graph the reference builds from that
 *     list (mirror, norm_graph, optional one-degree reduction, build_csc). */
int axbc_kron_edges(int scale, int edgefactor, uint64_t seed1, uint64_t seed2,
                    const double *initiator, int stage, int64_t *edges_host);
int axbc_graph_generate_kronecker(int scale, int edgefactor, uint64_t seed1, uint64_t seed2,
                                  const double *initiator, int H, axbc_graph **g);
/* side x side 4-neighbour grid; each grid edge dropped with probability
 * drop_prob; floor(longrange_frac * kept_edges) extra random edges; mirrored. */
int axbc_graph_generate_grid(uint32_t side, double drop_prob, double longrange_frac,
                             uint64_t seed, axbc_graph **g);

int axbc_graph_destroy(axbc_graph *g);
/* n, m, device bytes held, 1 if the adjacency is symmetric */
int axbc_graph_info(const axbc_graph *g, uint64_t *n, uint64_t *m, uint64_t *bytes,
                    int *symmetric);
/* Degrees (get_deg, src/cuda_kernels.cu:1452-1454), CSC arrays, reach. */
int axbc_graph_get_deg(const axbc_graph *g, uint32_t *deg_host);
int axbc_graph_get_csc(const axbc_graph *g, uint32_t *col_host, uint32_t *row_host,
                       uint32_t *reach_host);

/* -------------------------------------------------------------- contexts */

/* A context holds the BC state of one computation on one graph: bc (float),
 * per-pivot state, the multi-source batch state and the sampler.  `stream`
 * is a cudaStream_t or NULL for a stream of its own. */
int axbc_ctx_create(axbc_graph *g, void *stream, axbc_ctx **ctx);
int axbc_ctx_destroy(axbc_ctx *ctx);
/* bc = 0, sampler state cleared */
int axbc_ctx_reset(axbc_ctx *ctx);
/* device bytes held by the context */
int axbc_ctx_bytes(const axbc_ctx *ctx, uint64_t *bytes);

/* Tuning knobs (autotuner output).  push_factor: a forward level pushes from
 * the frontier when frontier_edges * push_factor < unvisited_edges, else it
 * pulls into unvisited vertices; a batched level also pushes when its
 * frontier's degree sum is below n/4, unless push_factor_batch >= 1e30 (every
 * level pulls).  Both default to 8 (measured on Graph500 scale 20 and 23 and a
 * 1024x1024 grid: factors 2-32 within a few percent of each other, 1 up to 50%
 * slower); axbc_autotune picks them per graph. */
int axbc_ctx_set_tuning(axbc_ctx *ctx, double push_factor_single, double push_factor_batch);

/* Autotuner: times trial passes from the given pivots (up to 128 batched, in
 * batches of the width; the first 4 plain) over a grid of direction-switch
 * factors and batch widths, keeps the fastest setting in the context and
 * returns it.  The context's bc and last dependency vector come back as they
 * were before the call: both are copied aside first and restored after the
 * trial passes.  On failure the factors stay unchanged. */
typedef struct {
    double push_factor_single;
    double push_factor_batch;
    int32_t batch_width;       /* fastest width <= AXBC_MAX_BATCH on these pivots */
    int32_t pad;
    double batch_te_per_s;     /* best trial rates */
    double plain_te_per_s;
} axbc_tuning;
int axbc_autotune(axbc_ctx *ctx, const uint32_t *pivots, int npivots, int H, axbc_tuning *out);

/* ---- per-pivot (plain form) ----
 * One Brandes pass from v0 with selection probability p: forward BFS with
 * uint32 path counts, backward float dependencies, bc update, exactly as
 * setcuda + bc_func_mono + update_bc_cuda (src/cuda_kernels.cu:1532-1554,
 * src/axbc2d.c:1514-1659, src/cuda_kernels.cu:289-302).  H == 1 adds the
 * reach sum of pre_update_bc_cuda (src/cuda_kernels.cu:358-373).  The host
 * drives one launch sequence per BFS level. */
typedef struct {
    uint64_t nvisited;  /* vertices reached, root included */
    uint64_t all;       /* reach total added in the root term */
    uint64_t te;        /* traversed edges: 2 * degree sum of reached vertices */
    int32_t levels;     /* first empty BFS level */
    int32_t pad;
} axbc_pivot_stats;

int axbc_run_pivot(axbc_ctx *ctx, uint32_t v0, double p, int H, axbc_pivot_stats *stats);

/* One plain Brandes pass from v0 that allocates no device memory.  It has
 * no counterpart in the reference.  It is for callers that cannot call
 * cudaMalloc: applications whose device memory belongs to another allocator or
 * a fixed budget, loops that must not synchronise the device through
 * cudaMalloc/cudaFree, or plug-ins that may only use the buffers handed to
 * them.  col/row/reach (reach may be NULL: all zero) describe the graph in the
 * reference's CSC layout and bc (n floats, updated in place) is the output --
 * all device pointers owned by the caller; stream is a cudaStream_t or NULL.
 * Scratch lives in one fixed __device__ array of about 5.6 MB that every GPU
 * loading the library holds until exit; graphs above 2^18 vertices, or with
 * more than 2^14 span items of vertices of degree > 1024, return
 * AXBC_ERR_RANGE.  The first call on a device looks the array's address up
 * (make it before any stream capture), and looks it up again when the
 * device's context changed (after cudaDeviceReset).  Calls share the array:
 * overlapping calls race, so serialise them.  Results equal axbc_run_pivot's. */
int axbc_bc_pivot_static(const uint32_t *col, const uint32_t *row, const uint32_t *reach,
                         uint64_t n, uint64_t m, uint32_t v0, double p, int H, float *bc,
                         void *stream, axbc_pivot_stats *stats);

/* ---- batched (multi-source) form ----
 * k <= AXBC_MAX_BATCH pivots in one multi-source pass (one bit per pivot in a
 * 32-bit mask per vertex for k <= 32, a 64-bit mask above; a pivot may
 * repeat).  bc receives the pivots' updates in list order, bit-identical to k
 * calls of axbc_run_pivot.  stats may be NULL. */
int axbc_run_batch(axbc_ctx *ctx, const uint32_t *v0, const double *p, int k, int H,
                   axbc_pivot_stats *stats);

/* ---- sampled run (the reference's main loop) ----
 * Draws pivots with heuristic z (-z 0..6), stops after nbfs rounds (-N) or
 * when Bader's criterion holds for nchecks check vertices (-c, -x).  Sampling
 * and the stop test run on the device.  batch_width 1 reproduces the
 * reference's round sequence; larger widths draw each batch from the
 * distributions as they stood before it (src/axbc2d.c:2729-3156). */
typedef struct {
    int32_t z;            /* heuristic 0..6 */
    int32_t bader_c;      /* Bader constant; 0 disables the stop test */
    uint64_t nbfs;        /* round limit (capped at n) */
    uint32_t nchecks;     /* check vertices */
    int32_t H;            /* 1: one-degree reach terms */
    int64_t seed;         /* srand48 seed; 4343543 is the reference default */
    int32_t batch_width;  /* 1..AXBC_MAX_WIDTH pivots drawn per snapshot */
    int32_t pad;
} axbc_run_params;

typedef struct {
    uint64_t nrounds;     /* pivots applied */
    uint64_t skipped;     /* degree-0 draws */
    uint64_t dropped;     /* rounds lost to the bad-sample limit */
    uint64_t rounds;      /* round counter at the end */
    uint64_t te;          /* traversed edges of the applied pivots */
    int32_t stopped;      /* 1 if Bader's criterion ended the run */
    int32_t batches;      /* batches launched */
} axbc_run_result;

int axbc_run_sampled(axbc_ctx *ctx, const axbc_run_params *prm, axbc_run_result *res);
/* ---- the sampler and the stop test, one call each ----
 * axbc_srand48: the drand48 state srand48(seed) sets (the reference seeds with
 * 4343543, src/axbc2d.c:2736).  axbc_sample: one draw of heuristic z
 * (src/axbc2d.c:2873-3051) from the context's current bc and last dependency
 * vector; *rng (drand48 state) and *mix (-z 6 mixture state, 0..4, ignored
 * for other z; the reference starts it at uniform_int(4, 0)) advance in place;
 * first = 1 before
 * any pivot is applied (the dynamic heuristics then draw uniformly).  Rejection
 * of repeated pivots and degree-0 roots is the caller's, as in the reference's
 * loop.  axbc_bader_check: *satisfied = 1 if every check vertex v has
 * bc[v] / 2 >= c * n (src/axbc2d.c:2846-2870). */
uint64_t axbc_srand48(int64_t seed);
int axbc_sample(axbc_ctx *ctx, int z, uint64_t *rng, uint32_t *mix, int first, uint32_t *v0,
                double *p);
int axbc_bader_check(axbc_ctx *ctx, const uint32_t *checks, uint32_t x, uint32_t c,
                     int *satisfied);

/* ---- request server (many sampled runs over resident graphs) ----
 * The reference serves one job per process.  The server keeps graphs resident
 * and runs submitted sampled runs (the parameters of axbc_run_sampled, widths
 * 1..AXBC_MAX_WIDTH) with one worker thread and stream per graph, packing the
 * drawn rounds of the requests of one graph into the up to 64 lanes of a
 * shared multi-source pass; passes on different graphs overlap on the device.  Each
 * request's bc, pivots and counters are bit-identical to axbc_run_sampled with
 * the same parameters.  Admission: a request's device state must fit in the
 * budget's remaining bytes; otherwise it waits in arrival order. */
typedef struct axbc_server axbc_server;

enum {
    AXBC_REQ_QUEUED = 0,   /* waiting for admission */
    AXBC_REQ_RUNNING = 1,  /* admitted; device state allocated */
    AXBC_REQ_DONE = 2,     /* result held on the host until released */
    AXBC_REQ_FAILED = 3
};

typedef struct {
    int32_t state;            /* AXBC_REQ_* */
    int32_t status;           /* AXBC_OK or the error of a failed request */
    axbc_run_result result;   /* valid once done */
    uint64_t bytes;           /* device bytes the request holds while running */
    uint64_t submit_ns, start_ns, finish_ns;  /* steady clock */
    char error[256];
} axbc_request_info;

typedef struct {
    uint64_t budget, in_use;  /* request-state device bytes */
    uint64_t queued, admitted, completed;
    uint64_t passes, lanes;   /* multi-source passes run, lanes filled */
} axbc_server_stats_t;

/* hbm_budget: device bytes for request state (0: 80% of free memory now). */
int axbc_server_create(uint64_t hbm_budget, axbc_server **server);
/* Make graph g (owned by the caller, alive until the server is destroyed)
 * resident, with its own stream and worker thread; H is the graph's one-degree
 * reduction (requests must match).  The graph's static sampling distributions
 * (degree-based and LCC) are built before the call returns, so that no request
 * waits for them. */
int axbc_server_add_graph(axbc_server *server, axbc_graph *g, int H, int *graph_id);
/* Queue a sampled run; AXBC_ERR_BUSY if it can never fit in the budget. */
int axbc_request_submit(axbc_server *server, int graph_id, const axbc_run_params *prm,
                        uint64_t *request_id);
int axbc_request_poll(axbc_server *server, uint64_t request_id, axbc_request_info *info);
/* Block until done or failed (timeout_ms < 0: no limit; AXBC_ERR_TIMEOUT). */
int axbc_request_wait(axbc_server *server, uint64_t request_id, int64_t timeout_ms,
                      axbc_request_info *info);
/* A done request's bc (n floats) and applied pivots (up to cap, *count = all). */
int axbc_request_result(axbc_server *server, uint64_t request_id, float *bc_host,
                        uint32_t *pivots, double *probs, uint64_t cap, uint64_t *count);
/* Forget a done, failed or still queued request (a running one: AXBC_ERR_STATE). */
int axbc_request_release(axbc_server *server, uint64_t request_id);
int axbc_server_stats(axbc_server *server, axbc_server_stats_t *stats);
/* Per resident graph: passes run, lanes filled, worker time spent on it (ns). */
int axbc_server_graph_stats(axbc_server *server, int graph_id, uint64_t *passes, uint64_t *lanes,
                            uint64_t *busy_ns);
/* Drops queued requests, finishes admitted ones, frees everything. */
int axbc_server_destroy(axbc_server *server);

/* The pivots applied by the last sampled run, in order, with their p. */
int axbc_get_pivots(const axbc_ctx *ctx, uint32_t *v0, double *p, uint64_t cap,
                    uint64_t *count);
/* The check vertices drawn by the last sampled run. */
int axbc_get_checks(const axbc_ctx *ctx, uint32_t *checks, uint32_t cap);

/* ---- results ---- */
/* get_bc (src/cuda_kernels.cu:1461-1463): n floats. */
int axbc_get_bc(axbc_ctx *ctx, float *bc_host);
/* get_delta (:1465-1467): the last applied pivot's dependencies, n floats. */
int axbc_get_delta(axbc_ctx *ctx, float *delta_host);
/* The last plain pivot's path counts and levels (get_sigma / get_lvl). */
int axbc_get_sigma(axbc_ctx *ctx, uint32_t *sigma_host);
int axbc_get_levels(axbc_ctx *ctx, int32_t *lvl_host);
/* One source of the last batch: its path counts, depths (-1 unreached) and
 * dependencies. */
int axbc_get_batch_source(axbc_ctx *ctx, int source, uint32_t *sigma_host, int32_t *lvl_host,
                          float *delta_host);
/* Device pointer of bc (n floats) for callers that keep results on the GPU. */
int axbc_bc_device_ptr(axbc_ctx *ctx, float **bc_dev);
/* Wait for all work of the context. */
int axbc_ctx_sync(axbc_ctx *ctx);

/* ---- profiling ----
 * With profiling on, the library records a CUDA event pair on the context's
 * stream around each of its kernel launches and the algorithmic bytes of the
 * launch (the traversed-edge byte model: per traversed edge 4/W+4 bytes
 * forward and 4/W+8 backward for a batch of W pivots, 8 and 12 for one pivot;
 * 20 bytes per vertex per pivot for the update).  Kinds:
 * 0 batched forward push, 1 batched forward pull, 2 level bookkeeping,
 * 3 batched backward, 4 heavy-vertex combine, 5 bc update, 6 sampler,
 * 7 plain forward, 8 plain backward, 9 plain other, 10 a whole batched
 * pass in one persistent launch. */
#define AXBC_PROF_KINDS 11
int axbc_ctx_profile(axbc_ctx *ctx, int enable);
/* per kind: total milliseconds, launches, algorithmic bytes; clears the records */
int axbc_ctx_profile_read(axbc_ctx *ctx, double *ms, uint64_t *count, double *bytes, int nkinds);
/* The individual timed launches, in order: kind (AXBC_PROF_KINDS order),
 * forward level (-1: none), ms and model bytes; up to cap records, *count =
 * all; the records stay (axbc_ctx_profile_read clears them). */
int axbc_ctx_profile_records(axbc_ctx *ctx, int32_t *kinds, int32_t *tags, float *ms, double *bytes,
                             uint64_t cap, uint64_t *count);
/* kernels launched by this context since it was created */
int axbc_ctx_launches(const axbc_ctx *ctx, uint64_t *launches);

/* ---- persistent level loop ----
 * A batched pass normally launches four kernels per forward level and two or
 * three per backward depth.  On graphs of many narrow levels it can instead
 * run as one cooperative launch (all blocks resident, a bounded grid barrier
 * between phases).  mode 1 always, -1 never, 0 (default) for batches of at
 * most 8 pivots when the context's last batch was deeper than 64 levels or,
 * for its first batch, when no vertex has more than 64 neighbours.
 * blocks_per_sm: blocks of the cooperative grid per SM (0 keeps the current
 * setting, default 4).  Results
 * are the same bits either way.  A barrier wait that runs out of its budget
 * (about 4 s) ends the pass with AXBC_ERR_TIMEOUT.  No counterpart in the
 * reference (its host synchronises every level). */
int axbc_ctx_set_persistent(axbc_ctx *ctx, int mode, int blocks_per_sm);
/* Self-test of that grid barrier on the current device: `rounds` barriers
 * over blocks_per_sm blocks per SM; block absent_block (>= 0) never arrives,
 * so the first wait runs out of budget_cycles (SM clock cycles) and every
 * block returns.  *err_site: 0, or the 1-based barrier whose wait ran out;
 * *leads: barriers completed; *ms: the launch's time. */
int axbc_selftest_grid_barrier(int blocks_per_sm, int rounds, long long budget_cycles, int absent_block,
                               int *err_site, uint32_t *leads, float *ms);

/* ---- work counting ----
 * With counting on, batched passes launch counting builds of the forward
 * push, forward pull and backward kernels (one launch per level, as with
 * profiling; slower, for measurement only).  Per kind (AXBC_PROF_KINDS order)
 * four counters: the bytes the launches must move at least (every 4-byte word
 * they must read or write once, whole sectors not counted), adjacency entries
 * scanned, (edge, pivot) gathers of a neighbour's per-pivot value, and
 * (vertex, pivot) values written.  No counterpart in the reference. */
#define AXBC_WORK_FIELDS 4
int axbc_ctx_count(axbc_ctx *ctx, int enable);
/* counts[kind * AXBC_WORK_FIELDS + field] for kinds < nkinds since the last read; clears them */
int axbc_ctx_count_read(axbc_ctx *ctx, uint64_t *counts, int nkinds);

/* Test hooks: the next n device allocations made by the library fail with
 * AXBC_ERR_NOMEM (host-side failure injection; 0 clears it); or the
 * allocation after the next `skip` ones fails (-1 clears it).  Device bytes the
 * library holds at the moment, for leak checks. */
void axbc_inject_alloc_failures(int n);
void axbc_inject_alloc_failure_after(int skip);
uint64_t axbc_device_bytes_live(void);

/* Per forward level of the last batch (up to max_levels; *levels = all):
 * vertices newly reached over all pivots, their degree sum, direction (1:
 * push), and the level's vertex list (count > cap: the level was scanned). */
int axbc_ctx_level_stats(axbc_ctx *ctx, uint64_t *count, uint64_t *te, int32_t *push,
                         uint32_t *list_count, uint32_t *list_cap, int max_levels, int *levels);

/* ---- diagnostics ----
 * The bc update computes float(double(x) / p) with a float two-product path
 * and falls back to the double divide near float rounding midpoints; this
 * runs both on n generated (x, p) pairs on the device and counts results
 * that differ (must be 0) and how many took the double divide. */
int axbc_selftest_division(uint64_t n, uint64_t seed, uint64_t *mismatches, uint64_t *exact_path);

/* ---- static pivot distributions (device) ---- */
/* (uint32)deg^2, neighbour-degree sums (sum_deg_neigh_func, src/axbc2d.c:
 * 1758-1845) and local clustering coefficients (lcc_func, :1847-1935). */
int axbc_graph_degree2(axbc_graph *g, uint32_t *out_host);
int axbc_graph_sum_deg_neigh(axbc_graph *g, uint32_t *out_host);
int axbc_graph_lcc(axbc_graph *g, float *out_host);

#ifdef __cplusplus
}
#endif
#endif /* AXBC_H */
