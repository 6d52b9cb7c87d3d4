/*
 * CPU oracle for the AxBC sampled-Brandes path.
 *
 * TEST INFRASTRUCTURE ONLY.  This is a plain-C restatement of the reference
 * algorithm (fvella/axbc, src/axbc2d.c + the single-GPU kernels of
 * src/cuda_kernels.cu) used as the parity checker by tests/, by
 * __graft_entry__.smoke() and by bench.py's CPU-baseline leg.  Nothing in the
 * product library links or calls it.
 *
 * Parity status: the reference BC path cannot be built here (it needs MPI and
 * pre-Volta warp intrinsics, and has no CPU implementation), so the BC
 * restatement is "parity unpinned" against reference outputs.  It is pinned
 * against textbook exact-BC graphs and against the reference's own graph
 * generator (compiled from its sources into oracle/_ref by oracle/Makefile).
 *
 * Arithmetic follows the reference types: uint32 sigma (wraps mod 2^32),
 * int32 levels, float delta / bc, double p.  The dependency sum of each vertex
 * uses one fixed summation order (the "canonical accumulation" below) that the
 * CUDA kernels reproduce bit for bit; the reference itself accumulates with
 * float atomics in an unspecified order.
 */
#ifndef AXBC_ORACLE_H
#define AXBC_ORACLE_H
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Canonical accumulation order of the dependency (delta) sum of one vertex:
 * successor terms in adjacency order, grouped into chunks of ORC_CHUNK
 * positions summed as a balanced binary tree, chunk sums added left to right
 * inside spans of ORC_SPAN positions, span sums added left to right onto
 * (float)reach[v]. */
#define ORC_CHUNK 32
#define ORC_SPAN 1024
/* Block size of the hierarchical (double) prefix used by the float-weighted
 * pivot distributions. */
#define ORC_SAMPLE_BLOCK 1024

typedef struct {
    uint64_t n;            /* vertices */
    uint64_t m;            /* adjacency entries */
    const uint32_t *col;   /* n+1 offsets (reference CSC "col") */
    const uint32_t *row;   /* m neighbour ids (reference CSC "row") */
    const uint32_t *reach; /* n removed-leaf counts (zeros unless -H 1) */
} orc_graph;

typedef struct {
    uint64_t nvisited; /* vertices reached incl. the root */
    uint64_t all;      /* reach sum added to nvisited in the root term */
    uint64_t te;       /* traversed edges: 2 * sum of degrees of reached vertices */
    int32_t levels;    /* the reference's final `level` (first empty level) */
    int32_t pad;
} orc_pivot_stats;

typedef struct {
    int32_t z;         /* -z heuristic 0..6 */
    int32_t bader_c;   /* -c */
    uint64_t nbfs;     /* -N */
    uint32_t nchecks;  /* -x */
    int32_t H;         /* -H 0/1 */
    int64_t seed;      /* srand48 seed (reference default 4343543) */
    int32_t W;         /* batch width: 1 = reference sequence */
    int32_t order;     /* 0 canonical accumulation, 1 plain adjacency order */
} orc_run_params;

typedef struct {
    uint64_t nrounds;  /* pivots whose Brandes pass was applied */
    uint64_t skipped;  /* degree-0 (or out-of-range) draws counted as skipped */
    uint64_t dropped;  /* rounds lost to the bad-sample limit */
    uint64_t ui_end;   /* value of the round counter when the loop ended */
    uint64_t te;       /* traversed edges of the applied pivots */
    int32_t stopped;   /* 1 if Bader's criterion ended the loop */
    int32_t pad;
} orc_run_result;

/* ---- drand48 family (POSIX), restated ---- */
typedef struct { uint64_t x; } orc_rng;
void orc_srand48(orc_rng *r, int64_t seed);
int64_t orc_lrand48(orc_rng *r);
void orc_lrand48_seq(int64_t seed, int64_t count, int64_t *out);

/* ---- graph pipeline (mirror, norm_graph, degree_reduction, build_csc) ---- */
int orc_pipeline(const uint64_t *edges, uint64_t ned, uint64_t n, int undirected, int H,
                 uint32_t **col_out, uint32_t **row_out, uint64_t *m_out,
                 uint32_t **reach_out, uint64_t *rem_ed_out);
void orc_free(void *p);

/* ---- one pivot (bc_func_mono + setcuda + update_bc) ---- */
int orc_bc_pivot(const orc_graph *g, uint32_t v0, double p, int H, int order,
                 float *bc, int32_t *lvl, uint32_t *sigma, float *delta,
                 orc_pivot_stats *st);
/* fixed pivot list, sequential order; bc accumulates in place */
int orc_bc_pivots(const orc_graph *g, const uint32_t *v0, const double *p, uint64_t k,
                  int H, int order, float *bc, float *delta_last, uint64_t *te_out);
/* fixed pivot list, OpenMP over pivots (timing baseline; per-thread partial bc) */
int orc_bc_pivots_omp(const orc_graph *g, const uint32_t *v0, const double *p, uint64_t k,
                      int H, int threads, float *bc, uint64_t *te_out);

/* ---- static distributions ---- */
void orc_degree2(const orc_graph *g, uint32_t *out);          /* (uint32)(deg*deg) */
void orc_sum_deg_neigh(const orc_graph *g, uint32_t *out);    /* sum of neighbour degrees */
void orc_lcc(const orc_graph *g, float *out);                  /* lcc_func */
/* hierarchical prefix: local[n] in-block prefix (runs of 32 inside blocks of
 * 1024), csum[nb] prefix of block totals (groups of 32 blocks) */
void orc_hprefix(const float *w, uint64_t n, double *local, double *csum);
uint64_t orc_hsearch(const double *local, const double *csum, uint64_t n, double r, int *found);

/* ---- the whole sampling loop of main() ---- */
int orc_run(const orc_graph *g, const orc_run_params *prm, float *bc_out, float *delta_last,
            uint32_t *pivots_out, double *p_out, uint64_t pivots_cap, uint32_t *checks_out,
            orc_run_result *res);

#ifdef __cplusplus
}
#endif
#endif
