/*
 * CPU oracle for the AxBC sampled-Brandes path -- TEST INFRASTRUCTURE ONLY.
 *
 * Restates, in plain C, what the reference does on one rank in single-GPU
 * ("mono") mode.  Every function cites the reference file:line it follows
 * (paths are relative to the fvella/axbc project root).  Only tests/,
 * __graft_entry__.smoke() and bench.py's CPU-baseline leg use this file.
 *
 * Compile with -ffp-contract=off: the float expressions below must round
 * exactly as written (the CUDA kernels use __fadd_rn/__fmul_rn/__fdiv_rn).
 */
#include "oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

/* ------------------------------------------------------------------------ */
/* drand48: X' = (0x5DEECE66D * X + 0xB) mod 2^48; lrand48 = X' >> 17;
 * srand48(s): X = (s & 0xffffffff) << 16 | 0x330E.  (POSIX; used through
 * init_rand / uniform_int / uniform_double, src/axbc2d.c:2143-2176.)       */
void orc_srand48(orc_rng *r, int64_t seed)
{
    r->x = (((uint64_t)seed & 0xffffffffULL) << 16) | 0x330EULL;
}

int64_t orc_lrand48(orc_rng *r)
{
    r->x = (0x5DEECE66DULL * r->x + 0xBULL) & 0xFFFFFFFFFFFFULL;
    return (int64_t)(r->x >> 17);
}

void orc_lrand48_seq(int64_t seed, int64_t count, int64_t *out)
{
    orc_rng r;
    orc_srand48(&r, seed);
    for (int64_t i = 0; i < count; i++) out[i] = orc_lrand48(&r);
}

#define ORC_RAND_MAX 2147483647.0

/* uniform_int(max, min) = lrand48() % (max-min+1) + min in LOCINT (uint32)
 * arithmetic, src/axbc2d.c:2155-2164.  A modulus that wraps to 0 (max =
 * 2^32-1) would divide by zero in the reference; here it leaves the draw
 * unreduced. */
static uint32_t uniform_int(orc_rng *r, uint32_t max, uint32_t min)
{
    uint32_t mod = max - min + 1u;
    int64_t x = orc_lrand48(r);
    if (mod == 0) return (uint32_t)x + min;
    return (uint32_t)(x % (int64_t)mod) + min;
}

/* uniform01 / uniform_double, src/axbc2d.c:2166-2176 */
static double uniform01(orc_rng *r)
{
    return (double)orc_lrand48(r) / ORC_RAND_MAX;
}

/* ------------------------------------------------------------------------ */
/* Graph pipeline                                                            */

static int cmp_edge(const void *a, const void *b)
{
    const uint64_t *x = (const uint64_t *)a, *y = (const uint64_t *)b;
    if (x[0] != y[0]) return x[0] < y[0] ? -1 : 1;
    if (x[1] != y[1]) return x[1] < y[1] ? -1 : 1;
    return 0;
}

/* norm_graph, src/axbc2d.c:818-841 (one rank: cmpedge == lexicographic).
 * The first edge is always kept, even if it is a self-loop. */
static uint64_t norm_graph(uint64_t *ed, uint64_t ned)
{
    uint64_t l, n;
    if (ned == 0) return 0;
    qsort(ed, ned, 2 * sizeof(uint64_t), cmp_edge);
    for (n = l = 1; n < ned; n++) {
        if (((ed[2 * n] != ed[2 * (n - 1)]) || (ed[2 * n + 1] != ed[2 * (n - 1) + 1])) &&
            (ed[2 * n] != ed[2 * n + 1])) {
            ed[2 * l] = ed[2 * n];
            ed[2 * l + 1] = ed[2 * n + 1];
            l++;
        }
    }
    return l;
}

/* degree_reduction on one rank, src/axbc2d.c:695-807.  Returns the kept edge
 * count; *o_ed receives the removed (neighbour, leaf) pairs sorted, *pnod_out
 * how many of them the merge consumed (the reference's rem_ed). */
static uint64_t degree_reduction(uint64_t *r_ed, uint64_t nedge, uint64_t **o_out,
                                 uint64_t *pnod_out)
{
    uint64_t u, v, next_u, next_v, prev_u = (uint64_t)-1;
    uint64_t nod = 0, ne = 0, pnod = 0, i;
    uint64_t *n_ed, *o_ed;

    *o_out = NULL;
    *pnod_out = 0;
    if (nedge == 0) return 0; /* the reference reads out of bounds here */
    qsort(r_ed, nedge, 2 * sizeof(uint64_t), cmp_edge);
    n_ed = (uint64_t *)calloc(2 * nedge + 2, sizeof(uint64_t));
    o_ed = (uint64_t *)calloc(2 * nedge + 2, sizeof(uint64_t));

    for (i = 0; i + 1 < nedge; i++) {
        u = r_ed[2 * i];
        v = r_ed[2 * i + 1];
        next_u = r_ed[2 * i + 2];
        next_v = r_ed[2 * i + 3];
        if ((u == v) || ((u == next_u) && (v == next_v))) {
            prev_u = u;
            continue;
        }
        if ((u != next_u) && (u != prev_u)) {
            o_ed[2 * nod] = v;
            o_ed[2 * nod + 1] = u;
            nod++;
        } else {
            n_ed[2 * ne] = u;
            n_ed[2 * ne + 1] = v;
            ne++;
        }
        prev_u = u;
    }
    u = r_ed[2 * nedge - 2];
    v = r_ed[2 * nedge - 1];
    if (u == prev_u) {
        n_ed[2 * ne] = u;
        n_ed[2 * ne + 1] = v;
        ne++;
    } else if (u != v) {
        o_ed[2 * nod] = v;
        o_ed[2 * nod + 1] = u;
        nod++;
    }

    qsort(o_ed, nod, 2 * sizeof(uint64_t), cmp_edge);

    if (nod > 0) {
        uint64_t kept = ne;
        ne = 0;
        for (i = 0; i < kept; i++) {
            while (pnod < nod && n_ed[2 * i] > o_ed[2 * pnod]) pnod++;
            if (pnod < nod && n_ed[2 * i] == o_ed[2 * pnod] && n_ed[2 * i + 1] == o_ed[2 * pnod + 1]) {
                pnod++;
                continue;
            }
            r_ed[2 * ne] = n_ed[2 * i];
            r_ed[2 * ne + 1] = n_ed[2 * i + 1];
            ne++;
        }
    } else {
        memcpy(r_ed, n_ed, 2 * ne * sizeof(uint64_t));
    }
    free(n_ed);
    *o_out = o_ed;
    *pnod_out = pnod;
    return ne;
}

/* mirror (src/axbc2d.c:333-351), norm_graph (2551, 2607), degree_reduction
 * (2566), init_bc_1degree (866-876), build_csc (883-907). */
int orc_pipeline(const uint64_t *edges, uint64_t ned, uint64_t n, int undirected, int H,
                 uint32_t **col_out, uint32_t **row_out, uint64_t *m_out,
                 uint32_t **reach_out, uint64_t *rem_ed_out)
{
    uint64_t *ed = (uint64_t *)malloc((4 * ned + 2) * sizeof(uint64_t));
    uint64_t i, cnt = ned;
    uint32_t *col, *row, *reach, *tmp;
    uint64_t rem_ed = 0;

    if (!ed) return 1;
    for (i = 0; i < ned; i++) {
        if (edges[2 * i] >= n || edges[2 * i + 1] >= n) {
            free(ed);
            return 2;
        }
    }
    memcpy(ed, edges, 2 * ned * sizeof(uint64_t));
    if (undirected) {
        uint64_t k = 0;
        for (i = 0; i < ned; i++) {
            if (ed[2 * i] != ed[2 * i + 1]) {
                ed[2 * ned + 2 * k] = ed[2 * i + 1];
                ed[2 * ned + 2 * k + 1] = ed[2 * i];
                k++;
            }
        }
        cnt = ned + k;
    }
    reach = (uint32_t *)calloc(n ? n : 1, sizeof(uint32_t));
    if (H != 0) {
        uint64_t *o_ed = NULL, pnod = 0;
        cnt = norm_graph(ed, cnt);
        if (H == 1) {
            cnt = degree_reduction(ed, cnt, &o_ed, &pnod);
            for (i = 0; i < pnod; i++) reach[o_ed[2 * i]]++;
            rem_ed = pnod;
            free(o_ed);
        }
    }
    cnt = norm_graph(ed, cnt);

    tmp = (uint32_t *)calloc(n ? n : 1, sizeof(uint32_t));
    col = (uint32_t *)calloc(n + 1, sizeof(uint32_t));
    row = (uint32_t *)malloc((cnt ? cnt : 1) * sizeof(uint32_t));
    for (i = 0; i < cnt; i++) tmp[ed[2 * i + 1]]++;
    col[0] = 0;
    for (i = 1; i <= n; i++) col[i] = col[i - 1] + tmp[i - 1];
    memcpy(tmp, col, n * sizeof(uint32_t));
    for (i = 0; i < cnt; i++) {
        uint64_t c = ed[2 * i + 1];
        row[tmp[c]] = (uint32_t)ed[2 * i];
        tmp[c]++;
    }
    free(tmp);
    free(ed);
    *col_out = col;
    *row_out = row;
    *m_out = cnt;
    *reach_out = reach;
    *rem_ed_out = rem_ed;
    return 0;
}

void orc_free(void *p) { free(p); }

/* ------------------------------------------------------------------------ */
/* One pivot                                                                 */

/* Dependency of vertex c at depth d.  Successor term (scan_frt_mono,
 * src/cuda_kernels.cu:763-767):
 *   ((delta[r] + 1) / (float)sigma[r]) * (float)sigma[c]   if lvl[r] == d+1
 * accumulated onto delta[c] = (float)reach[c] (init_delta, :1521-1530). */
static float dependency(const orc_graph *g, uint32_t c, int d, const int32_t *lvl,
                        const uint32_t *sigma, const float *delta, int order)
{
    const uint32_t beg = g->col[c];
    const uint32_t deg = g->col[c + 1] - beg;
    const float sc = (float)sigma[c];
    float acc = (float)g->reach[c];
    uint32_t s0, c0, j;

    if (order == 1) {
        for (j = 0; j < deg; j++) {
            uint32_t r = g->row[beg + j];
            if (lvl[r] == d + 1) {
                float a = ((delta[r] + 1.0f) / (float)sigma[r]) * sc;
                acc = acc + a;
            }
        }
        return acc;
    }
    for (s0 = 0; s0 < deg; s0 += ORC_SPAN) {
        uint32_t s1 = s0 + ORC_SPAN < deg ? s0 + ORC_SPAN : deg;
        float P = 0.0f;
        int first = 1;
        for (c0 = s0; c0 < s1; c0 += ORC_CHUNK) {
            float t[ORC_CHUNK];
            int w;
            for (j = 0; j < ORC_CHUNK; j++) {
                uint32_t pos = c0 + j;
                t[j] = 0.0f;
                if (pos < s1) {
                    uint32_t r = g->row[beg + pos];
                    if (lvl[r] == d + 1) t[j] = ((delta[r] + 1.0f) / (float)sigma[r]) * sc;
                }
            }
            for (w = 1; w < ORC_CHUNK; w <<= 1)
                for (j = 0; j < ORC_CHUNK; j += 2 * w) t[j] = t[j] + t[j + w];
            P = first ? t[0] : P + t[0];
            first = 0;
        }
        acc = acc + P;
    }
    return acc;
}

/* setcuda (src/cuda_kernels.cu:1532-1554) + set_mlp_cuda (:862-876) +
 * bc_func_mono (src/axbc2d.c:1514-1659) + scan_col_mono2 (:588-658) +
 * scan_frt_mono (:719-772) + pre_update_bc_cuda (:358-373, gated by -H 1 at
 * src/axbc2d.c:1636) + update_bc (:269-286). */
/* The traversal of one pivot: levels, path counts, dependencies and the
 * counts its bc update needs (st->all includes reach[v0]). */
static int pivot_traverse(const orc_graph *g, uint32_t v0, int H, int order, int32_t *lvl,
                          uint32_t *sigma, float *delta, uint32_t *queue, uint64_t *levstart,
                          orc_pivot_stats *st)
{
    const uint64_t n = g->n;
    uint64_t v, q, qend, nvisited = 1, te = 0;
    int level = 0, depth;
    uint32_t all = 0, reach_v0;

    if (v0 >= n) return 1;
    reach_v0 = g->reach[v0];
    for (v = 0; v < n; v++) {
        lvl[v] = -1;
        sigma[v] = 0;
        delta[v] = (float)g->reach[v];
    }
    lvl[v0] = 0;
    sigma[v0] = 1;
    queue[0] = v0;
    levstart[0] = 0;
    levstart[1] = 1;
    qend = 1;

    /* forward: level-synchronous, sigma sums over every parent at level-1 */
    for (;;) {
        uint64_t fs, fe, nfrt;
        level++;
        fs = levstart[level - 1];
        fe = levstart[level];
        for (q = fs; q < fe; q++) {
            uint32_t c = queue[q];
            uint32_t e;
            for (e = g->col[c]; e < g->col[c + 1]; e++) {
                uint32_t r = g->row[e];
                if (lvl[r] == -1) {
                    lvl[r] = level;
                    queue[qend++] = r;
                }
                if (lvl[r] == level) sigma[r] += sigma[c];
            }
        }
        nfrt = qend - fe;
        levstart[level + 1] = qend;
        if (!nfrt) break;
        nvisited += nfrt;
    }

    /* backward: depth level-2 down to 1 (do-while: depth 0 only when level==2) */
    depth = level - 2;
    if (depth >= 0) {
        do {
            for (q = levstart[depth]; q < levstart[depth + 1]; q++) {
                uint32_t c = queue[q];
                delta[c] = dependency(g, c, depth, lvl, sigma, delta, order);
            }
            depth--;
        } while (depth > 0);
    }

    if (H == 1) {
        for (v = 0; v < n; v++)
            if (lvl[v] > 0) all += g->reach[v];
    }
    all += reach_v0;

    for (q = 0; q < qend; q++) {
        uint32_t c = queue[q];
        te += (uint64_t)(g->col[c + 1] - g->col[c]);
    }
    st->nvisited = nvisited;
    st->all = all;
    st->te = 2 * te;
    st->levels = level;
    return 0;
}

/* update_bc (src/cuda_kernels.cu:269-286) with the traversal's dependencies */
static void pivot_apply(const orc_graph *g, uint32_t v0, double p, const float *delta,
                        const orc_pivot_stats *st, float *bc)
{
    const uint64_t n = g->n, nv = st->nvisited + st->all;
    const uint32_t reach_v0 = g->reach[v0];
    uint64_t v;
    for (v = 0; v < n; v++) {
        if (v == v0) {
            if (reach_v0 > 0) bc[v] = bc[v] + (float)((uint64_t)reach_v0 * (nv - 2));
            continue;
        }
        bc[v] = bc[v] + (float)((double)(delta[v] * (float)(reach_v0 + 1u)) / p);
    }
}

static int bc_pivot_ws(const orc_graph *g, uint32_t v0, double p, int H, int order, float *bc,
                       int32_t *lvl, uint32_t *sigma, float *delta, uint32_t *queue,
                       uint64_t *levstart, orc_pivot_stats *st)
{
    orc_pivot_stats s;
    memset(&s, 0, sizeof(s));
    int rc = pivot_traverse(g, v0, H, order, lvl, sigma, delta, queue, levstart, &s);
    if (st) *st = s;
    if (rc) return rc;
    pivot_apply(g, v0, p, delta, &s, bc);
    return 0;
}

int orc_bc_pivot(const orc_graph *g, uint32_t v0, double p, int H, int order, float *bc,
                 int32_t *lvl, uint32_t *sigma, float *delta, orc_pivot_stats *st)
{
    uint32_t *queue = (uint32_t *)malloc((g->n + 1) * sizeof(uint32_t));
    uint64_t *levstart = (uint64_t *)malloc((g->n + 3) * sizeof(uint64_t));
    int rc = bc_pivot_ws(g, v0, p, H, order, bc, lvl, sigma, delta, queue, levstart, st);
    free(queue);
    free(levstart);
    return rc;
}

int orc_bc_pivots(const orc_graph *g, const uint32_t *v0, const double *p, uint64_t k, int H,
                  int order, float *bc, float *delta_last, uint64_t *te_out)
{
    const uint64_t n = g->n;
    int32_t *lvl = (int32_t *)malloc((n + 1) * sizeof(int32_t));
    uint32_t *sigma = (uint32_t *)malloc((n + 1) * sizeof(uint32_t));
    float *delta = (float *)malloc((n + 1) * sizeof(float));
    uint32_t *queue = (uint32_t *)malloc((n + 1) * sizeof(uint32_t));
    uint64_t *levstart = (uint64_t *)malloc((n + 3) * sizeof(uint64_t));
    uint64_t i, te = 0;
    int rc = 0;
    for (i = 0; i < k && !rc; i++) {
        orc_pivot_stats st;
        rc = bc_pivot_ws(g, v0[i], p[i], H, order, bc, lvl, sigma, delta, queue, levstart, &st);
        te += st.te;
    }
    if (delta_last && k) memcpy(delta_last, delta, n * sizeof(float));
    if (te_out) *te_out = te;
    free(lvl);
    free(sigma);
    free(delta);
    free(queue);
    free(levstart);
    return rc;
}

int orc_bc_pivots_omp(const orc_graph *g, const uint32_t *v0, const double *p, uint64_t k, int H,
                      int threads, float *bc, uint64_t *te_out)
{
    const uint64_t n = g->n;
    uint64_t te_total = 0;
    int rc_total = 0;
#ifdef _OPENMP
    if (threads > 0) omp_set_num_threads(threads);
#pragma omp parallel reduction(+ : te_total) reduction(| : rc_total)
#endif
    {
        int32_t *lvl = (int32_t *)malloc((n + 1) * sizeof(int32_t));
        uint32_t *sigma = (uint32_t *)malloc((n + 1) * sizeof(uint32_t));
        float *delta = (float *)malloc((n + 1) * sizeof(float));
        uint32_t *queue = (uint32_t *)malloc((n + 1) * sizeof(uint32_t));
        uint64_t *levstart = (uint64_t *)malloc((n + 3) * sizeof(uint64_t));
        float *part = (float *)calloc(n + 1, sizeof(float));
        int64_t i;
#ifdef _OPENMP
#pragma omp for schedule(dynamic, 1)
#endif
        for (i = 0; i < (int64_t)k; i++) {
            orc_pivot_stats st;
            rc_total |= bc_pivot_ws(g, v0[i], p[i], H, 0, part, lvl, sigma, delta, queue,
                                    levstart, &st);
            te_total += st.te;
        }
#ifdef _OPENMP
#pragma omp critical
#endif
        {
            uint64_t v;
            for (v = 0; v < n; v++) bc[v] += part[v];
        }
        free(lvl);
        free(sigma);
        free(delta);
        free(queue);
        free(levstart);
        free(part);
    }
    if (te_out) *te_out = te_total;
    return rc_total;
}

/* ------------------------------------------------------------------------ */
/* Static distributions                                                      */

/* degree2[i] = pow(degree[i], 2) stored in uint32 (src/axbc2d.c:2681-2685);
 * the x86-64 conversion keeps the low 32 bits of the square. */
void orc_degree2(const orc_graph *g, uint32_t *out)
{
    uint64_t i;
    for (i = 0; i < g->n; i++) {
        uint64_t d = g->col[i + 1] - g->col[i];
        out[i] = (uint32_t)(d * d);
    }
}

/* sum_deg_neigh_func, src/axbc2d.c:1758-1845 (one rank). */
void orc_sum_deg_neigh(const orc_graph *g, uint32_t *out)
{
    uint64_t i;
    for (i = 0; i < g->n; i++) {
        uint32_t cnt = 0, e;
        for (e = g->col[i]; e < g->col[i + 1]; e++) {
            uint32_t w = g->row[e];
            cnt += g->col[w + 1] - g->col[w];
        }
        out[i] = cnt;
    }
}

/* lcc_func, src/axbc2d.c:1847-1935 (one rank): for every neighbour w of i
 * count the entries x of adj(w), x != i, that also occur in adj(i);
 * lcc = (float)count / (float)(uint32)(deg*(deg-1)); 0 for deg < 2. */
void orc_lcc(const orc_graph *g, float *out)
{
    int64_t i;
#ifdef _OPENMP
#pragma omp parallel for schedule(dynamic, 64)
#endif
    for (i = 0; i < (int64_t)g->n; i++) {
        const uint32_t *ai = g->row + g->col[i];
        const uint32_t di = g->col[i + 1] - g->col[i];
        uint32_t counter = 0, j;
        if (di < 2) {
            out[i] = 0.0f;
            continue;
        }
        for (j = 0; j < di; j++) {
            uint32_t w = ai[j];
            const uint32_t *aw = g->row + g->col[w];
            const uint32_t dw = g->col[w + 1] - g->col[w];
            uint32_t a = 0, b = 0;
            /* both lists are sorted ascending: count matching pairs with
             * multiplicity (equal runs multiply) */
            while (a < dw && b < di) {
                if (aw[a] < ai[b]) a++;
                else if (aw[a] > ai[b]) b++;
                else {
                    uint32_t x = aw[a], ra = 0, rb = 0;
                    while (a < dw && aw[a] == x) { a++; ra++; }
                    while (b < di && ai[b] == x) { b++; rb++; }
                    if (x != (uint32_t)i) counter += ra * rb;
                }
            }
        }
        out[i] = (float)counter / (float)(uint32_t)(di * (di - 1u));
    }
}

/* Hierarchical prefix used for every float-weighted distribution (the
 * reference's prefix_by_row_float / prefix_by_col_float, src/axbc2d.c:
 * 1985-2058 and 2105-2139, accumulate in float left to right; here the sums
 * are double and two-level at both the element and the block scale, so that
 * no chain of dependent additions is longer than about 32 + n/32768 and the
 * device computes identical values in parallel). */
void orc_hprefix(const float *w, uint64_t n, double *local, double *csum)
{
    /* Two-level running sums in double, each level left to right:
     *  - a block of 1024 weights is 32 runs of 32; s = running sum inside the
     *    run, P = running sum of the finished runs' totals; local[i] = P + s;
     *    the block total is P after its last run;
     *  - blocks form groups of 32: L = running sum of block totals inside the
     *    group, G = running sum of the finished groups' totals; csum[b] = G + L.
     * The prefix is monotone for non-negative weights; the search below is
     * block-first, then inside the block. */
    const uint64_t B = ORC_SAMPLE_BLOCK, R = 32;
    const uint64_t nb = (n + B - 1) / B;
    uint64_t b, j, i;
    double G = 0.0, L = 0.0;
    for (b = 0; b < nb; b++) {
        double P = 0.0;
        const uint64_t e = (b + 1) * B < n ? (b + 1) * B : n;
        for (j = b * B; j < e; j += R) {
            const uint64_t je = j + R < e ? j + R : e;
            double s = 0.0;
            for (i = j; i < je; i++) {
                s = s + (double)w[i];
                local[i] = P + s;
            }
            P = P + s;
        }
        if (b % R == 0) L = 0.0;
        L = L + P;
        csum[b] = G + L;
        if (b % R == R - 1 || b == nb - 1) G = G + L;
    }
}

/* First index whose prefix reaches r (findsample_float, src/axbc2d.c:
 * 2199-2211), searched block-wise: first block with csum >= r, then the first
 * element with local >= r - csum[b-1]; the block's last element if rounding
 * leaves none.  *found = 0 when the total is NaN or below r. */
uint64_t orc_hsearch(const double *local, const double *csum, uint64_t n, double r, int *found)
{
    const uint64_t B = ORC_SAMPLE_BLOCK;
    const uint64_t nb = (n + B - 1) / B;
    uint64_t lo = 0, hi = nb, b, i, e;
    double rr;
    *found = 0;
    if (n == 0) return 0;
    if (isnan(csum[nb - 1]) || !(csum[nb - 1] >= r)) return n - 1;
    while (lo < hi) {
        uint64_t mid = (lo + hi) / 2;
        if (csum[mid] >= r) hi = mid;
        else lo = mid + 1;
    }
    b = lo;
    rr = r - (b > 0 ? csum[b - 1] : 0.0);
    e = (b + 1) * B < n ? (b + 1) * B : n;
    lo = b * B;
    hi = e;
    while (lo < hi) {
        uint64_t mid = (lo + hi) / 2;
        if (local[mid] >= rr) hi = mid;
        else lo = mid + 1;
    }
    i = lo < e ? lo : e - 1;
    *found = 1;
    return i;
}

/* first index i with prefix[i] >= r over a uint32 prefix that may wrap
 * (findsample_LOCINT, src/axbc2d.c:2188-2198) */
static uint64_t find_u32(const uint32_t *prefix, uint64_t n, uint32_t r, int *found)
{
    uint64_t i;
    *found = 0;
    for (i = 0; i < n; i++) {
        if (prefix[i] >= r) {
            *found = 1;
            return i;
        }
    }
    return n;
}

/* ------------------------------------------------------------------------ */
/* The sampling loop of main(), src/axbc2d.c:2729-3156, on one rank.
 *
 * W == 1 reproduces the reference's round sequence.  W > 1 is the batched
 * semantics: the pivots of a batch are drawn in the reference's order from the
 * distributions as they stood at the start of the batch; Bader's test is then
 * replayed between the batch's pivots so the loop stops exactly where the
 * sequential loop would, given those pivots.
 *
 * Guards (the reference reads out of bounds in these cases): a draw of v0 == N
 * from uniform_int(N,0) is counted as a skipped degree-0 round; a check vertex
 * equal to N reads bc = 0. */

typedef struct {
    int have_deg;
    uint32_t *deg, *deg2p, *sdn;
    uint32_t sum_deg;
    int have_lcc;
    float *lcc;
    double *lcc_local, *lcc_csum;
} static_dists;

static void pick_neighbour_z1(const orc_graph *g, const static_dists *sd, orc_rng *rng, uint64_t N,
                              uint32_t *v0)
{
    int found;
    uint32_t r = uniform_int(rng, sd->sum_deg, 0);
    uint64_t x = find_u32(sd->deg2p, g->n, r, &found);
    if (!found) x = N - 1;
    if (sd->deg[x] > 0) {
        uint32_t nb = 0;
        if (sd->deg[x] != 1) nb = uniform_int(rng, sd->deg[x] - 1, 0);
        x = g->row[g->col[x] + nb];
    }
    *v0 = (uint32_t)x;
}

/* Bader's stop test (src/axbc2d.c:2846-2870): every check vertex v has
 * bc[v]/2.0 >= c*N, with c a LOCINT (uint32). */
static int bader_satisfied(const float *bc, const uint32_t *checks, uint32_t x, uint64_t N,
                           uint32_t c)
{
    uint32_t i;
    for (i = 0; i < x; i++) {
        double b = checks[i] < N ? (double)bc[checks[i]] : 0.0;
        if (b / 2.0 < (double)((uint64_t)c * N)) return 0;
    }
    return 1;
}

int orc_run(const orc_graph *g, const orc_run_params *prm, float *bc_out, float *delta_last,
            uint32_t *pivots_out, double *p_out, uint64_t pivots_cap, uint32_t *checks_out,
            orc_run_result *res)
{
    const uint64_t N = g->n;
    const int z = prm->z;
    const int W = prm->W > 0 ? prm->W : 1;
    orc_rng rng;
    static_dists sd;
    uint64_t nbfs = prm->nbfs < N ? prm->nbfs : N;
    uint32_t *checks = (uint32_t *)calloc(prm->nchecks + 1, sizeof(uint32_t));
    uint32_t dist_mix = (uint32_t)z;
    int LIM;
    uint32_t *vs = (uint32_t *)calloc(N + 1, sizeof(uint32_t));
    float *bc = bc_out;
    float *bc_snap = (float *)calloc(N + 1, sizeof(float));
    float *delta_snap = (float *)calloc(N + 1, sizeof(float));
    double *bloc = (double *)malloc((N + 1) * sizeof(double));
    double *bcs = (double *)malloc((N / ORC_SAMPLE_BLOCK + 2) * sizeof(double));
    double *dloc = (double *)malloc((N + 1) * sizeof(double));
    double *dcs = (double *)malloc((N / ORC_SAMPLE_BLOCK + 2) * sizeof(double));
    float *wtmp = (float *)malloc((N + 1) * sizeof(float));
    uint64_t nrounds_snap = 0, ui = 0, i;
    uint32_t *bv = (uint32_t *)malloc(W * sizeof(uint32_t));
    double *bp = (double *)malloc(W * sizeof(double));
    uint64_t *bskip = (uint64_t *)malloc(W * sizeof(uint64_t));
    /* per-thread traversal workspaces: a batch's pivots are traversed in
     * parallel and applied in order, which gives the sequential result */
#ifdef _OPENMP
    const int nthr = (W > 1 && N >= 65536) ? omp_get_max_threads() : 1;
#else
    const int nthr = 1;
#endif
    int32_t **lvl = (int32_t **)calloc(nthr, sizeof(int32_t *));
    uint32_t **sigma = (uint32_t **)calloc(nthr, sizeof(uint32_t *));
    uint32_t **queue = (uint32_t **)calloc(nthr, sizeof(uint32_t *));
    uint64_t **levstart = (uint64_t **)calloc(nthr, sizeof(uint64_t *));
    float **bdelta = (float **)calloc(W, sizeof(float *));
    orc_pivot_stats *bst = (orc_pivot_stats *)calloc(W, sizeof(orc_pivot_stats));

    memset(res, 0, sizeof(*res));
    memset(&sd, 0, sizeof(sd));
    memset(bc, 0, N * sizeof(float));
    for (i = 0; i < (uint64_t)W; i++) bdelta[i] = (float *)malloc((N + 1) * sizeof(float));
    for (i = 0; i < (uint64_t)nthr; i++) {
        lvl[i] = (int32_t *)malloc((N + 1) * sizeof(int32_t));
        sigma[i] = (uint32_t *)malloc((N + 1) * sizeof(uint32_t));
        queue[i] = (uint32_t *)malloc((N + 1) * sizeof(uint32_t));
        levstart[i] = (uint64_t *)malloc((N + 3) * sizeof(uint64_t));
    }

    /* int LIMxSAMPLE = N*N (src/axbc2d.c:2835): the product is truncated */
    LIM = (int)(uint32_t)(N * N);

    orc_srand48(&rng, prm->seed);
    for (i = 0; i < prm->nchecks; i++) checks[i] = uniform_int(&rng, (uint32_t)N, 0);
    if (checks_out)
        for (i = 0; i < prm->nchecks; i++) checks_out[i] = checks[i];

    sd.deg = (uint32_t *)malloc((N + 1) * sizeof(uint32_t));
    for (i = 0; i < N; i++) sd.deg[i] = g->col[i + 1] - g->col[i];
    if (z == 0) {
        (void)uniform_int(&rng, (uint32_t)N, 0); /* discarded select_root1 (2760) */
    } else if (z == 6) {
        dist_mix = uniform_int(&rng, 4, 0);
    }
    if (z == 1 || z == 6) {
        sd.have_deg = 1;
        sd.deg2p = (uint32_t *)malloc((N + 1) * sizeof(uint32_t));
        sd.sdn = (uint32_t *)malloc((N + 1) * sizeof(uint32_t));
        orc_degree2(g, sd.deg2p);
        for (i = 1; i < N; i++) sd.deg2p[i] += sd.deg2p[i - 1];
        sd.sum_deg = N ? sd.deg2p[N - 1] : 0;
        orc_sum_deg_neigh(g, sd.sdn);
    }
    if (z == 2 || z == 6) {
        sd.have_lcc = 1;
        sd.lcc = (float *)malloc((N + 1) * sizeof(float));
        sd.lcc_local = (double *)malloc((N + 1) * sizeof(double));
        sd.lcc_csum = (double *)malloc((N / ORC_SAMPLE_BLOCK + 2) * sizeof(double));
        orc_lcc(g, sd.lcc);
        orc_hprefix(sd.lcc, N, sd.lcc_local, sd.lcc_csum);
    }

    while (ui < nbfs) {
        int nb = 0, j, stop = 0;
        uint64_t skipped_run = 0;
        double S_bc = 0, S_bci = 0, S_d = 0, S_lcc = 0;
        /* distributions of this batch's snapshot */
        if (N && nrounds_snap > 0) {
            if (z == 3 || z == 6) {
                orc_hprefix(bc_snap, N, bloc, bcs);
                S_bc = bcs[(N - 1) / ORC_SAMPLE_BLOCK];
            }
            if (z == 5) {
                for (i = 0; i < N; i++) wtmp[i] = 1.0f / (1.0f + bc_snap[i]);
                orc_hprefix(wtmp, N, bloc, bcs);
                S_bci = bcs[(N - 1) / ORC_SAMPLE_BLOCK];
            }
            if (z == 4 || z == 6) {
                orc_hprefix(delta_snap, N, dloc, dcs);
                S_d = dcs[(N - 1) / ORC_SAMPLE_BLOCK];
            }
        }
        if (sd.have_lcc && N) S_lcc = sd.lcc_csum[(N - 1) / ORC_SAMPLE_BLOCK];

        /* Bader check before the round (2846-2870) */
        if ((uint32_t)prm->bader_c > 0) {
            int sat = bader_satisfied(bc, checks, prm->nchecks, N, (uint32_t)prm->bader_c);
            if (sat) {
                res->stopped = 1;
                break;
            }
        }

        /* draw rounds until W pivots are accepted */
        while (nb < W && ui < nbfs) {
            uint32_t v0 = 0;
            double prob = 0;
            uint32_t BSM = 0;
            int isgood = 0;
            while (!isgood) {
                int found;
                if (BSM > (uint32_t)LIM) break;
                prob = 0;
                if (dist_mix == 0 || z == 0) {
                    v0 = uniform_int(&rng, (uint32_t)N, 0);
                    prob = 1.0 / (double)N;
                } else if (dist_mix == 1 || z == 1) {
                    pick_neighbour_z1(g, &sd, &rng, N, &v0);
                    if (v0 < N) prob = (double)sd.sdn[v0] / (double)sd.sum_deg;
                } else if (dist_mix == 2 || z == 2) {
                    double r = uniform01(&rng) * S_lcc;
                    uint64_t x = orc_hsearch(sd.lcc_local, sd.lcc_csum, N, r, &found);
                    if (!found) x = N - 1;
                    v0 = (uint32_t)x;
                    prob = (double)sd.lcc[v0] / S_lcc;
                } else if (dist_mix == 3 || z == 3) {
                    if (nrounds_snap == 0) {
                        v0 = uniform_int(&rng, (uint32_t)N, 0);
                        prob = 1.0 / (double)N;
                    } else {
                        double r = uniform01(&rng) * S_bc;
                        uint64_t x = orc_hsearch(bloc, bcs, N, r, &found);
                        if (!found) x = N - 1;
                        v0 = (uint32_t)x;
                        prob = (double)bc_snap[v0] / S_bc;
                    }
                } else if (dist_mix == 4 || z == 4) {
                    if (nrounds_snap == 0) {
                        v0 = uniform_int(&rng, (uint32_t)N, 0);
                        prob = 1.0 / (double)N;
                    } else {
                        double r = uniform01(&rng) * S_d;
                        uint64_t x = orc_hsearch(dloc, dcs, N, r, &found);
                        if (!found) x = N - 1;
                        v0 = (uint32_t)x;
                        prob = (double)delta_snap[v0] / S_d;
                    }
                } else if (dist_mix == 5 || z == 5) {
                    if (nrounds_snap == 0) {
                        v0 = uniform_int(&rng, (uint32_t)N, 0);
                        prob = 1.0 / (double)N;
                    } else {
                        double r = uniform01(&rng) * S_bci;
                        uint64_t x = orc_hsearch(bloc, bcs, N, r, &found);
                        if (!found) x = N - 1;
                        v0 = (uint32_t)x;
                        prob = 1.0 / ((double)bc_snap[v0] + 1.0) / S_bci;
                    }
                }
                if (z == 6) {
                    /* mixture probability (3026-3051) */
                    prob = 1.0 / (double)N;
                    if (nrounds_snap == 0) {
                        prob = prob + 1.0 / (double)N;
                        prob = prob + 1.0 / (double)N;
                    } else if (v0 < N) {
                        prob = prob + (double)bc_snap[v0] / S_bc;
                        prob = prob + (double)delta_snap[v0] / S_d;
                    }
                    if (v0 < N) {
                        prob = prob + (double)sd.sdn[v0] / (double)sd.sum_deg;
                        prob = prob + (double)sd.lcc[v0] / S_lcc;
                        prob = prob / 5.0;
                    }
                    dist_mix = uniform_int(&rng, 2, 0);
                }
                if (v0 < N && vs[v0] == 1) BSM++;
                else isgood = 1;
            }
            if (BSM > (uint32_t)LIM) { /* round dropped (3072-3077) */
                res->dropped++;
                ui++;
                continue;
            }
            if (v0 >= N || sd.deg[v0] == 0) { /* degree-0 root (3095-3111) */
                skipped_run++;
                if (v0 < N) vs[v0] = 1;
                ui++;
                continue;
            }
            vs[v0] = 1;
            bv[nb] = v0;
            bp[nb] = prob;
            bskip[nb] = skipped_run;
            skipped_run = 0;
            nb++;
            ui++;
        }

        /* run the batch: the pivots' traversals (in parallel when the graph
         * is large), then their bc updates in order */
#ifdef _OPENMP
#pragma omp parallel for schedule(dynamic, 1) num_threads(nthr) if (nthr > 1 && nb > 1)
#endif
        for (j = 0; j < nb; j++) {
#ifdef _OPENMP
            const int t = omp_get_thread_num();
#else
            const int t = 0;
#endif
            pivot_traverse(g, bv[j], prm->H, prm->order, lvl[t], sigma[t], bdelta[j], queue[t],
                           levstart[t], &bst[j]);
        }
        for (j = 0; j < nb; j++) {
            /* Bader replay before pivot j > 0 of the batch */
            if (j > 0 && prm->bader_c > 0) {
                int sat = bader_satisfied(bc, checks, prm->nchecks, N, (uint32_t)prm->bader_c);
                if (sat) {
                    stop = 1;
                    break;
                }
            }
            pivot_apply(g, bv[j], bp[j], bdelta[j], &bst[j], bc);
            res->skipped += bskip[j];
            if (pivots_out && res->nrounds < pivots_cap) {
                pivots_out[res->nrounds] = bv[j];
                if (p_out) p_out[res->nrounds] = bp[j];
            }
            res->nrounds++;
            res->te += bst[j].te;
            memcpy(delta_snap, bdelta[j], N * sizeof(float));
        }
        if (stop) {
            res->stopped = 1;
            break;
        }
        if (skipped_run) {
            int sat = 0;
            if ((uint32_t)prm->bader_c > 0 && nb > 0) {
                sat = bader_satisfied(bc, checks, prm->nchecks, N, (uint32_t)prm->bader_c);
            }
            if (sat) {
                res->stopped = 1;
                break;
            }
            res->skipped += skipped_run;
        }
        memcpy(bc_snap, bc, N * sizeof(float));
        nrounds_snap = res->nrounds;
    }
    res->ui_end = ui;
    if (delta_last) memcpy(delta_last, delta_snap, N * sizeof(float));

    for (i = 0; i < (uint64_t)W; i++) free(bdelta[i]);
    free(bdelta);
    free(bst);
    free(checks);
    free(vs);
    free(bc_snap);
    free(delta_snap);
    free(bloc);
    free(bcs);
    free(dloc);
    free(dcs);
    free(wtmp);
    free(bv);
    free(bp);
    free(bskip);
    for (i = 0; i < (uint64_t)nthr; i++) {
        free(lvl[i]);
        free(sigma[i]);
        free(queue[i]);
        free(levstart[i]);
    }
    free(lvl);
    free(sigma);
    free(queue);
    free(levstart);
    free(sd.deg);
    free(sd.deg2p);
    free(sd.sdn);
    free(sd.lcc);
    free(sd.lcc_local);
    free(sd.lcc_csum);
    return 0;
}
