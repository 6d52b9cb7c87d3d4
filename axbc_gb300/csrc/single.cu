// Plain form: one pivot, one launch sequence per BFS level, the host reading
// the frontier size after every level -- the structure of bc_func_mono
// (src/axbc2d.c:1514-1659) with GB300 kernels:
//   forward level: push from the frontier queue (warp per frontier vertex,
//     lanes over its neighbours, atomicCAS claims, atomicAdd path counts) or
//     pull into every unvisited vertex (warp per vertex, integer warp sum);
//   backward level: warp per vertex of the depth, the canonical dependency
//     sum (lane = adjacency position, tree per 32, chunks then spans in order);
//   update: one thread per vertex.
// Vertices with more than AXBC_SPAN neighbours are split into span items.
#include "common.cuh"

__global__ void k_reset1(int32_t *__restrict__ lvl, uint32_t *__restrict__ sigma,
                         float *__restrict__ delta, const uint32_t *__restrict__ reach, uint64_t n)
{
    for (uint64_t v = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; v < n;
         v += (uint64_t)gridDim.x * blockDim.x) {
        lvl[v] = -1;
        sigma[v] = 0;
        delta[v] = __uint2float_rn(reach[v]);
    }
}

// warp-aggregated append of the lanes' newly discovered vertices
__device__ __forceinline__ void append_new(bool isnew, uint32_t r, uint32_t deg_r, uint32_t rdeg_r,
                                           uint32_t *queue, PivotCounters *pc)
{
    const unsigned lane = lane_id();
    unsigned m = __ballot_sync(FULL_MASK, isnew);
    if (!m) return;
    const int leader = __ffs(m) - 1;
    uint32_t base = 0;
    if ((int)lane == leader) base = atomicAdd(&pc->qtail, (uint32_t)__popc(m));
    base = __shfl_sync(FULL_MASK, base, leader);
    if (isnew) queue[base + __popc(m & ((1u << lane) - 1u))] = r;
    uint32_t d = __reduce_add_sync(FULL_MASK, isnew ? deg_r : 0u);
    uint32_t rd = __reduce_add_sync(FULL_MASK, isnew ? rdeg_r : 0u);
    if ((int)lane == leader) {
        atomicAdd(&pc->newdeg, (unsigned long long)d);
        atomicAdd(&pc->visited_rdeg, (unsigned long long)rd);
    }
}

// Forward level L, push: tasks [0,nf) are the frontier vertices of depth L-1
// (light ones), then the span items of heavy vertices at depth L-1
// (scan_col_mono2, src/cuda_kernels.cu:588-658: a neighbour r is new if its
// level is unset; sigma[r] += sigma[c] when r's level is L).
__global__ void k_fwd_push1(Adj a, const uint32_t *__restrict__ rcol, uint32_t qs, uint32_t nf,
                            int32_t *lvl, uint32_t *sigma, uint32_t *queue, PivotCounters *pc, int L)
{
    const unsigned lane = lane_id();
    const uint64_t ntask = nf + a.n_heavy_items;
    const uint64_t nw = (uint64_t)gridDim.x * blockDim.x / 32;
    for (uint64_t t = (blockIdx.x * (uint64_t)blockDim.x + threadIdx.x) / 32; t < ntask; t += nw) {
        uint32_t c, b0, b1;
        if (t < nf) {
            c = queue[qs + t];
            b0 = a.col[c];
            b1 = a.col[c + 1];
            if (b1 - b0 > AXBC_SPAN) continue;
        } else {
            const uint64_t h = t - nf;
            c = a.hitem_v[h];
            if (lvl[c] != L - 1) continue;
            b0 = a.col[c] + a.hitem_k[h] * AXBC_SPAN;
            b1 = min(a.col[c + 1], b0 + AXBC_SPAN);
        }
        const uint32_t sc = sigma[c];
        for (uint32_t base = b0; base < b1; base += 32) {
            const uint32_t e = base + lane;
            bool isnew = false;
            uint32_t r = 0, dr = 0, rdr = 0;
            if (e < b1) {
                r = a.row[e];
                int l = lvl[r];
                if (l == -1) {
                    int old = atomicCAS(&lvl[r], -1, L);
                    isnew = (old == -1);
                    l = isnew ? L : old;
                }
                if (l == L) atomicAdd(&sigma[r], sc);
                if (isnew) {
                    dr = a.col[r + 1] - a.col[r];
                    rdr = rcol[r + 1] - rcol[r];
                }
            }
            append_new(isnew, r, dr, rdr, queue, pc);
        }
    }
}

// Forward level L, pull: every unvisited vertex sums sigma over all of its
// in-neighbours at level L-1 (no early exit: every parent counts).  Tasks:
// blocks of 32 vertex ids, then the span items of heavy vertices.
__global__ void k_fwd_pull1(Adj rv, const uint32_t *__restrict__ fcol, int32_t *lvl,
                            uint32_t *sigma, uint32_t *queue, PivotCounters *pc, int L)
{
    const unsigned lane = lane_id();
    const uint64_t n = rv.n;
    const uint64_t nblk = (n + 31) / 32;
    const uint64_t ntask = nblk + rv.n_heavy_items;
    const uint64_t nw = (uint64_t)gridDim.x * blockDim.x / 32;
    for (uint64_t t = (blockIdx.x * (uint64_t)blockDim.x + threadIdx.x) / 32; t < ntask; t += nw) {
        if (t < nblk) {
            const uint64_t u_l = t * 32 + lane;
            bool cand = false;
            if (u_l < n && lvl[u_l] == -1) {
                uint32_t d = rv.col[u_l + 1] - rv.col[u_l];
                cand = d > 0 && d <= AXBC_SPAN;
            }
            unsigned act = __ballot_sync(FULL_MASK, cand);
            bool mine_new = false;
            uint32_t mine_sigma = 0;
            while (act) {
                const int j = __ffs(act) - 1;
                act &= act - 1;
                const uint32_t u = (uint32_t)(t * 32 + j);
                const uint32_t b0 = rv.col[u], b1 = rv.col[u + 1];
                uint32_t acc = 0;
                bool found = false;
                for (uint32_t e = b0 + lane; e < b1; e += 32) {
                    const uint32_t v = rv.row[e];
                    if (lvl[v] == L - 1) {
                        acc += sigma[v];
                        found = true;
                    }
                }
                acc = __reduce_add_sync(FULL_MASK, acc);
                const bool any = __any_sync(FULL_MASK, found);
                if ((int)lane == j) {
                    mine_new = any;
                    mine_sigma = acc;
                }
            }
            if (mine_new) {
                lvl[u_l] = L;
                sigma[u_l] = mine_sigma;
            }
            uint32_t dr = 0, rdr = 0;
            if (mine_new) {
                dr = fcol[u_l + 1] - fcol[u_l];
                rdr = rv.col[u_l + 1] - rv.col[u_l];
            }
            append_new(mine_new, (uint32_t)u_l, dr, rdr, queue, pc);
        } else {
            const uint64_t h = t - nblk;
            const uint32_t u = rv.hitem_v[h];
            const int lu = lvl[u];
            if (lu != -1 && lu != L) continue;
            const uint32_t b0 = rv.col[u] + rv.hitem_k[h] * AXBC_SPAN;
            const uint32_t b1 = min(rv.col[u + 1], b0 + AXBC_SPAN);
            uint32_t acc = 0;
            bool found = false;
            for (uint32_t e = b0 + lane; e < b1; e += 32) {
                const uint32_t v = rv.row[e];
                if (lvl[v] == L - 1) {
                    acc += sigma[v];
                    found = true;
                }
            }
            acc = __reduce_add_sync(FULL_MASK, acc);
            const bool any = __any_sync(FULL_MASK, found);
            bool isnew = false;
            if (any && lane == 0) {
                atomicAdd(&sigma[u], acc);
                isnew = atomicCAS(&lvl[u], -1, L) == -1;
            }
            uint32_t dr = 0, rdr = 0;
            if (isnew) {
                dr = fcol[u + 1] - fcol[u];
                rdr = rv.col[u + 1] - rv.col[u];
            }
            append_new(isnew, u, dr, rdr, queue, pc);
        }
    }
}

// Backward depth d (scan_frt_mono, src/cuda_kernels.cu:719-772): tasks
// [0,nseg) are the light vertices of the depth, then heavy span items whose
// partial sums go to partial[item].
__global__ void k_bwd1(Adj a, const uint32_t *__restrict__ queue, uint32_t ls, uint32_t nseg,
                       const int32_t *__restrict__ lvl, const uint32_t *__restrict__ sigma,
                       float *delta, const uint32_t *__restrict__ reach, float *partial, int d)
{
    const unsigned lane = lane_id();
    const uint64_t ntask = nseg + a.n_heavy_items;
    const uint64_t nw = (uint64_t)gridDim.x * blockDim.x / 32;
    for (uint64_t t = (blockIdx.x * (uint64_t)blockDim.x + threadIdx.x) / 32; t < ntask; t += nw) {
        uint32_t c, b0, b1;
        const bool light = t < nseg;
        if (light) {
            c = queue[ls + t];
            b0 = a.col[c];
            b1 = a.col[c + 1];
            if (b1 - b0 > AXBC_SPAN) continue;
        } else {
            const uint64_t h = t - nseg;
            c = a.hitem_v[h];
            if (lvl[c] != d) continue;
            b0 = a.col[c] + a.hitem_k[h] * AXBC_SPAN;
            b1 = min(a.col[c + 1], b0 + AXBC_SPAN);
        }
        const float sc = __uint2float_rn(sigma[c]);
        float P = 0.0f;
        for (uint32_t base = b0; base < b1; base += 32) {
            const uint32_t e = base + lane;
            float tl = 0.0f;
            bool succ = false;
            if (e < b1) {
                const uint32_t r = a.row[e];
                if (lvl[r] == d + 1) {
                    succ = true;
                    tl = dep_term(delta[r], sigma[r], sc);
                }
            }
            if (!__any_sync(FULL_MASK, succ)) continue;
            P = __fadd_rn(P, warp_tree_sum(tl));
        }
        if (lane == 0) {
            if (light) delta[c] = __fadd_rn(__uint2float_rn(reach[c]), P);
            else partial[t - nseg] = P;
        }
    }
}

// heavy vertices of depth d: reach + span partials, in span order
__global__ void k_bwd_combine1(Adj a, const int32_t *__restrict__ lvl, float *delta,
                               const uint32_t *__restrict__ reach, const float *__restrict__ partial,
                               int d)
{
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < a.n_heavy;
         i += gridDim.x * blockDim.x) {
        const uint32_t v = a.heavy_v[i];
        if (lvl[v] != d) continue;
        float acc = __uint2float_rn(reach[v]);
        for (uint32_t k = a.heavy_first[i]; k < a.heavy_first[i + 1]; k++)
            acc = __fadd_rn(acc, partial[k]);
        delta[v] = acc;
    }
}

// pre_update_bc_cuda (src/cuda_kernels.cu:339-373): sum of reach over lvl > 0
__global__ void k_reach_sum1(const int32_t *__restrict__ lvl, const uint32_t *__restrict__ reach,
                             uint64_t n, PivotCounters *pc)
{
    unsigned long long s = 0;
    for (uint64_t v = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; v < n;
         v += (uint64_t)gridDim.x * blockDim.x)
        if (lvl[v] > 0) s += reach[v];
    s = __reduce_add_sync(FULL_MASK, (unsigned)s);
    if (lane_id() == 0 && s) atomicAdd(&pc->reach_sum, s);
}

// update_bc (src/cuda_kernels.cu:269-286), applied to every vertex.  The
// root term uses nvt = nvt_base (+ all, when add_all: all = reach_v0, plus
// the reach sum when add_sum), all in uint32 as in bc_func_mono.
__global__ void k_update1(float *bc, const float *__restrict__ delta, uint64_t n, uint32_t v0,
                          double p, const uint32_t *__restrict__ reach_v0_ptr,
                          unsigned long long nvt_base, const PivotCounters *__restrict__ pc,
                          int add_all, int add_sum)
{
    const uint32_t reach_v0 = *reach_v0_ptr;
    uint32_t all = 0;
    if (add_all) all = (add_sum ? (uint32_t)pc->reach_sum : 0u) + reach_v0;
    const unsigned long long nvt = nvt_base + all;
    const InvSplit iv = inv_split(p);
    for (uint64_t v = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; v < n;
         v += (uint64_t)gridDim.x * blockDim.x) {
        if (v == v0) {
            if (reach_v0 > 0) bc[v] = __fadd_rn(bc[v], bc_root_term(reach_v0, nvt));
            continue;
        }
        const float dv = delta[v];
        if (dv == 0.0f && p > 0.0) continue;  // x + float(0/p) == x
        bc[v] = __fadd_rn(bc[v], bc_term_fast(dv, reach_v0, p, iv));
    }
}

__global__ void k_set_root1(uint32_t v0, int level, uint32_t sig, int32_t *lvl, uint32_t *sigma,
                            uint32_t *queue, PivotCounters *pc, const uint32_t *col,
                            const uint32_t *rcol)
{
    lvl[v0] = level;
    sigma[v0] = sig;
    queue[0] = v0;
    pc->qtail = 1;
    pc->newdeg = col[v0 + 1] - col[v0];
    pc->reach_sum = 0;
    pc->visited_rdeg = rcol[v0 + 1] - rcol[v0];
}

int axbc_ensure_single(axbc_ctx *c)
{
    if (c->single_ready) return AXBC_OK;
    const uint64_t n = c->g->n;
    ALLOC_MISSING(c->lvl, n * 4, &c->bytes);
    ALLOC_MISSING(c->sigma, n * 4, &c->bytes);
    ALLOC_MISSING(c->delta, n * 4, &c->bytes);
    ALLOC_MISSING(c->queue, (n + 1) * 4, &c->bytes);
    ALLOC_MISSING(c->partial, (c->g->fwd.n_heavy_items + 1) * 4, &c->bytes);
    ALLOC_MISSING(c->pc, sizeof(PivotCounters), &c->bytes);
    if (!c->pc_host) CU(cudaMallocHost((void **)&c->pc_host, sizeof(PivotCounters)));
    CU(cudaMemset(c->pc, 0, sizeof(PivotCounters)));
    c->single_ready = true;
    return AXBC_OK;
}

// setcuda (src/cuda_kernels.cu:1532-1554): levels unset, sigma 0, delta = reach
int axbc_single_reset(axbc_ctx *c)
{
    TRY(axbc_ensure_single(c));
    ProfScope ps(c, KP_PLAIN_OTHER, (double)c->g->n * 16.0);
    k_reset1<<<axbc_grid_for(c, 256, 8), 256, 0, c->stream>>>(c->lvl, c->sigma, c->delta,
                                                             c->g->reach, c->g->n);
    CU_LAUNCH("k_reset1");
    return AXBC_OK;
}

// set_mlp_cuda (:862-876) for the root: level, sigma, queue[0]; counters
int axbc_single_set_root(axbc_ctx *c, uint32_t v0, int level, uint32_t sig)
{
    cudaStream_t s = c->stream;
    {
        ProfScope ps(c, KP_PLAIN_OTHER, 0);
        k_set_root1<<<1, 1, 0, s>>>(v0, level, sig, c->lvl, c->sigma, c->queue, c->pc,
                                    c->g->fwd.col, c->g->rev.col);
    }
    CU_LAUNCH("k_set_root1");
    CU(cudaMemcpyAsync(c->pc_host, c->pc, sizeof(PivotCounters), cudaMemcpyDeviceToHost, s));
    CU(cudaStreamSynchronize(s));
    c->s_front_deg = c->pc_host->newdeg;
    c->s_prev_newdeg = c->pc_host->newdeg;
    c->s_visited_rdeg = c->pc_host->visited_rdeg;
    c->level_te.assign(1, (double)c->pc_host->newdeg);
    return AXBC_OK;
}

// One forward level (scan_col_csc_cuda_mono, src/cuda_kernels.cu:1088-1177):
// the frontier is queue[qs, qs+nf); new vertices are appended after it.
int axbc_single_forward_level(axbc_ctx *c, uint32_t qs, uint32_t nf, int level, uint64_t *nfrt)
{
    axbc_graph *g = c->g;
    cudaStream_t s = c->stream;
    const int grid = axbc_grid_for(c, 256, 8);
    const uint32_t tail = qs + nf;
    CU(cudaMemcpyAsync(&c->pc->qtail, &tail, 4, cudaMemcpyHostToDevice, s));
    const uint64_t unvisited = g->m - c->s_visited_rdeg;
    const bool push = (double)c->s_front_deg * c->push_factor_single < (double)unvisited;
    {
        ProfScope ps(c, KP_PLAIN_FWD, (double)c->s_front_deg * 8.0);
        if (push) k_fwd_push1<<<grid, 256, 0, s>>>(g->fwd, g->rev.col, qs, nf, c->lvl, c->sigma,
                                                  c->queue, c->pc, level);
        else k_fwd_pull1<<<grid, 256, 0, s>>>(g->rev, g->fwd.col, c->lvl, c->sigma, c->queue,
                                             c->pc, level);
    }
    CU_LAUNCH("forward level");
    CU(cudaMemcpyAsync(c->pc_host, c->pc, sizeof(PivotCounters), cudaMemcpyDeviceToHost, s));
    CU(cudaStreamSynchronize(s));
    *nfrt = c->pc_host->qtail - tail;
    c->s_front_deg = c->pc_host->newdeg - c->s_prev_newdeg;
    c->s_prev_newdeg = c->pc_host->newdeg;
    c->s_visited_rdeg = c->pc_host->visited_rdeg;
    c->level_te.push_back((double)c->s_front_deg);
    return AXBC_OK;
}

// One backward depth (scan_frt_csc_cuda_mono, src/cuda_kernels.cu:1013-1080)
// over the vertices queue[ls, ls+nseg) at depth d.
int axbc_single_backward_level(axbc_ctx *c, uint32_t ls, uint32_t nseg, int d)
{
    axbc_graph *g = c->g;
    cudaStream_t s = c->stream;
    const double te = d >= 0 && d < (int)c->level_te.size() ? c->level_te[d] : 0.0;
    {
        ProfScope ps(c, KP_PLAIN_BWD, te * 12.0);
        k_bwd1<<<axbc_grid_for(c, 256, 8), 256, 0, s>>>(g->fwd, c->queue, ls, nseg, c->lvl,
                                                       c->sigma, c->delta, g->reach, c->partial, d);
    }
    if (g->fwd.n_heavy) {
        ProfScope ps(c, KP_PLAIN_BWD, 0);
        k_bwd_combine1<<<(g->fwd.n_heavy + 255) / 256, 256, 0, s>>>(g->fwd, c->lvl, c->delta,
                                                                   g->reach, c->partial, d);
    }
    CU_LAUNCH("backward level");
    return AXBC_OK;
}

// sum of reach over vertices with level > 0 into pc->reach_sum
int axbc_single_reach_sum(axbc_ctx *c)
{
    CU(cudaMemsetAsync(&c->pc->reach_sum, 0, 8, c->stream));
    ProfScope ps(c, KP_PLAIN_OTHER, (double)c->g->n * 8.0);
    k_reach_sum1<<<axbc_grid_for(c, 256, 8), 256, 0, c->stream>>>(c->lvl, c->g->reach, c->g->n, c->pc);
    CU_LAUNCH("reach sum");
    return AXBC_OK;
}

int axbc_single_update(axbc_ctx *c, uint32_t v0, double p, const uint32_t *reach_v0_dev,
                       uint64_t nvt_base, int add_all, int add_sum)
{
    {
        ProfScope ps(c, KP_PLAIN_OTHER, (double)c->g->n * 12.0);
        k_update1<<<axbc_grid_for(c, 256, 8), 256, 0, c->stream>>>(
            c->bc, c->delta, c->g->n, v0, p, reach_v0_dev, nvt_base, c->pc, add_all, add_sum);
    }
    CU_LAUNCH("update");
    c->delta_last_valid = false;  // the last pivot's delta is c->delta
    return AXBC_OK;
}

extern "C" int axbc_run_pivot(axbc_ctx *c, uint32_t v0, double p, int H, axbc_pivot_stats *st)
{
    CHECK_ARG(c, "axbc_run_pivot: null context");
    axbc_graph *g = c->g;
    CHECK_ARG(v0 < g->n, "axbc_run_pivot: v0 >= n");
    CHECK_ARG(H == 0 || H == 1, "axbc_run_pivot: H must be 0 or 1");
    TRY(axbc_single_reset(c));
    TRY(axbc_single_set_root(c, v0, 0, 1));

    c->levstart.assign(2, 0);
    c->levstart[1] = 1;
    uint64_t nvisited = 1;
    int level = 0;
    for (;;) {
        level++;
        const uint32_t qs = (uint32_t)c->levstart[level - 1];
        const uint32_t nf = (uint32_t)(c->levstart[level] - c->levstart[level - 1]);
        uint64_t nfrt = 0;
        TRY(axbc_single_forward_level(c, qs, nf, level, &nfrt));
        c->levstart.push_back(c->levstart[level] + nfrt);
        if (!nfrt) break;
        nvisited += nfrt;
    }
    // backward: depth level-2 down to 1; depth 0 only when level == 2
    int depth = level - 2;
    if (depth >= 0) {
        do {
            TRY(axbc_single_backward_level(c, (uint32_t)c->levstart[depth],
                                           (uint32_t)(c->levstart[depth + 1] - c->levstart[depth]),
                                           depth));
            depth--;
        } while (depth > 0);
    }
    if (H == 1) TRY(axbc_single_reach_sum(c));
    else CU(cudaMemsetAsync(&c->pc->reach_sum, 0, 8, c->stream));
    TRY(axbc_single_update(c, v0, p, g->reach + v0, nvisited, 1, H == 1));
    if (st) {
        cudaStream_t s = c->stream;
        CU(cudaMemcpyAsync(c->pc_host, c->pc, sizeof(PivotCounters), cudaMemcpyDeviceToHost, s));
        uint32_t reach_v0 = 0;
        CU(cudaMemcpyAsync(&reach_v0, g->reach + v0, 4, cudaMemcpyDeviceToHost, s));
        CU(cudaStreamSynchronize(s));
        st->nvisited = nvisited;
        st->all = (H == 1 ? (uint32_t)c->pc_host->reach_sum : 0u) + reach_v0;
        st->te = 2 * c->pc_host->newdeg;
        st->levels = level;
        st->pad = 0;
    }
    return AXBC_OK;
}
