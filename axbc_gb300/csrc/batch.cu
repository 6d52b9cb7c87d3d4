// Batched form: up to 64 pivots in one multi-source pass.  Lane s of a warp
// owns pivot s (and s + 32 in a pass of more than 32); every vertex carries one
// 32- or 64-bit mask per BFS level (bit s: the vertex is at that depth from
// pivot s), a `seen` mask, and per-pivot path counts / dependencies laid out
// [vertex][32 or 64] so a warp touches one 128-byte line per 32 pivots.
// Results equal those of the plain form bit for bit: path counts are integers,
// and each lane accumulates its dependency sum in the canonical order
// (32-position chunks summed as a tree in registers, chunks then spans left to
// right).
#include <algorithm>
#include <cstddef>
#include <vector>

#include "common.cuh"

#define BATCH_TPB 256

// K: 32-bit mask words per vertex.  K = 1: a pass of up to 32 pivots, lane s
// of a warp owns pivot s.  K = 2: up to 64 pivots, lane l owns pivots l and
// l + 32 (its two "halves"), masks are 64-bit, per-pivot rows hold 64 values
// and one adjacency entry and one mask load serve all 64 pivots.
template <int K> struct MaskOf;
template <> struct MaskOf<1> {
    typedef uint32_t T;
};
template <> struct MaskOf<2> {
    typedef unsigned long long T;
};

template <int K> __device__ __forceinline__ uint64_t row_base(uint64_t v) { return v * (uint64_t)(AXBC_W * K); }

// bit of this lane's pivot of half h (a 32-bit mask has only half 0)
__device__ __forceinline__ bool pbit(uint32_t m, int) { return (m >> lane_id()) & 1u; }
__device__ __forceinline__ bool pbit(unsigned long long m, int h)
{
    return (uint32_t)(m >> (32 * h)) >> lane_id() & 1u;
}
template <class M> __device__ __forceinline__ M lane_mask(int s) { return (M)1 << s; }

__device__ __forceinline__ uint32_t warp_or(uint32_t m) { return __reduce_or_sync(FULL_MASK, m); }
__device__ __forceinline__ unsigned long long warp_or(unsigned long long m)
{
    const uint32_t lo = __reduce_or_sync(FULL_MASK, (uint32_t)m);
    const uint32_t hi = __reduce_or_sync(FULL_MASK, (uint32_t)(m >> 32));
    return (unsigned long long)lo | ((unsigned long long)hi << 32);
}

// A warp stages the masks of a 32-position chunk in shared memory as K
// arrays of 32 words, one per 32-bit half (sg + 32 h), so that a half's
// consumer holds 32-bit words only.
template <int K> __device__ __forceinline__ typename MaskOf<K>::T staged_mask(const uint32_t *sg, int i)
{
    typedef typename MaskOf<K>::T M;
    if (K == 1) return (M)sg[i];
    return (M)((unsigned long long)sg[i] | ((unsigned long long)sg[32 + i] << 32));
}

// Stage the chunk's positions that have a parent (act: their lanes),
// compacted to slots 0..nh-1 in position order, and zero masks in slots
// nh..31, so that the consumer walks ceil(nh / 8) groups of 8 instead of every
// group holding a hit.  Returns nh.
template <int K, class M>
__device__ __forceinline__ int stage_compact(uint32_t *su, uint32_t *sg, uint32_t *sk, unsigned act, uint32_t v,
                                             M fm, uint32_t k)
{
    const unsigned lane = lane_id();
    const int nh = __popc(act);
    if (fm) {
        const int pos = __popc(act & ((1u << lane) - 1u));
        su[pos] = v;
        sg[pos] = (uint32_t)fm;
        if (K == 2) sg[32 + pos] = (uint32_t)((unsigned long long)fm >> 32);
        if (sk) sk[pos] = k;
    }
    if ((int)lane >= nh) {
        su[lane] = 0;
        sg[lane] = 0;
        if (K == 2) sg[32 + lane] = 0;
    }
    return nh;
}

// eight staged words of group g (16-byte shared loads)
__device__ __forceinline__ void load8u(const uint32_t *su, int g, uint32_t u[8])
{
    const uint4 *p = reinterpret_cast<const uint4 *>(su) + 2 * g;
    const uint4 a = p[0], b = p[1];
    u[0] = a.x, u[1] = a.y, u[2] = a.z, u[3] = a.w, u[4] = b.x, u[5] = b.y, u[6] = b.z, u[7] = b.w;
}

// resident blocks per SM the kernels are compiled for (their register
// budgets); the backward runs 32 pivots at a time at either width
#ifndef AXBC_PULL_MIN_BLOCKS
#define AXBC_PULL_MIN_BLOCKS 6
#endif
#ifndef AXBC_BWD_MIN_BLOCKS
#define AXBC_BWD_MIN_BLOCKS 8
#endif
#ifndef AXBC_PUSH_MIN_BLOCKS2
#define AXBC_PUSH_MIN_BLOCKS2 5
#endif
#ifndef AXBC_PULL_MIN_BLOCKS2
#define AXBC_PULL_MIN_BLOCKS2 4
#endif
#define PUSH_BLOCKS(K) ((K) == 1 ? 8 : AXBC_PUSH_MIN_BLOCKS2)
#define PULL_BLOCKS(K) ((K) == 1 ? AXBC_PULL_MIN_BLOCKS : AXBC_PULL_MIN_BLOCKS2)

// Per-level vertex lists: the vertices whose level-L mask is nonzero, appended
// by the forward kernels that set the mask.  A level whose list would exceed
// its capacity keeps counting but stops storing (count > cap: no list), and
// its consumers fall back to the degree-ordered task scan.
struct LevelLists {
    uint32_t *pool;
    uint32_t *start;  // per level: offset into pool
    uint32_t *count;  // per level: vertices appended
    uint32_t *cap;    // per level: capacity
    uint32_t *heavy;  // per level: listed vertices with more than AXBC_SPAN neighbours
};


// Clear the level masks first..last of the previous batch (levels 0 and 1
// are cleared with memsets): a level whose list was stored has nonzero
// entries only at its listed vertices; an overflowed level is cleared whole.
// The grid walks the levels in order, all blocks sharing each level.
template <int K>
__global__ void k_clean_levels(uint32_t *const *__restrict__ tab, const uint32_t *__restrict__ pool,
                               const uint32_t *__restrict__ lstart,
                               const uint32_t *__restrict__ lcount,
                               const uint32_t *__restrict__ lcap, uint64_t n, int first, int last)
{
    typedef typename MaskOf<K>::T M;
    const uint64_t tid = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
    const uint64_t nt = (uint64_t)gridDim.x * blockDim.x;
    for (int L = first; L <= last; L++) {
        M *f = reinterpret_cast<M *>(tab[L]);
        const uint32_t cnt = lcount[L];
        if (cnt <= lcap[L]) {
            const uint32_t *lst = pool + lstart[L];
            for (uint64_t i = tid; i < cnt; i += nt) f[lst[i]] = 0;
        } else {
            for (uint64_t i = tid; i < n; i += nt) f[i] = 0;
        }
    }
}

// roots: depth 0, sigma 1 (set_mlp_cuda, src/cuda_kernels.cu:862-876); one
// warp, lane l setting up pivots l + 32 h
template <int K>
__global__ void k_batch_init(BatchInfo *bi, int nsrc, int H, float *bc, uint32_t *fmask0_, uint32_t *seen_,
                             uint32_t *msigma, const uint32_t *__restrict__ col,
                             const uint32_t *__restrict__ rcol, unsigned long long m,
                             double push_factor, unsigned long long push_min,
                             unsigned long long *level_te,
                             unsigned long long *level_cnt, LevelLists ll, uint32_t pool_cap,
                             uint32_t list_max, const uint32_t *__restrict__ to_view)
{
    typedef typename MaskOf<K>::T M;
    M *fmask0 = reinterpret_cast<M *>(fmask0_), *seen = reinterpret_cast<M *>(seen_);
    const int l = threadIdx.x;
    // the roots arrive as vertex ids; the pass runs in the graph's view
    if (to_view) {
#pragma unroll
        for (int h = 0; h < K; h++)
            if (l + 32 * h < nsrc) bi->root[l + 32 * h] = to_view[bi->root[l + 32 * h]];
        __syncwarp();
    }
    if (l == 0) {
        bi->nsrc = nsrc;
        bi->srcmask = nsrc >= 64 ? ~0ull : ((1ull << nsrc) - 1ull);
        bi->applymask = bi->srcmask;
        bi->depth0mask = 0;
        bi->H = H;
        bi->cur = 0;
        bi->alive = 1;
        bi->lend = 0;
        bi->dmax = -1;
        bi->bd = -1;
        bi->push_factor = push_factor;
        bi->lvl_te = 0;
        bi->any_new = 0;
        bi->pool_short = 0;
    }
    unsigned long long fd = 0, rd = 0;
    uint32_t nroots = 0, heavy_roots = 0;
    const uint32_t rt0 = l < nsrc ? bi->root[l] : 0xffffffffu;
#pragma unroll
    for (int h = 0; h < K; h++) {
        const int s = l + 32 * h;
        bi->Ls[s] = 0;
        bi->lvl_new[s] = 0;
        bi->lane_bc[s] = bc;
        if (s < nsrc) {
            const uint32_t v = bi->root[s];
            atomicOr(&fmask0[v], lane_mask<M>(s));
            atomicOr(&seen[v], lane_mask<M>(s));
            msigma[row_base<K>(v) + s] = 1;
            bi->nvis[s] = 1;
            bi->rsum[s] = 0;
            bi->te[s] = col[v + 1] - col[v];
            fd += col[v + 1] - col[v];
            rd += rcol[v + 1] - rcol[v];
        } else {
            bi->nvis[s] = 0;
            bi->rsum[s] = 0;
            bi->te[s] = 0;
        }
        // the level-0 list: each root once (lanes of different runs may share one)
        const uint32_t rt = s < nsrc ? bi->root[s] : 0xffffffffu;
        const uint32_t same = __match_any_sync(FULL_MASK, rt);
        bool first = s < nsrc && (__ffs(same) - 1) == l;
        if (h == 1) {
            bool dup = false;
            for (int j = 0; j < 32; j++) dup |= __shfl_sync(FULL_MASK, rt0, j) == rt;
            first = first && !dup;
        }
        const uint32_t firsts = __ballot_sync(FULL_MASK, first);
        if (first) ll.pool[nroots + __popc(firsts & ((1u << l) - 1u))] = rt;
        nroots += __popc(firsts);
        heavy_roots += __popc(__ballot_sync(FULL_MASK, first && col[rt + 1] - col[rt] > AXBC_SPAN));
    }
    for (int o = 16; o; o >>= 1) {
        fd += __shfl_xor_sync(FULL_MASK, fd, o);
        rd += __shfl_xor_sync(FULL_MASK, rd, o);
    }
    if (l == 0) {
        ll.heavy[0] = heavy_roots;
        // a vertex counts as unvisited until every pivot has seen it: with one
        // pivot its root is fully seen at once
        const unsigned long long unvis = nsrc == 1 ? m - rd : m;
        bi->front_deg = 0;
        bi->unvis_deg = unvis;
        bi->unvis_dec = 0;
        bi->push_min = push_min;
        bi->push_next = (double)fd * push_factor < (double)unvis || fd < push_min;
        level_te[0] = fd;
        level_cnt[0] = nsrc;
        ll.start[0] = 0;
        ll.count[0] = nroots;
        ll.cap[0] = nroots;
        ll.start[1] = nroots;
        ll.cap[1] = min(list_max, pool_cap - nroots);
    }
}

// ---------------------------------------------------------- task scheduling
// Work units handed out by an atomic counter: units [0, nhi) are the span
// items of heavy vertices (largest first), the remaining units cover four
// light tasks each (light tasks: degree-ordered groups of <= 32 vertices with
// about one span of adjacency).
#define LIGHT_PER_UNIT 4

__device__ __forceinline__ uint32_t grab_unit(uint32_t *ctr)
{
    uint32_t t = 0;
    if (lane_id() == 0) t = atomicAdd(ctr, 1u);
    return __shfl_sync(FULL_MASK, t, 0);
}

// A level with fewer work units than the grid has warps lets only as many
// warps as units reach the counter: ~10^4 warps contending for one address
// would cost tens of microseconds on a small level.
__device__ __forceinline__ uint32_t warp_global()
{
    return (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
}

__host__ __device__ __forceinline__ uint64_t n_units(const Adj &a)
{
    return a.n_heavy_items + (a.n_ltask + LIGHT_PER_UNIT - 1) / LIGHT_PER_UNIT;
}

__device__ __forceinline__ void list_append(const LevelLists &ll, int L, bool isnew, uint32_t v)
{
    const unsigned lane = lane_id();
    const unsigned m = __ballot_sync(FULL_MASK, isnew);
    if (!m) return;
    const int leader = __ffs(m) - 1;
    uint32_t base = 0;
    if ((int)lane == leader) base = atomicAdd(&ll.count[L], (uint32_t)__popc(m));
    base = __shfl_sync(FULL_MASK, base, leader);
    const uint32_t idx = base + __popc(m & ((1u << lane) - 1u));
    if (isnew && idx < ll.cap[L]) ll.pool[ll.start[L] + idx] = v;
}

// List entries per work unit: 32, or fewer when the list is too short to give
// every resident warp a unit (a short list of high-degree vertices would
// otherwise sit on a few warps).
__device__ __forceinline__ uint32_t list_unit(uint32_t lcnt)
{
    const uint32_t nwarps = gridDim.x * (blockDim.x / 32);
    return max(1u, min(32u, lcnt / nwarps));
}

// the stored list of level L, or nullptr when the level overflowed its capacity
__device__ __forceinline__ const uint32_t *level_list(const LevelLists &ll, int L, uint32_t &cnt)
{
    cnt = ll.count[L];
    if (cnt > ll.cap[L]) return nullptr;
    return ll.pool + ll.start[L];
}

// Forward level L, push from the vertices of depth L-1: for each neighbour u
// and each pivot s with v at depth L-1 and u unseen, sigma_s[u] += sigma_s[v]
// and bit s joins u's level-L mask.  Atomics are fire-and-forget reductions.
template <int K, class WC>
__device__ __forceinline__ void push_span(const Adj &a, uint32_t v, typename MaskOf<K>::T f, uint32_t b0,
                                          uint32_t b1, const typename MaskOf<K>::T *__restrict__ seen,
                                          typename MaskOf<K>::T *fcur, uint32_t *msigma,
                                          const LevelLists &ll, int L, WC &wc)
{
    typedef typename MaskOf<K>::T M;
    const unsigned lane = lane_id();
    uint32_t sig[K];
#pragma unroll
    for (int h = 0; h < K; h++) {
        sig[h] = pbit(f, h) ? msigma[row_base<K>(v) + 32 * h + lane] : 0u;
        if (pbit(f, h)) wc.add(WC_BYTES, 4);
    }
    for (uint32_t base = b0; base < b1; base += 32) {
        const uint32_t e = base + lane;
        uint32_t u = 0;
        M nm = 0;
        if (e < b1) {
            u = a.row[e];
            nm = f & ~seen[u];
            wc.add(WC_ENTRIES, 1);
            wc.add(WC_BYTES, 4 + 4 * K);  // adjacency entry, seen mask
        }
        const M old = nm ? atomicOr(&fcur[u], nm) : (M)1;
        if (nm) wc.add(WC_BYTES, old == 0 ? 4 + 4 * K : 4 * K);  // level mask, list entry
        list_append(ll, L, old == 0, u);
        unsigned act = __ballot_sync(FULL_MASK, nm != 0);
        while (act) {
            const int j = __ffs(act) - 1;
            act &= act - 1;
            const uint32_t uj = __shfl_sync(FULL_MASK, u, j);
            const M mj = __shfl_sync(FULL_MASK, nm, j);
#pragma unroll
            for (int h = 0; h < K; h++)
                if (pbit(mj, h)) {
                    atomicAdd(&msigma[row_base<K>(uj) + 32 * h + lane], sig[h]);
                    wc.add(WC_PAIRS, 1);
                    wc.add(WC_BYTES, 4);
                }
        }
    }
}

// Push from up to 32 light frontier vertices at once, one per lane (f_l = 0:
// none), edge-parallel: the warp walks the concatenation of their adjacency
// lists 32 positions at a time, so a chunk of low-degree vertices costs one
// pass instead of one pass per vertex.  Lane e finds its vertex by a binary
// search over the inclusive degree prefix held across the lanes.
template <int K, class WC>
__device__ __forceinline__ void push_light32(const Adj &a, uint32_t v_l, typename MaskOf<K>::T f_l,
                                             const typename MaskOf<K>::T *__restrict__ seen,
                                             typename MaskOf<K>::T *fcur, uint32_t *msigma,
                                             const LevelLists &ll, int L, WC &wc)
{
    typedef typename MaskOf<K>::T M;
    const unsigned lane = lane_id();
    uint32_t b = 0, d = 0;
    if (f_l) {
        b = a.col[v_l];
        d = a.col[v_l + 1] - b;
        wc.add(WC_BYTES, 8);  // adjacency bounds
    }
    uint32_t inc = d;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const uint32_t t = __shfl_up_sync(FULL_MASK, inc, o);
        if ((int)lane >= o) inc += t;
    }
    const uint32_t total = __shfl_sync(FULL_MASK, inc, 31);
    const uint32_t shift = b - (inc - d);  // position of concatenated index e: shift_k + e
    for (uint32_t base = 0; base < total; base += 32) {
        const uint32_t e = base + lane;
        uint32_t k = 0;  // lanes whose inclusive prefix is <= e
#pragma unroll
        for (int step = 16; step; step >>= 1)
            if (__shfl_sync(FULL_MASK, inc, k + step - 1) <= e) k += step;
        const uint32_t pk = __shfl_sync(FULL_MASK, shift, k) + e;
        const M fk = __shfl_sync(FULL_MASK, f_l, k);
        uint32_t u = 0;
        M nm = 0;
        if (e < total) {
            u = a.row[pk];
            nm = fk & ~seen[u];
            wc.add(WC_ENTRIES, 1);
            wc.add(WC_BYTES, 4 + 4 * K);  // adjacency entry, seen mask
        }
        const M old = nm ? atomicOr(&fcur[u], nm) : (M)1;
        if (nm) wc.add(WC_BYTES, old == 0 ? 4 + 4 * K : 4 * K);  // level mask, list entry
        list_append(ll, L, old == 0, u);
        unsigned act = __ballot_sync(FULL_MASK, nm != 0);
        while (act) {
            // up to 4 edges: gather the parents' sigma rows, then add
            uint32_t uu[4], sg[4][K];
            M mm[4];
#pragma unroll
            for (int q = 0; q < 4; q++) {
                const int j = act ? __ffs(act) - 1 : 0;
                const bool ok = act != 0;
                act &= act - 1;
                uu[q] = __shfl_sync(FULL_MASK, u, j);
                const M mj = __shfl_sync(FULL_MASK, nm, j);
                mm[q] = ok ? mj : (M)0;
                const uint32_t vj = __shfl_sync(FULL_MASK, v_l, __shfl_sync(FULL_MASK, k, j));
#pragma unroll
                for (int h = 0; h < K; h++)
                    sg[q][h] = pbit(mm[q], h) ? msigma[row_base<K>(vj) + 32 * h + lane] : 0u;
            }
#pragma unroll
            for (int q = 0; q < 4; q++)
#pragma unroll
                for (int h = 0; h < K; h++)
                    if (pbit(mm[q], h)) {
                        atomicAdd(&msigma[row_base<K>(uu[q]) + 32 * h + lane], sg[q][h]);
                        wc.add(WC_GATHERS, 1);
                        wc.add(WC_PAIRS, 1);
                        wc.add(WC_BYTES, 8);  // parent's path count, child's sum
                    }
        }
    }
}

template <int K, class WC>
__device__ __forceinline__ void fwd_push_body(const Adj &a, const typename MaskOf<K>::T *__restrict__ fprev,
                                              typename MaskOf<K>::T *fcur,
                                              const typename MaskOf<K>::T *__restrict__ seen,
                                              uint32_t *msigma, uint32_t *ctr, const LevelLists &ll,
                                              int L, WC &wc)
{
    typedef typename MaskOf<K>::T M;
    const unsigned lane = lane_id();
    uint32_t lcnt = 0;
    const uint32_t *lst = level_list(ll, L - 1, lcnt);  // the frontier, when stored
    // heavy span items only when a heavy vertex is in the frontier
    const uint64_t nhi = lst && ll.heavy[L - 1] == 0 ? 0 : a.n_heavy_items;
    const uint32_t ent = list_unit(lcnt);
    const uint64_t nu = lst ? nhi + (lcnt + ent - 1) / ent : n_units(a);
    if (warp_global() >= nu) return;  // fewer units than warps: no contention
    for (;;) {
        const uint32_t t = grab_unit(ctr);
        if (t >= nu) break;
        if (t < nhi) {
            const uint32_t v = a.hitem_v[t];
            const M f = fprev[v];
            if (lane == 0) wc.add(WC_BYTES, 4 * K);
            if (!f) continue;
            const uint32_t b0 = a.col[v] + a.hitem_k[t] * AXBC_SPAN;
            push_span<K>(a, v, f, b0, min(a.col[v + 1], b0 + AXBC_SPAN), seen, fcur, msigma, ll, L, wc);
            continue;
        }
        if (lst) {
            const uint32_t i = (uint32_t)(t - nhi) * ent + lane;
            uint32_t v_l = 0;
            M f_l = 0;
            if (lane < ent && i < lcnt) {
                v_l = lst[i];
                if (a.col[v_l + 1] - a.col[v_l] <= AXBC_SPAN) f_l = fprev[v_l];
                wc.add(WC_BYTES, 4 + 4 * K);  // list entry, level mask
            }
            push_light32<K>(a, v_l, f_l, seen, fcur, msigma, ll, L, wc);
            continue;
        }
        const uint64_t l0 = (uint64_t)(t - nhi) * LIGHT_PER_UNIT;
        for (uint64_t lt = l0; lt < l0 + LIGHT_PER_UNIT && lt < a.n_ltask; lt++) {
            const uint32_t beg = a.ltask[lt], cnt = a.ltask[lt + 1] - beg;
            uint32_t v_l = 0;
            M f_l = 0;
            if (lane < cnt) {
                v_l = a.order[beg + lane];
                f_l = fprev[v_l];
                wc.add(WC_BYTES, 4 * K);  // level mask
            }
            push_light32<K>(a, v_l, f_l, seen, fcur, msigma, ll, L, wc);
        }
    }
}

// Forward level L, pull into vertex u for the pivots `ns` that have not seen
// it: sum sigma_s over every in-neighbour at depth L-1 from pivot s (u32 sums:
// any order gives the same bits).  The positions of a 32-wide chunk that have
// a parent are staged in shared memory, compacted; each group of 8 issues its
// gathers (8 per half) before any is consumed.
template <int K, class WC>
__device__ __forceinline__ typename MaskOf<K>::T pull_span(const Adj &rv, typename MaskOf<K>::T ns, uint32_t b0,
                                                           uint32_t b1,
                                                           const typename MaskOf<K>::T *__restrict__ fprev,
                                                           const uint32_t *__restrict__ msigma, uint32_t *su,
                                                           uint32_t *sg, uint32_t acc[K], WC &wc)
{
    typedef typename MaskOf<K>::T M;
    const unsigned lane = lane_id();
    M found = 0;
#pragma unroll
    for (int h = 0; h < K; h++) acc[h] = 0;
    // the next chunk's adjacency entries load while this chunk is consumed
    uint32_t vn = b0 + lane < b1 ? rv.row[b0 + lane] : 0u;
    for (uint32_t base = b0; base < b1; base += 32) {
        const uint32_t e = base + lane;
        const uint32_t v = vn;
        vn = e + 32 < b1 ? rv.row[e + 32] : 0u;
        const M fm = e < b1 ? fprev[v] & ns : (M)0;
        if (e < b1) {
            wc.add(WC_ENTRIES, 1);
            wc.add(WC_GATHERS, __popcll((unsigned long long)fm));
            wc.add(WC_BYTES, 4 + 4 * K + 4 * __popcll((unsigned long long)fm));  // entry, mask, parents' counts
        }
        const unsigned act = __ballot_sync(FULL_MASK, fm != 0);
        if (!act) continue;
        found |= warp_or(fm);
        const int nh = stage_compact<K>(su, sg, (uint32_t *)nullptr, act, v, fm, 0u);
        __syncwarp();
#pragma unroll 1
        for (int g = 0; 8 * g < nh; g++) {
            uint32_t u[8];
            load8u(su, g, u);
#pragma unroll
            for (int h = 0; h < K; h++) {
                uint32_t m[8], x[8];
                load8u(sg + 32 * h, g, m);
#pragma unroll
                for (int q = 0; q < 8; q++)
                    x[q] = ((m[q] >> lane) & 1u) ? msigma[row_base<K>(u[q]) + 32 * h + lane] : 0u;
#pragma unroll
                for (int q = 0; q < 8; q++) acc[h] += x[q];
            }
        }
        __syncwarp();
    }
    return found;
}

// Pull into up to 32 light vertices at once, one per lane (pivots ns_l; 0:
// none), edge-parallel over the concatenation of their in-adjacency lists:
// lane e finds its vertex by a binary search over the inclusive degree prefix
// held across the lanes.  Positions arrive grouped by vertex (compaction keeps
// their order), so one running sum per lane (pivot) is written out whenever
// the vertex changes.  Returns the discovered mask of the lane's own vertex.
template <int K, class WC>
__device__ __forceinline__ typename MaskOf<K>::T pull_light32(const Adj &rv, uint32_t u_l,
                                                              typename MaskOf<K>::T ns_l,
                                                              const typename MaskOf<K>::T *__restrict__ fprev,
                                                              uint32_t *msigma, uint32_t *su,
                                                              uint32_t *sg, uint32_t *sk, WC &wc)
{
    typedef typename MaskOf<K>::T M;
    const unsigned lane = lane_id();
    uint32_t b = 0, d = 0;
    if (ns_l) {
        b = rv.col[u_l];
        d = rv.col[u_l + 1] - b;
        wc.add(WC_BYTES, 8);  // adjacency bounds
    }
    uint32_t inc = d;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const uint32_t t = __shfl_up_sync(FULL_MASK, inc, o);
        if ((int)lane >= o) inc += t;
    }
    const uint32_t total = __shfl_sync(FULL_MASK, inc, 31);
    const uint32_t shift = b - (inc - d);  // position of concatenated index e: shift_k + e
    M mine = 0, fo = 0;
    uint32_t acc[K];
#pragma unroll
    for (int h = 0; h < K; h++) acc[h] = 0;
    int cur = -1;
    // the finished running sums of vertex `cur` go to its row
    auto flush = [&]() {
        const uint32_t uc = __shfl_sync(FULL_MASK, u_l, cur);
#pragma unroll
        for (int h = 0; h < K; h++)
            if (pbit(fo, h)) msigma[row_base<K>(uc) + 32 * h + lane] = acc[h];
        if ((int)lane == cur) mine = fo;
    };
    for (uint32_t base = 0; base < total; base += 32) {
        const uint32_t e = base + lane;
        uint32_t k = 0;
#pragma unroll
        for (int step = 16; step; step >>= 1)
            if (__shfl_sync(FULL_MASK, inc, k + step - 1) <= e) k += step;
        const uint32_t pk = __shfl_sync(FULL_MASK, shift, k) + e;
        const M nk = __shfl_sync(FULL_MASK, ns_l, k);
        uint32_t v = 0;
        M fm = 0;
        if (e < total) {
            v = rv.row[pk];
            fm = fprev[v] & nk;
            wc.add(WC_ENTRIES, 1);
            wc.add(WC_GATHERS, __popcll((unsigned long long)fm));
            wc.add(WC_BYTES, 4 + 4 * K + 4 * __popcll((unsigned long long)fm));  // entry, mask, parents' counts
        }
        const unsigned act = __ballot_sync(FULL_MASK, fm != 0);
        if (!act) continue;
        const int nh = stage_compact<K>(su, sg, sk, act, v, fm, k);
        __syncwarp();
#pragma unroll 1
        for (int g = 0; 8 * g < nh; g++) {
            uint32_t u4[8];
            load8u(su, g, u4);
            uint32_t x[K][8];
            M mor = 0;
#pragma unroll
            for (int h = 0; h < K; h++) {
                uint32_t m4[8], mh = 0;
                load8u(sg + 32 * h, g, m4);
#pragma unroll
                for (int q = 0; q < 8; q++) {
                    x[h][q] = ((m4[q] >> lane) & 1u) ? msigma[row_base<K>(u4[q]) + 32 * h + lane] : 0u;
                    mh |= m4[q];
                }
                mor |= (M)((unsigned long long)mh << (32 * h));
            }
            const int k0 = (int)sk[8 * g], k7 = (int)sk[min(8 * g + 7, nh - 1)];
            if (k0 == k7) {
                // all eight positions belong to one vertex (k is nondecreasing)
                if (k0 != cur) {
                    if (cur >= 0) flush();
                    cur = k0;
#pragma unroll
                    for (int h = 0; h < K; h++) acc[h] = 0;
                    fo = 0;
                }
#pragma unroll
                for (int h = 0; h < K; h++)
                    acc[h] += ((x[h][0] + x[h][1]) + (x[h][2] + x[h][3])) + ((x[h][4] + x[h][5]) + (x[h][6] + x[h][7]));
                fo |= mor;
                continue;
            }
#pragma unroll
            for (int q = 0; q < 8; q++) {
                const M mq = staged_mask<K>(sg, 8 * g + q);
                if (!mq) continue;
                const int kq = (int)sk[8 * g + q];
                if (kq != cur) {
                    if (cur >= 0) flush();
                    cur = kq;
#pragma unroll
                    for (int h = 0; h < K; h++) acc[h] = 0;
                    fo = 0;
                }
#pragma unroll
                for (int h = 0; h < K; h++) acc[h] += x[h][q];
                fo |= mq;
            }
        }
        __syncwarp();
    }
    if (cur >= 0) flush();
    return mine;
}

template <int K, class WC>
__device__ __forceinline__ void fwd_pull_body(const Adj &rv, typename MaskOf<K>::T srcmask,
                                              const typename MaskOf<K>::T *__restrict__ fprev,
                                              typename MaskOf<K>::T *fcur,
                                              const typename MaskOf<K>::T *__restrict__ seen, uint32_t *msigma,
                                              uint32_t *ctr, uint32_t *su, uint32_t *sg,
                                              uint32_t *sk, const LevelLists &ll, int L, WC &wc)
{
    typedef typename MaskOf<K>::T M;
    const unsigned lane = lane_id();
    const uint64_t nhi = rv.n_heavy_items, nu = n_units(rv);
    if (warp_global() >= nu) return;  // fewer units than warps: no contention
    for (;;) {
        const uint32_t t = grab_unit(ctr);
        if (t >= nu) break;
        if (t < nhi) {
            const uint32_t u = rv.hitem_v[t];
            const M ns = srcmask & ~seen[u];
            if (lane == 0) wc.add(WC_BYTES, 4 * K);  // seen mask
            if (!ns) continue;
            const uint32_t b0 = rv.col[u] + rv.hitem_k[t] * AXBC_SPAN;
            uint32_t acc[K];
            const M nm = pull_span<K>(rv, ns, b0, min(rv.col[u + 1], b0 + AXBC_SPAN), fprev, msigma, su, sg,
                                      acc, wc);
#pragma unroll
            for (int h = 0; h < K; h++)
                if (pbit(nm, h)) {
                    atomicAdd(&msigma[row_base<K>(u) + 32 * h + lane], acc[h]);
                    wc.add(WC_PAIRS, 1);
                    wc.add(WC_BYTES, 4);
                }
            bool first = false;
            if (lane == 0 && nm) first = atomicOr(&fcur[u], nm) == 0;
            if (lane == 0 && nm) wc.add(WC_BYTES, first ? 4 + 4 * K : 4 * K);  // level mask, list entry
            list_append(ll, L, first, u);
            continue;
        }
        const uint64_t l0 = (uint64_t)(t - nhi) * LIGHT_PER_UNIT;
        for (uint64_t lt = l0; lt < l0 + LIGHT_PER_UNIT && lt < rv.n_ltask; lt++) {
            const uint32_t beg = rv.ltask[lt], cnt = rv.ltask[lt + 1] - beg;
            uint32_t u_l = 0;
            M ns_l = 0;
            if (lane < cnt) {
                u_l = rv.order[beg + lane];
                ns_l = srcmask & ~seen[u_l];
                wc.add(WC_BYTES, 4 * K);  // seen mask
            }
            const M mine = pull_light32<K>(rv, u_l, ns_l, fprev, msigma, su, sg, sk, wc);
            if (mine) {
                fcur[u_l] = mine;
                wc.add(WC_PAIRS, __popcll((unsigned long long)mine));
                wc.add(WC_BYTES, 4 + 4 * K + 4 * __popcll((unsigned long long)mine));  // mask, list, counts
            }
            list_append(ll, L, mine != 0, u_l);
        }
    }
}

// One forward level, device-driven: the level is bi->cur + 1 and the direction
// bi->push_next (set by the previous k_level_advance).  Both direction kernels
// are launched every level; the one not chosen returns at once, as both do
// once a level discovered nothing.  CNT: the counting build (work counts into
// wc[KP_FWD_PUSH / KP_FWD_PULL]).
template <int K, bool CNT>
__global__ void __launch_bounds__(BATCH_TPB, PUSH_BLOCKS(K)) k_fwd_push_step(Adj a, const BatchInfo *__restrict__ bi,
                                                             uint32_t *const *__restrict__ tab,
                                                             const uint32_t *__restrict__ seen,
                                                             uint32_t *msigma, uint32_t *ctrs,
                                                             LevelLists ll, unsigned long long *wc)
{
    typedef typename MaskOf<K>::T M;
    if (!bi->alive || !bi->push_next) return;
    const int L = bi->cur + 1;
    WorkCount<CNT> cnt;
    fwd_push_body<K>(a, reinterpret_cast<const M *>(tab[L - 1]), reinterpret_cast<M *>(tab[L]),
                     reinterpret_cast<const M *>(seen), msigma, ctrs + 2 * L, ll, L, cnt);
    cnt.flush(wc);
}

template <int K, bool CNT>
__global__ void __launch_bounds__(BATCH_TPB, PULL_BLOCKS(K)) k_fwd_pull_step(Adj rv, const BatchInfo *__restrict__ bi,
                                                             uint32_t *const *__restrict__ tab,
                                                             const uint32_t *__restrict__ seen,
                                                             uint32_t *msigma, uint32_t *ctrs,
                                                             LevelLists ll, unsigned long long *wc)
{
    typedef typename MaskOf<K>::T M;
    __shared__ __align__(16) uint32_t s_u[BATCH_TPB];
    __shared__ __align__(16) uint32_t s_g[BATCH_TPB * K];
    __shared__ uint32_t s_k[BATCH_TPB];
    if (!bi->alive || bi->push_next) return;
    const int L = bi->cur + 1;
    const unsigned w0 = threadIdx.x & ~31u;
    WorkCount<CNT> cnt;
    fwd_pull_body<K>(rv, (M)bi->srcmask, reinterpret_cast<const M *>(tab[L - 1]), reinterpret_cast<M *>(tab[L]),
                     reinterpret_cast<const M *>(seen), msigma, ctrs + 2 * L, s_u + w0, s_g + w0 * K, s_k + w0,
                     ll, L, cnt);
    cnt.flush(wc);
}

// After level L = bi->cur + 1: fold the level mask into `seen` and count, per
// pivot, the vertices reached, their degree sum and their reach sum; subtract
// from the unvisited-edge total the in-degrees of vertices now seen by every
// pivot.  Visits only level L's list when stored.
template <class M>
__device__ __forceinline__ void stats_vertex(uint64_t u, M srcmask, const M *__restrict__ fcur, M *seen,
                                             const uint32_t *__restrict__ col,
                                             const uint32_t *__restrict__ rcol,
                                             const uint32_t *__restrict__ reach, M &nm,
                                             uint32_t &d, uint32_t &r, unsigned long long &fdeg,
                                             unsigned long long &udec, bool &any)
{
    nm = fcur[u];
    if (!nm) return;
    any = true;
    const M sn = seen[u];
    const M sn2 = sn | nm;
    seen[u] = sn2;
    d = col[u + 1] - col[u];
    r = reach[u];
    fdeg += d;
    if ((sn & srcmask) != srcmask && (sn2 & srcmask) == srcmask) udec += rcol[u + 1] - rcol[u];
}

template <int K>
__device__ __forceinline__ void stats_body(uint64_t n, BatchInfo *bi, int L, typename MaskOf<K>::T srcmask,
                                           const typename MaskOf<K>::T *__restrict__ fcur,
                                           typename MaskOf<K>::T *seen, const uint32_t *__restrict__ col,
                                           const uint32_t *__restrict__ rcol,
                                           const uint32_t *__restrict__ reach, const LevelLists &ll)
{
    typedef typename MaskOf<K>::T M;
    const unsigned lane = lane_id();
    const uint64_t tid = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
    const uint64_t nthreads = (uint64_t)gridDim.x * blockDim.x;
    uint32_t lcnt = 0;
    const uint32_t *lst = level_list(ll, L, lcnt);
    const uint64_t items = lst ? lcnt : n;
    const uint64_t nblk = (items + 31) / 32;
    const uint64_t nw = nthreads / 32;
    unsigned long long cnt[K], te[K], rs[K];
#pragma unroll
    for (int h = 0; h < K; h++) cnt[h] = te[h] = rs[h] = 0;
    unsigned long long fdeg = 0, udec = 0, tsum = 0;
    uint32_t hv = 0;  // heavy vertices of the level (their span items are scanned)
    bool any = false;
    for (uint64_t t = tid / 32; t < nblk; t += nw) {
        const uint64_t i = t * 32 + lane;
        M nm = 0;
        uint32_t d = 0, r = 0;
        if (i < items) {
            const uint64_t u = lst ? lst[i] : i;
            stats_vertex<M>(u, srcmask, fcur, seen, col, rcol, reach, nm, d, r, fdeg, udec, any);
            if (nm && d > AXBC_SPAN) hv++;
            tsum += (unsigned long long)d * __popcll((unsigned long long)nm);
        }
        unsigned act = __ballot_sync(FULL_MASK, nm != 0);
        while (act) {
            const int j = __ffs(act) - 1;
            act &= act - 1;
            const M mj = __shfl_sync(FULL_MASK, nm, j);
            const uint32_t dj = __shfl_sync(FULL_MASK, d, j);
            const uint32_t rj = __shfl_sync(FULL_MASK, r, j);
#pragma unroll
            for (int h = 0; h < K; h++)
                if (pbit(mj, h)) {
                    cnt[h]++;
                    te[h] += dj;
                    rs[h] += rj;
                }
        }
    }
    {
        uint32_t hsum = hv;
        for (int o = 16; o; o >>= 1) {
            tsum += __shfl_xor_sync(FULL_MASK, tsum, o);
            hsum += __shfl_xor_sync(FULL_MASK, hsum, o);
        }
        if (lane == 0 && tsum) atomicAdd(&bi->lvl_te, tsum);
        if (lane == 0 && hsum) atomicAdd(&ll.heavy[L], hsum);
    }
#pragma unroll
    for (int h = 0; h < K; h++)
        if (cnt[h]) {
            const int s = lane + 32 * h;
            atomicAdd(&bi->lvl_new[s], cnt[h]);
            atomicAdd(&bi->nvis[s], cnt[h]);
            atomicAdd(&bi->te[s], te[h]);
            atomicAdd(&bi->rsum[s], rs[h]);
        }
    for (int o = 16; o; o >>= 1) {
        fdeg += __shfl_xor_sync(FULL_MASK, fdeg, o);
        udec += __shfl_xor_sync(FULL_MASK, udec, o);
    }
    any = __any_sync(FULL_MASK, any);
    if (lane == 0) {
        if (fdeg) atomicAdd(&bi->front_deg, fdeg);
        if (udec) atomicAdd(&bi->unvis_dec, udec);
        if (any) atomicOr(&bi->any_new, 1u);
    }
}

template <int K>
__global__ void __launch_bounds__(BATCH_TPB) k_stats_step(uint64_t n, BatchInfo *bi,
                                                          uint32_t *const *__restrict__ tab,
                                                          uint32_t *seen,
                                                          const uint32_t *__restrict__ col,
                                                          const uint32_t *__restrict__ rcol,
                                                          const uint32_t *__restrict__ reach,
                                                          LevelLists ll)
{
    typedef typename MaskOf<K>::T M;
    if (!bi->alive) return;
    const int L = bi->cur + 1;
    stats_body<K>(n, bi, L, (M)bi->srcmask, reinterpret_cast<const M *>(tab[L]), reinterpret_cast<M *>(seen),
                  col, rcol, reach, ll);
}

// Close forward level L = bi->cur + 1 (one warp, lane l for pivots l + 32 h):
// per-pivot termination, the per-level totals, the direction of the next
// level, and -- once nothing was discovered -- the deepest depth and the
// depth-0 pivots of the backward pass.
template <int K>
__device__ __forceinline__ void level_advance_warp(BatchInfo *bi, unsigned long long *level_te,
                                                   unsigned long long *level_cnt, int32_t *level_mode,
                                                   const LevelLists &ll, uint32_t pool_cap,
                                                   uint32_t list_max)
{
    const unsigned l = lane_id();
    const int L = bi->cur + 1;
    const uint32_t nsrc = bi->nsrc;
    unsigned long long cnt = 0, d0 = 0;
#pragma unroll
    for (int h = 0; h < K; h++) {
        const uint32_t s = l + 32 * h;
        const unsigned long long nw = s < nsrc ? bi->lvl_new[s] : 0ull;
        if (s < nsrc && bi->Ls[s] == 0 && nw == 0) bi->Ls[s] = L;
        cnt += nw;
        const bool two = s < nsrc && bi->Ls[s] == 2;
        d0 |= (unsigned long long)__ballot_sync(FULL_MASK, two) << (32 * h);
    }
    for (int o = 16; o; o >>= 1) cnt += __shfl_xor_sync(FULL_MASK, cnt, o);
    __syncwarp();
    if (l == 0) {
        level_te[L] = bi->lvl_te;
        level_cnt[L] = cnt;
        level_mode[L] = bi->push_next;
        bi->unvis_deg -= bi->unvis_dec;
        bi->unvis_dec = 0;
        // push from a frontier whose degree sum is small against the graph:
        // a pull would scan every vertex some pivot has not seen
        const bool push = (double)bi->front_deg * bi->push_factor < (double)bi->unvis_deg ||
                          bi->front_deg < bi->push_min;
        // where level L+1's list goes and how long it may grow
        const uint32_t used = ll.start[L] + (ll.count[L] <= ll.cap[L] ? ll.count[L] : 0u);
        ll.start[L + 1] = used;
        ll.cap[L + 1] = min(list_max, pool_cap - min(pool_cap, used));
        if (pool_cap - min(pool_cap, used) < list_max) bi->pool_short = 1;
        if (!bi->any_new) {
            bi->alive = 0;
            bi->lend = L;
            bi->dmax = L - 1;
            bi->bd = L - 1;
            bi->depth0mask = d0;
        }
        bi->push_next = push;
        bi->cur = L;
        bi->lvl_te = 0;
        bi->front_deg = 0;
        bi->any_new = 0;
    }
#pragma unroll
    for (int h = 0; h < K; h++) bi->lvl_new[l + 32 * h] = 0;
}

template <int K>
__global__ void k_level_advance(BatchInfo *bi, unsigned long long *level_te,
                                unsigned long long *level_cnt, int32_t *level_mode,
                                LevelLists ll, uint32_t pool_cap, uint32_t list_max)
{
    if (!bi->alive) return;
    level_advance_warp<K>(bi, level_te, level_cnt, level_mode, ll, pool_cap, list_max);
}

// The backward pass runs one 32-pivot half of a pass at a time (hh = 0, or 0
// and 1 for a 64-pivot pass): lane l owns pivot l + 32 hh.  The functions
// below see the half through offset pointers: level masks as 32-bit words at
// stride K (word hh of each vertex's mask, little-endian), rows and span
// partials shifted by 32 hh columns.  A half has the register footprint of a
// 32-pivot pass, which keeps 8 blocks per SM resident for this latency-bound
// kernel.
template <int K> __device__ __forceinline__ uint32_t half_of(typename MaskOf<K>::T m, int hh)
{
    return (uint32_t)((unsigned long long)m >> (32 * hh));
}

// Sum of the 8 staged successor terms of group g as a balanced tree (pairs
// differing in the lowest position bit first).  mq_l points at the lane's
// column of row 0.
template <int K>
__device__ __forceinline__ float tree8(const uint32_t *su, const uint32_t *sg, int g,
                                       const float *__restrict__ mq_l, float sv)
{
    uint32_t u[8], m[8];
    load8u(su, g, u);
    load8u(sg, g, m);
    const unsigned lane = lane_id();
    float t[8];
#pragma unroll
    for (int jj = 0; jj < 8; jj++) {
        const bool hit = (m[jj] >> lane) & 1u;
        const float q = hit ? mq_l[(uint64_t)u[jj] * (AXBC_W * K)] : 0.0f;
        t[jj] = hit ? __fmul_rn(q, sv) : 0.0f;
    }
    const float a = __fadd_rn(__fadd_rn(t[0], t[1]), __fadd_rn(t[2], t[3]));
    const float b = __fadd_rn(__fadd_rn(t[4], t[5]), __fadd_rn(t[6], t[7]));
    return __fadd_rn(a, b);
}

// Canonical dependency sum of vertex v over adjacency positions [b0,b1) for
// the half's pivots in f.  q[u][s] = (delta_s[u] + 1) / sigma_s[u] was stored
// when u's dependency was final, so a successor term is q * sigma_s[v], bit for
// bit the reference's ((delta + 1) / sigma[r]) * sigma[c].  The 32 positions
// of a chunk form four 8-position subtrees of the canonical tree; a subtree
// without successors sums to +0 and is skipped.  `un` holds the adjacency
// entries of the first chunk (row[b0 + lane]).
template <int K, class WC>
__device__ __forceinline__ float dep_span_from(const Adj &a, uint32_t f, float sv, uint32_t b0, uint32_t b1,
                                               uint32_t un, const uint32_t *__restrict__ fnext,
                                               const float *__restrict__ mq, uint32_t *su, uint32_t *sg, WC &wc)
{
    const unsigned lane = lane_id();
    const float *mq_l = mq + lane;
    float P = 0.0f;
    // the next chunk's adjacency entries load while this chunk is consumed
    for (uint32_t base = b0; base < b1; base += 32) {
        const uint32_t e = base + lane;
        const uint32_t u = un;
        un = e + 32 < b1 ? a.row[e + 32] : 0u;
        const uint32_t gm = e < b1 ? fnext[(uint64_t)u * K] & f : 0u;
        if (e < b1) {
            wc.add(WC_ENTRIES, 1);
            wc.add(WC_GATHERS, __popc(gm));
            wc.add(WC_BYTES, 8 + 4 * __popc(gm));  // adjacency entry, level mask word, successors' q
        }
        const unsigned pm = __ballot_sync(FULL_MASK, gm != 0);
        if (!pm) continue;
        su[lane] = u;
        sg[lane] = gm;
        __syncwarp();
        float g0 = 0.0f, g1 = 0.0f, g2 = 0.0f, g3 = 0.0f;
        if (pm & 0x000000ffu) g0 = tree8<K>(su, sg, 0, mq_l, sv);
        if (pm & 0x0000ff00u) g1 = tree8<K>(su, sg, 1, mq_l, sv);
        if (pm & 0x00ff0000u) g2 = tree8<K>(su, sg, 2, mq_l, sv);
        if (pm & 0xff000000u) g3 = tree8<K>(su, sg, 3, mq_l, sv);
        P = __fadd_rn(P, __fadd_rn(__fadd_rn(g0, g1), __fadd_rn(g2, g3)));
        __syncwarp();
    }
    return P;
}

template <int K, class WC>
__device__ __forceinline__ float dep_span(const Adj &a, uint32_t f, float sv, uint32_t b0, uint32_t b1,
                                          const uint32_t *__restrict__ fnext, const float *__restrict__ mq,
                                          uint32_t *su, uint32_t *sg, WC &wc)
{
    const uint32_t e = b0 + lane_id();
    return dep_span_from<K>(a, f, sv, b0, b1, e < b1 ? a.row[e] : 0u, fnext, mq, su, sg, wc);
}

// delta and q of vertex v for the half's pivots in f
template <int K>
__device__ __forceinline__ void write_dep(float *mdelta, float *mq, uint32_t v, uint32_t f, float delta,
                                          uint32_t sig)
{
    const unsigned lane = lane_id();
    if ((f >> lane) & 1u) {
        mdelta[row_base<K>(v) + lane] = delta;
        mq[row_base<K>(v) + lane] = __fdiv_rn(__fadd_rn(delta, 1.0f), __uint2float_rn(sig));
    }
}

// Backward depth d for the half's pivots in dmask.  With no_succ (the deepest
// depth) nothing lies below, so delta = reach.
template <int K, class WC>
__device__ __forceinline__ void bwd_vertices(const Adj &a, uint32_t v_l, uint32_t f_l, int no_succ,
                                             const uint32_t *__restrict__ fnext,
                                             const uint32_t *__restrict__ msigma, float *mdelta,
                                             float *mq, const uint32_t *__restrict__ reach,
                                             uint32_t *su, uint32_t *sg, WC &wc)
{
    const unsigned lane = lane_id();
    unsigned act = __ballot_sync(FULL_MASK, f_l != 0);
    if (!act) return;
    // adjacency bounds and reach of each vertex; per pivot its path count
    // read, its dependency and q written
    if (f_l) {
        wc.add(WC_BYTES, (no_succ ? 4 : 12) + 12 * __popc(f_l));
        wc.add(WC_PAIRS, __popc(f_l));
    }
    // the adjacency bounds of all listed vertices load at once; the first
    // chunk of the next vertex's adjacency loads while a vertex is summed
    uint32_t c0_l = 0, c1_l = 0;
    if (f_l && !no_succ) {
        c0_l = a.col[v_l];
        c1_l = a.col[v_l + 1];
    }
    int j = __ffs(act) - 1;
    uint32_t b0 = __shfl_sync(FULL_MASK, c0_l, j), b1 = __shfl_sync(FULL_MASK, c1_l, j);
    uint32_t un = b0 + lane < b1 ? a.row[b0 + lane] : 0u;
    for (;;) {
        act &= act - 1;
        const uint32_t v = __shfl_sync(FULL_MASK, v_l, j);
        const uint32_t f = __shfl_sync(FULL_MASK, f_l, j);
        const uint32_t cb0 = b0, cb1 = b1, cu = un;
        const int jn = act ? __ffs(act) - 1 : -1;
        if (jn >= 0) {
            b0 = __shfl_sync(FULL_MASK, c0_l, jn);
            b1 = __shfl_sync(FULL_MASK, c1_l, jn);
            un = b0 + lane < b1 ? a.row[b0 + lane] : 0u;
        }
        const uint32_t sig = ((f >> lane) & 1u) ? msigma[row_base<K>(v) + lane] : 0u;
        float P = 0.0f;
        if (!no_succ) P = dep_span_from<K>(a, f, __uint2float_rn(sig), cb0, cb1, cu, fnext, mq, su, sg, wc);
        write_dep<K>(mdelta, mq, v, f, __fadd_rn(__uint2float_rn(reach[v]), P), sig);
        if (jn < 0) break;
        j = jn;
    }
}

template <int K, class WC>
__device__ __forceinline__ void bwd_body(const Adj &a, uint32_t dmask, int no_succ,
                                         const uint32_t *__restrict__ fd, const uint32_t *__restrict__ fnext,
                                         const uint32_t *__restrict__ msigma, float *mdelta,
                                         float *mq, float *mpartial,
                                         const uint32_t *__restrict__ reach, uint32_t *ctr,
                                         uint32_t *su, uint32_t *sg, const uint32_t *lst,
                                         uint32_t lcnt, uint32_t lheavy, WC &wc)
{
    const unsigned lane = lane_id();
    // heavy span items only when a heavy vertex is at this depth
    const uint64_t nhi = lst && lheavy == 0 ? 0 : a.n_heavy_items;
    const uint32_t ent = list_unit(lcnt);
    const uint64_t nu = lst ? nhi + (lcnt + ent - 1) / ent : n_units(a);
    if (warp_global() >= nu) return;  // fewer units than warps: no contention
    for (;;) {
        const uint32_t t = grab_unit(ctr);
        if (t >= nu) break;
        if (t < nhi) {
            const uint32_t v = a.hitem_v[t];
            const uint32_t f = fd[(uint64_t)v * K] & dmask;
            if (lane == 0) wc.add(WC_BYTES, 4);  // level mask word
            if (!f) continue;
            float P = 0.0f;
            if (!no_succ) {
                const float sv =
                    __uint2float_rn(((f >> lane) & 1u) ? msigma[row_base<K>(v) + lane] : 0u);
                const uint32_t b0 = a.col[v] + a.hitem_k[t] * AXBC_SPAN;
                P = dep_span<K>(a, f, sv, b0, min(a.col[v + 1], b0 + AXBC_SPAN), fnext, mq, su, sg, wc);
            }
            mpartial[(uint64_t)t * (AXBC_W * K) + lane] = P;
            if ((f >> lane) & 1u) wc.add(WC_BYTES, 8);  // path count read, span partial written
            continue;
        }
        if (lst) {
            const uint32_t i = (uint32_t)(t - nhi) * ent + lane;
            uint32_t v_l = 0, f_l = 0;
            if (lane < ent && i < lcnt) {
                v_l = lst[i];
                if (a.col[v_l + 1] - a.col[v_l] <= AXBC_SPAN) f_l = fd[(uint64_t)v_l * K] & dmask;
                wc.add(WC_BYTES, 8);  // list entry, level mask word
            }
            bwd_vertices<K>(a, v_l, f_l, no_succ, fnext, msigma, mdelta, mq, reach, su, sg, wc);
            continue;
        }
        const uint64_t l0 = (uint64_t)(t - nhi) * LIGHT_PER_UNIT;
        for (uint64_t lt = l0; lt < l0 + LIGHT_PER_UNIT && lt < a.n_ltask; lt++) {
            const uint32_t beg = a.ltask[lt], cnt = a.ltask[lt + 1] - beg;
            uint32_t v_l = 0, f_l = 0;
            if (lane < cnt) {
                v_l = a.order[beg + lane];
                f_l = fd[(uint64_t)v_l * K] & dmask;
                wc.add(WC_BYTES, 4);  // level mask word
            }
            bwd_vertices<K>(a, v_l, f_l, no_succ, fnext, msigma, mdelta, mq, reach, su, sg, wc);
        }
    }
}

// One backward depth, device-driven: d = bi->bd (a no-op once below 0).  The
// grid's y index is the half: the blocks of half 1 of a 64-pivot pass start as
// those of half 0 run out of work, each half with its own work counter.  CNT:
// the counting build (work counts into wc[KP_BWD]).
template <int K, bool CNT>
__global__ void __launch_bounds__(BATCH_TPB, AXBC_BWD_MIN_BLOCKS) k_bwd_step(Adj a, const BatchInfo *__restrict__ bi,
                                                        uint32_t *const *__restrict__ tab,
                                                        const uint32_t *__restrict__ msigma,
                                                        float *mdelta, float *mq, float *mpartial,
                                                        const uint32_t *__restrict__ reach,
                                                        uint32_t *ctrs, LevelLists ll,
                                                        unsigned long long *wc)
{
    typedef typename MaskOf<K>::T M;
    __shared__ __align__(16) uint32_t s_u[BATCH_TPB];
    __shared__ __align__(16) uint32_t s_g[BATCH_TPB];
    const int d = bi->bd;
    if (d < 0) return;
    const int hh = K == 1 ? 0 : blockIdx.y;
    const uint32_t dmask = half_of<K>((M)(d >= 1 ? bi->srcmask : bi->depth0mask), hh);
    if (!dmask) return;
    uint32_t *su = s_u + (threadIdx.x & ~31u), *sg = s_g + (threadIdx.x & ~31u);
    uint32_t lcnt = 0;
    const uint32_t *lst = level_list(ll, d, lcnt);
    WorkCount<CNT> cnt;
    bwd_body<K>(a, dmask, d == bi->dmax, tab[d] + hh, tab[d + 1] + hh, msigma + 32 * hh, mdelta + 32 * hh,
                mq + 32 * hh, mpartial + 32 * hh, reach, ctrs + 2 * AXBC_MAX_LEVELS * hh + 2 * d + 1, su, sg, lst,
                lcnt, ll.heavy[d], cnt);
    cnt.flush(wc);
}

template <int K>
__device__ __forceinline__ void combine_body(const Adj &a, uint32_t dmask, const uint32_t *__restrict__ fd,
                                             const uint32_t *__restrict__ msigma, float *mdelta,
                                             float *mq, const float *__restrict__ mpartial,
                                             const uint32_t *__restrict__ reach)
{
    const unsigned lane = lane_id();
    const uint64_t nw = (uint64_t)gridDim.x * blockDim.x / 32;
    for (uint64_t i = (blockIdx.x * (uint64_t)blockDim.x + threadIdx.x) / 32; i < a.n_heavy; i += nw) {
        const uint32_t v = a.heavy_v[i];
        const uint32_t f = fd[(uint64_t)v * K] & dmask;
        if (!f) continue;
        float acc = __uint2float_rn(reach[v]);
        for (uint32_t k = a.heavy_first[i]; k < a.heavy_first[i + 1]; k++)
            acc = __fadd_rn(acc, mpartial[(uint64_t)k * (AXBC_W * K) + lane]);
        const uint32_t sig = ((f >> lane) & 1u) ? msigma[row_base<K>(v) + lane] : 0u;
        write_dep<K>(mdelta, mq, v, f, acc, sig);
    }
}

template <int K>
__global__ void k_bwd_combine_step(Adj a, const BatchInfo *__restrict__ bi,
                                   uint32_t *const *__restrict__ tab,
                                   const uint32_t *__restrict__ msigma, float *mdelta, float *mq,
                                   const float *__restrict__ mpartial,
                                   const uint32_t *__restrict__ reach, LevelLists ll)
{
    typedef typename MaskOf<K>::T M;
    const int d = bi->bd;
    if (d < 0) return;
    uint32_t lcnt;
    if (level_list(ll, d, lcnt) && ll.heavy[d] == 0) return;  // no heavy vertex at this depth
    const int hh = K == 1 ? 0 : blockIdx.y;
    const uint32_t dmask = half_of<K>((M)(d >= 1 ? bi->srcmask : bi->depth0mask), hh);
    if (!dmask) return;
    combine_body<K>(a, dmask, tab[d] + hh, msigma + 32 * hh, mdelta + 32 * hh, mq + 32 * hh, mpartial + 32 * hh,
                    reach);
}

__global__ void k_bwd_advance(BatchInfo *bi)
{
    if (bi->bd >= 0) bi->bd--;
}
// ------------------------------------------------ persistent level loop
// On graphs of many narrow levels (grids, roads) a level's work is a few
// microseconds and the four launches per forward level and three per
// backward depth dominate.  k_traverse_persist runs a whole batch -- every
// forward level, then every backward depth -- in one cooperative launch whose
// blocks are all resident, with the step kernels' device bodies separated by a
// grid barrier: two barriers per forward level (expansion | statistics and
// level close) and one or two per backward depth.

// Wait budget of one barrier in SM clock cycles (about 4 s at 2 GHz): a wait
// that runs out records its site and every block returns; the host reports
// AXBC_ERR_TIMEOUT.
#define AXBC_BAR_BUDGET (1ll << 33)

__device__ __forceinline__ unsigned vload_u(const unsigned *p) { return *(const volatile unsigned *)p; }
__device__ __forceinline__ int vload_i(const int *p) { return *(const volatile int *)p; }

// All blocks of the cooperative grid meet here.  The last block to arrive runs
// lead() with its first warp, then releases the others.  Thread 0 of each block
// fences before arriving and after the wait, as cooperative groups' grid sync
// does, so the block's later loads see what every block wrote before
// arriving.  Returns false when this wait, or an earlier one of any block, ran
// out of its budget.
struct NoLead {
    __device__ void operator()() const {}
};
template <class F>
__device__ __forceinline__ bool grid_barrier(GridSync *gs, long long budget, int site, const F &lead)
{
    __shared__ int s_role;  // 1 leader, 0 released, -1 failed
    __syncthreads();
    if (threadIdx.x == 0) {
        const unsigned g = vload_u(&gs->gen);
        __threadfence();
        const unsigned arrived = atomicAdd(&gs->count, 1u);
        int role = arrived == gridDim.x - 1 ? 1 : 0;
        if (role == 0) {
            const long long t0 = clock64();
            while (vload_u(&gs->gen) == g) {
                if (vload_i(&gs->err)) {
                    role = -1;
                    break;
                }
                if (clock64() - t0 > budget) {
                    atomicCAS(&gs->err, 0, site);
                    role = -1;
                    break;
                }
                __nanosleep(32);
            }
        }
        __threadfence();
        s_role = role;
    }
    __syncthreads();
    const int role = s_role;
    if (role == 1) {
        if (threadIdx.x < 32) lead();
        __syncthreads();
        if (threadIdx.x == 0) {
            gs->count = 0;
            __threadfence();
            atomicAdd(&gs->gen, 1u);
        }
    }
    return role >= 0;
}

template <int K> struct AdvanceLead {
    BatchInfo *bi;
    unsigned long long *level_te, *level_cnt;
    int32_t *level_mode;
    LevelLists ll;
    uint32_t pool_cap, list_max;
    __device__ void operator()() const
    {
        level_advance_warp<K>(bi, level_te, level_cnt, level_mode, ll, pool_cap, list_max);
    }
};
struct BwdLead {
    BatchInfo *bi;
    __device__ void operator()() const
    {
        if (lane_id() == 0 && bi->bd >= 0) bi->bd--;
    }
};

// The arrays the loop writes are passed without const/__restrict__, so that
// no load of them goes through the read-only cache: they change between
// phases of the one launch.  Levels stop at lmax (the masks allocated): the
// kernel sets gs->need and the host grows the tables and launches again, the
// loop resuming from the level state in bi.
template <int K>
__global__ void __launch_bounds__(BATCH_TPB) k_traverse_persist(
    Adj a, Adj rv, BatchInfo *bi, uint32_t **tab, uint32_t *seen_, uint32_t *msigma, float *mdelta,
    float *mq, float *mpartial, const uint32_t *reach, uint32_t *ctrs, LevelLists ll,
    unsigned long long *level_te, unsigned long long *level_cnt, int32_t *level_mode,
    uint32_t pool_cap, uint32_t list_max, uint64_t n, int lmax, GridSync *gs, long long budget)
{
    typedef typename MaskOf<K>::T M;
    __shared__ __align__(16) uint32_t s_u[BATCH_TPB];
    __shared__ __align__(16) uint32_t s_g[BATCH_TPB * K];
    __shared__ uint32_t s_k[BATCH_TPB];
    const unsigned w0 = threadIdx.x & ~31u;
    M *seen = reinterpret_cast<M *>(seen_);
    WorkCount<false> none;
    const AdvanceLead<K> adv{bi, level_te, level_cnt, level_mode, ll, pool_cap, list_max};
    for (;;) {
        if (!vload_i(&bi->alive)) break;
        const int L = vload_i(&bi->cur) + 1;
        if (L >= lmax) {
            if (blockIdx.x == 0 && threadIdx.x == 0) gs->need = 1;
            return;
        }
        const M srcmask = (M)bi->srcmask;
        M *fprev = reinterpret_cast<M *>(tab[L - 1]), *fcur = reinterpret_cast<M *>(tab[L]);
        if (vload_i(&bi->push_next))
            fwd_push_body<K>(a, fprev, fcur, seen, msigma, ctrs + 2 * L, ll, L, none);
        else
            fwd_pull_body<K>(rv, srcmask, fprev, fcur, seen, msigma, ctrs + 2 * L, s_u + w0, s_g + w0 * K,
                             s_k + w0, ll, L, none);
        if (!grid_barrier(gs, budget, 1, NoLead{})) return;
        stats_body<K>(n, bi, L, srcmask, fcur, seen, a.col, rv.col, reach, ll);
        if (!grid_barrier(gs, budget, 2, adv)) return;
    }
    const BwdLead down{bi};
    for (;;) {
        const int d = vload_i(&bi->bd);
        if (d < 0) break;
        const M dmask = (M)(d >= 1 ? bi->srcmask : bi->depth0mask);
        if (dmask) {
            uint32_t lcnt = 0;
            const uint32_t *lst = level_list(ll, d, lcnt);
            const uint32_t lheavy = ll.heavy[d];
            // the halves touch disjoint columns and have their own work
            // counters: one phase takes both
        #pragma unroll 1
    for (int hh = 0; hh < K; hh++)
                if (half_of<K>(dmask, hh))
                    bwd_body<K>(a, half_of<K>(dmask, hh), d == bi->dmax, tab[d] + hh, tab[d + 1] + hh,
                                msigma + 32 * hh, mdelta + 32 * hh, mq + 32 * hh, mpartial + 32 * hh, reach,
                                ctrs + 2 * AXBC_MAX_LEVELS * hh + 2 * d + 1, s_u + w0, s_g + w0, lst, lcnt, lheavy,
                                none);
            if (a.n_heavy && !(lst && lheavy == 0)) {
                if (!grid_barrier(gs, budget, 3, NoLead{})) return;
            #pragma unroll 1
    for (int hh = 0; hh < K; hh++)
                    if (half_of<K>(dmask, hh))
                        combine_body<K>(a, half_of<K>(dmask, hh), tab[d] + hh, msigma + 32 * hh, mdelta + 32 * hh,
                                        mq + 32 * hh, mpartial + 32 * hh, reach);
            }
        }
        if (!grid_barrier(gs, budget, 4, down)) return;
    }
}

// Self-test of the grid barrier: `rounds` barriers, the leader of each adding
// one to out[0]; block `absent` (if >= 0) never arrives, so the first wait runs
// out of its budget and every block returns.
struct CountLead {
    unsigned *out;
    __device__ void operator()() const
    {
        if (lane_id() == 0) out[0]++;
    }
};
__global__ void __launch_bounds__(BATCH_TPB) k_barrier_selftest(GridSync *gs, int rounds, long long budget,
                                                                int absent, unsigned *out)
{
    if ((int)blockIdx.x == absent) return;
    const CountLead lead{out};
    for (int r = 0; r < rounds; r++)
        if (!grid_barrier(gs, budget, r + 1, lead)) return;
}

// bc update for the applied pivots in lane order (update_bc, src/cuda_kernels.cu:
// 269-286), each into its lane's bc vector.  A pivot that did not reach v
// contributes delta = reach[v].  Zero terms are skipped: x + float(0/p) == x for
// p > 0.  One thread per vertex, its 32 K dependencies read from rows a warp
// staged in shared memory.
// 4-byte global -> shared copies that bypass registers (cp.async), so a warp
// keeps up to 32 row loads of one chunk and the next chunk's in flight
__device__ __forceinline__ void cp_async4(void *smem, const void *gmem)
{
    const unsigned sa = (unsigned)__cvta_generic_to_shared(smem);
    asm volatile("cp.async.ca.shared.global [%0], [%1], 4;\n" ::"r"(sa), "l"(gmem) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
template <int N> __device__ __forceinline__ void cp_async_wait()
{
    asm volatile("cp.async.wait_group %0;\n" ::"n"(N) : "memory");
}

// stage the dependency rows of the chunk's vertices reached by pivots of half
// hh (sv: their masks for that half): lane l copies column 32 hh + l
template <int K>
__device__ __forceinline__ void stage_half(float (*rows)[AXBC_W + 1], const float *__restrict__ mdelta,
                                           uint64_t base, uint32_t sv, int hh)
{
    const unsigned lane = lane_id();
    unsigned need = __ballot_sync(FULL_MASK, sv != 0);
    while (need) {
        const int r = __ffs(need) - 1;
        need &= need - 1;
        cp_async4(&rows[r][lane], mdelta + row_base<K>(base + r) + 32 * hh + lane);
    }
    cp_async_commit();
}

// threads of the update (34 KB of staged rows)
#define UPD_TPB(K) 128
template <int K>
__global__ void __launch_bounds__(UPD_TPB(K)) k_update_m(const float *__restrict__ mdelta,
                                                         const uint32_t *__restrict__ seen_,
                                                         const uint32_t *__restrict__ reach, uint64_t n,
                                                         const BatchInfo *__restrict__ bi,
                                                         float *__restrict__ delta_out,
                                                         const uint32_t *__restrict__ from_view)
{
    typedef typename MaskOf<K>::T M;
    constexpr int NS = AXBC_W * K;  // pivot slots
    constexpr int TPB = UPD_TPB(K);
    const M *seen = reinterpret_cast<const M *>(seen_);
    __shared__ uint32_t s_root[NS], s_reach[NS], s_skip0[NS];
    __shared__ double s_p[NS];
    __shared__ unsigned long long s_nvt[NS];
    __shared__ InvSplit s_iv[NS];
    __shared__ float *s_bc[NS];
    // per lane: float(reach_v0 + 1), the split 1/p, and whether the fast
    // division applies (bit 0) and zero terms may be skipped (bit 1)
    __shared__ float4 s_k[NS];
    __shared__ int s_single;  // every applied lane updates the same vector
    __shared__ int s_allpos;  // every applied lane has p > 0 (zero terms vanish)
    // per warp, two staged units: the dependency rows of 32 vertices for one
    // 32-pivot half, padded to 33 floats so that thread t reading row t,
    // column s hits bank (t + s) mod 32
    __shared__ float s_rows[TPB / 32][2][32][AXBC_W + 1];
    const M amask = (M)(bi->applymask & bi->srcmask);
    for (int s = threadIdx.x; s < NS; s += TPB) {
        s_bc[s] = bi->lane_bc[s];
        if ((amask >> s) & 1u) {
            const uint32_t r = bi->root[s];
            const uint32_t rv = reach[r];
            const uint32_t all = (bi->H == 1 ? (uint32_t)bi->rsum[s] : 0u) + rv;
            s_root[s] = r;
            s_reach[s] = rv;
            s_p[s] = bi->p[s];
            s_skip0[s] = bi->p[s] > 0.0;
            s_nvt[s] = bi->nvis[s] + all;
            s_iv[s] = inv_split(bi->p[s]);
        } else {
            s_root[s] = 0xffffffffu;
            s_reach[s] = 0;
            s_p[s] = 1.0;
            s_skip0[s] = 1;
            s_nvt[s] = 2;
            s_iv[s] = inv_split(1.0);
        }
        const InvSplit iv = s_iv[s];
        s_k[s] = make_float4(__uint2float_rn(s_reach[s] + 1u), iv.hi, iv.lo,
                             __uint_as_float((iv.ok ? 1u : 0u) | (s_skip0[s] ? 2u : 0u)));
        if (s == 0) {
            int single = 1, allpos = 1;
            float *t0 = nullptr;
            for (int l = 0; l < NS; l++)
                if ((amask >> l) & 1u) {
                    if (!t0) t0 = bi->lane_bc[l];
                    else if (bi->lane_bc[l] != t0) single = 0;
                    if (!(bi->p[l] > 0.0)) allpos = 0;
                }
            s_single = single;
            s_allpos = allpos;
        }
    }
    __syncthreads();
    if (amask == 0) return;
    const bool single = s_single != 0;
    // a vertex no pivot reached, with reach 0, gets only zero terms: skipped
    // when they vanish (p > 0; 0/0 is NaN, as in the reference)
    const bool skip_unreached = s_allpos != 0;
    const int slast = 63 - __clzll((unsigned long long)amask);
    // delta_out (when given): the last applied pivot's dependencies, taken
    // from the staged rows (k_extract_delta's rule)
    const uint32_t dl_root = bi->root[slast];
    const bool dl_root_done = (bi->depth0mask >> slast) & 1u;
    const unsigned lane = lane_id();
    const unsigned wid = threadIdx.x >> 5;
    const uint64_t stride = (uint64_t)gridDim.x * (TPB / 32) * 32;
    uint64_t base = (blockIdx.x * (uint64_t)(TPB / 32) + wid) * 32;
    if (base >= n) return;
    M sv = 0;
    uint32_t rv = 0;
    if (base + lane < n) {
        sv = seen[base + lane];
        rv = reach[base + lane];
    }
    // units of (chunk of 32 vertices, 32-pivot half), in order; each vertex
    // sums its slots in slot order across the halves of its chunk
    stage_half<K>(s_rows[wid][0], mdelta, base, (uint32_t)sv, 0);
    int buf = 0;
    for (; base < n; base += stride) {
        const uint64_t next = base + stride;
        M svn = 0;
        uint32_t rvn = 0;
        if (next + lane < n) {
            svn = seen[next + lane];
            rvn = reach[next + lane];
        }
        const uint64_t v = base + lane;
        // v numbers the graph's view; the bc vectors and delta_out are indexed
        // by vertex id
        const uint64_t vo = from_view && v < n ? from_view[v] : v;
        const float rf = __uint2float_rn(rv);
        // unreached by every pivot with delta 0: only a root term could apply,
        // and roots are reached
        const bool work = v < n && (sv != 0 || rv != 0u || !skip_unreached);
        // one target vector, reach 0, every p > 0: a pivot that did not reach
        // v adds +0, so only the reached lanes are visited
        const bool sparse = work && single && rv == 0u && skip_unreached;
        float *tgt = nullptr;
        float b = 0.0f;
        if (work && single) {
            tgt = s_bc[slast];
            b = tgt[vo];
        }
#pragma unroll 1
        for (int hh = 0; hh < K; hh++, buf ^= 1) {
            // the next unit's rows load while this one is summed
            if (hh + 1 < K) {
                stage_half<K>(s_rows[wid][buf ^ 1], mdelta, base, (uint32_t)((unsigned long long)sv >> 32), 1);
                cp_async_wait<1>();
            } else if (next < n) {
                stage_half<K>(s_rows[wid][buf ^ 1], mdelta, next, (uint32_t)svn, 0);
                cp_async_wait<1>();
            } else {
                cp_async_wait<0>();
            }
            __syncwarp();
            const float(*rows)[AXBC_W + 1] = s_rows[wid][buf];
            const uint32_t svh = (uint32_t)((unsigned long long)sv >> (32 * hh));
            const uint32_t amh = (uint32_t)((unsigned long long)amask >> (32 * hh));
            const int s0 = 32 * hh;
            if (delta_out && v < n && (slast >> 5) == hh) {
                const bool have = v == dl_root ? dl_root_done : ((svh >> (slast & 31)) & 1u) != 0u;
                delta_out[vo] = have ? rows[lane][slast & 31] : rf;
            }
            if (sparse) {
                for (uint32_t bits = svh & amh; bits; bits &= bits - 1) {
                    const int j = __ffs(bits) - 1, s = s0 + j;
                    if ((uint32_t)v == s_root[s]) {
                        if (s_reach[s] > 0) b = __fadd_rn(b, bc_root_term(s_reach[s], s_nvt[s]));
                        continue;
                    }
                    const float dv = rows[lane][j];
                    if (dv == 0.0f) continue;
                    const float4 k = s_k[s];
                    const uint32_t fl = __float_as_uint(k.w);
                    b = __fadd_rn(b, div_to_float_hl(__fmul_rn(dv, k.x), s_p[s], k.y, k.z, (fl & 1u) != 0u));
                }
            } else if (work && single) {
                // one target vector: every slot in order
#pragma unroll
                for (int j = 0; j < AXBC_W; j++) {
                    if (!((amh >> j) & 1u)) continue;
                    const int s = s0 + j;
                    if ((uint32_t)v == s_root[s]) {
                        if (s_reach[s] > 0) b = __fadd_rn(b, bc_root_term(s_reach[s], s_nvt[s]));
                        continue;
                    }
                    const float dv = ((svh >> j) & 1u) ? rows[lane][j] : rf;
                    const float4 k = s_k[s];
                    const uint32_t fl = __float_as_uint(k.w);
                    if (dv == 0.0f && (fl & 2u)) continue;
                    b = __fadd_rn(b, div_to_float_hl(__fmul_rn(dv, k.x), s_p[s], k.y, k.z, (fl & 1u) != 0u));
                }
            } else if (work) {
                // lanes in order; consecutive lanes of one run add into one
                // register, written back when the target vector changes
                for (int j = 0; j < AXBC_W && s0 + j <= slast; j++) {
                    if (!((amh >> j) & 1u)) continue;
                    const int s = s0 + j;
                    if (s_bc[s] != tgt) {
                        if (tgt) tgt[vo] = b;
                        tgt = s_bc[s];
                        b = tgt[vo];
                    }
                    if ((uint32_t)v == s_root[s]) {
                        if (s_reach[s] > 0) b = __fadd_rn(b, bc_root_term(s_reach[s], s_nvt[s]));
                        continue;
                    }
                    const float dv = ((svh >> j) & 1u) ? rows[lane][j] : rf;
                    if (dv == 0.0f && s_skip0[s]) continue;
                    b = __fadd_rn(b, bc_term_fast(dv, s_reach[s], s_p[s], s_iv[s]));
                }
            }
            __syncwarp();
        }
        if (tgt) tgt[vo] = b;
        sv = svn;
        rv = rvn;
    }
}

// the last applied pivot's dependencies as a plain n-vector
template <int K>
__global__ void k_extract_delta(float *out, const float *__restrict__ mdelta,
                                const uint32_t *__restrict__ seen_,
                                const uint32_t *__restrict__ reach, uint64_t n,
                                const BatchInfo *__restrict__ bi, int lane_lo, int lane_hi,
                                const uint32_t *__restrict__ from_view)
{
    typedef typename MaskOf<K>::T M;
    const M *seen = reinterpret_cast<const M *>(seen_);
    // the highest applied lane of [lane_lo, lane_hi)
    unsigned long long range = lane_hi >= 64 ? ~0ull : ((1ull << lane_hi) - 1ull);
    range &= ~((1ull << lane_lo) - 1ull);
    const unsigned long long am = bi->applymask & bi->srcmask & range;
    if (am == 0) return;
    const int s = 63 - __clzll(am);
    const uint32_t root = bi->root[s];
    const bool root_done = (bi->depth0mask >> s) & 1ull;
    for (uint64_t v = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; v < n;
         v += (uint64_t)gridDim.x * blockDim.x) {
        bool have = ((unsigned long long)seen[v] >> s) & 1ull;
        if (v == root) have = root_done;
        out[from_view ? from_view[v] : v] = have ? mdelta[row_base<K>(v) + s] : __uint2float_rn(reach[v]);
    }
}

// one pivot of the last batch: path counts, depths, dependencies
template <int K>
__global__ void k_source_view(int s, int levels, uint32_t *const *fm, const uint32_t *__restrict__ seen_,
                              const uint32_t *__restrict__ msigma, const float *__restrict__ mdelta,
                              const uint32_t *__restrict__ reach, uint64_t n, unsigned long long depth0,
                              uint32_t *sig, int32_t *lvl, float *dl, const uint32_t *__restrict__ from_view)
{
    typedef typename MaskOf<K>::T M;
    const M *seen = reinterpret_cast<const M *>(seen_);
    for (uint64_t v = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; v < n;
         v += (uint64_t)gridDim.x * blockDim.x) {
        int L = -1;
        if (((unsigned long long)seen[v] >> s) & 1ull) {
            for (int l = 0; l < levels; l++)
                if (((unsigned long long)reinterpret_cast<const M *>(fm[l])[v] >> s) & 1ull) {
                    L = l;
                    break;
                }
        }
        // v numbers the graph's view; the outputs are indexed by vertex id
        const uint64_t vo = from_view ? from_view[v] : v;
        lvl[vo] = L;
        sig[vo] = L >= 0 ? msigma[row_base<K>(v) + s] : 0u;
        bool have = L > 0 || (L == 0 && ((depth0 >> s) & 1ull));
        dl[vo] = have ? mdelta[row_base<K>(v) + s] : __uint2float_rn(reach[v]);
    }
}

static int ensure_level_tables(axbc_ctx *c)
{
    if (c->tables_ready) return AXBC_OK;
    ALLOC_MISSING(c->fmtab, AXBC_MAX_LEVELS * sizeof(uint32_t *), &c->bytes);
    ALLOC_MISSING(c->ctrs, 2 * AXBC_WMAX / 32 * AXBC_MAX_LEVELS * 4, &c->bytes);
    ALLOC_MISSING(c->d_level_te, AXBC_MAX_LEVELS * 8, &c->bytes);
    ALLOC_MISSING(c->d_level_cnt, AXBC_MAX_LEVELS * 8, &c->bytes);
    ALLOC_MISSING(c->d_level_mode, AXBC_MAX_LEVELS * 4, &c->bytes);
    // level lists: a vertex joins a level's list once per distinct depth at
    // which the batch's pivots reach it (at most 64 n entries); the pool
    // starts at 32 n and grows when a batch runs short; a level may hold up to
    // n/8 vertices before it falls back to the task scan
    if (!c->lpool) {
        const uint32_t cap = (uint32_t)std::min<uint64_t>((uint64_t)AXBC_W * c->g->n + 64, 0xffffffffull);
        TRY(axbc_dalloc((void **)&c->lpool, (uint64_t)cap * 4, &c->bytes));
        c->lpool_cap = cap;
    }
    ALLOC_MISSING(c->lstart, AXBC_MAX_LEVELS * 4, &c->bytes);
    ALLOC_MISSING(c->lcount, AXBC_MAX_LEVELS * 4, &c->bytes);
    ALLOC_MISSING(c->lcap, AXBC_MAX_LEVELS * 4, &c->bytes);
    ALLOC_MISSING(c->lheavy, AXBC_MAX_LEVELS * 4, &c->bytes);
    c->tables_ready = true;
    return AXBC_OK;
}

static LevelLists lists_of(const axbc_ctx *c)
{
    return LevelLists{c->lpool, c->lstart, c->lcount, c->lcap, c->lheavy};
}

// Largest stored level list: n/8 vertices, or n/2 when no vertex has more than
// 64 neighbours (a list unit then carries little work whatever it holds, and a
// wide level of a high-diameter graph is still cheaper to walk than to scan).
static uint32_t list_max_of(const axbc_ctx *c)
{
    const uint64_t n = c->g->n;
    return (uint32_t)std::max<uint64_t>(64, c->g->max_deg <= 64 ? n / 2 : n / 8);
}

// Level masks 0..levels-1 exist (two words per vertex, enough for either
// width), and their pointers are in the device table.  Every mask array is
// all zero between batches.
int axbc_batch_levels_alloc(axbc_ctx *c, int levels)
{
    TRY(ensure_level_tables(c));
    if (levels > AXBC_MAX_LEVELS) {
        axbc_set_error("traversal deeper than %d levels", AXBC_MAX_LEVELS - 2);
        return AXBC_ERR_RANGE;
    }
    // masks allocated by an earlier, partly failed call reach the device table
    // here too: fmtab_synced counts the entries copied so far
    int rc = AXBC_OK;
    while ((int)c->fmask.size() < levels) {
        uint32_t *p = nullptr;
        if ((rc = axbc_dalloc((void **)&p, c->g->n * 8, &c->bytes)) != AXBC_OK) break;
        c->fmask.push_back(p);
        CU(cudaMemset(p, 0, c->g->n * 8));
    }
    if (c->fmask.size() > c->fmtab_synced) {
        CU(cudaMemcpy(c->fmtab + c->fmtab_synced, c->fmask.data() + c->fmtab_synced,
                      (c->fmask.size() - c->fmtab_synced) * sizeof(uint32_t *), cudaMemcpyHostToDevice));
        c->fmtab_synced = c->fmask.size();
    }
    return rc;
}

// per-pivot rows of 64 values, masks of two words: a pass of either width
int axbc_ensure_batch(axbc_ctx *c)
{
    if (c->batch_ready) return AXBC_OK;
    const uint64_t n = c->g->n;
    ALLOC_MISSING(c->seen, n * 8, &c->bytes);
    ALLOC_MISSING(c->msigma, n * AXBC_WMAX * 4, &c->bytes);
    ALLOC_MISSING(c->mdelta, n * AXBC_WMAX * 4, &c->bytes);
    ALLOC_MISSING(c->mq, n * AXBC_WMAX * 4, &c->bytes);
    ALLOC_MISSING(c->task_ctr, 64, &c->bytes);
    ALLOC_MISSING(c->mpartial, (c->g->bfwd.n_heavy_items + 1) * AXBC_WMAX * 4, &c->bytes);
    ALLOC_MISSING(c->bi, sizeof(BatchInfo), &c->bytes);
    if (!c->bi_host) CU(cudaMallocHost((void **)&c->bi_host, sizeof(BatchInfo)));
    CU(cudaMemset(c->bi, 0, sizeof(BatchInfo)));
    CU(cudaMemset(c->seen, 0, n * 8));
    TRY(axbc_batch_levels_alloc(c, 10));
    c->batch_ready = true;
    return AXBC_OK;
}

// mask words per vertex for a pass of nsrc pivots
static int width_k(int nsrc) { return nsrc > AXBC_W ? 2 : 1; }

// dynamic kernels: as many blocks as stay resident; work comes from counters
template <int K> static int occupancy(axbc_ctx *c)
{
    const int i = K - 1;
    if (!c->dyn_blocks_per_sm[i]) {
        int a = 0, b = 0, d = 0;
        CU(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&a, k_fwd_push_step<K, false>, BATCH_TPB, 0));
        CU(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, k_bwd_step<K, false>, BATCH_TPB, 0));
        CU(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&d, k_fwd_pull_step<K, false>, BATCH_TPB, 0));
        c->dyn_blocks_per_sm[i] = std::max(1, a);
        c->pull_blocks_per_sm[i] = std::max(1, d);
        c->bwd_blocks_per_sm[i] = std::max(1, b);
    }
    return AXBC_OK;
}
template <int K> static int push_grid(axbc_ctx *c) { return axbc_grid_for(c, BATCH_TPB, c->dyn_blocks_per_sm[K - 1]); }
template <int K> static int pull_grid(axbc_ctx *c) { return axbc_grid_for(c, BATCH_TPB, c->pull_blocks_per_sm[K - 1]); }
template <int K> static int bwd_grid(axbc_ctx *c) { return axbc_grid_for(c, BATCH_TPB, c->bwd_blocks_per_sm[K - 1]); }

// the kernels of one forward level / one backward depth, in stream order
template <int K> static void fwd_step_kernels(axbc_ctx *c, int sgrid)
{
    axbc_graph *g = c->g;
    const LevelLists ll = lists_of(c);
    k_fwd_push_step<K, false><<<push_grid<K>(c), BATCH_TPB, 0, c->stream>>>(g->bfwd, c->bi, c->fmtab, c->seen,
                                                                           c->msigma, c->ctrs, ll, nullptr);
    k_fwd_pull_step<K, false><<<pull_grid<K>(c), BATCH_TPB, 0, c->stream>>>(g->brev, c->bi, c->fmtab, c->seen,
                                                                           c->msigma, c->ctrs, ll, nullptr);
    k_stats_step<K><<<sgrid, BATCH_TPB, 0, c->stream>>>(g->n, c->bi, c->fmtab, c->seen, g->bfwd.col, g->brev.col,
                                                        g->breach, ll);
    k_level_advance<K><<<1, 32, 0, c->stream>>>(c->bi, c->d_level_te, c->d_level_cnt, c->d_level_mode, ll,
                                                c->lpool_cap, list_max_of(c));
}

template <int K> static void bwd_step_kernels(axbc_ctx *c)
{
    axbc_graph *g = c->g;
    k_bwd_step<K, false><<<dim3(bwd_grid<K>(c), K), BATCH_TPB, 0, c->stream>>>(g->bfwd, c->bi, c->fmtab, c->msigma,
                                                                     c->mdelta, c->mq, c->mpartial, g->breach,
                                                                     c->ctrs, lists_of(c), nullptr);
    if (g->bfwd.n_heavy)
        k_bwd_combine_step<K><<<dim3((g->bfwd.n_heavy + 7) / 8, K), 256, 0, c->stream>>>(
            g->bfwd, c->bi, c->fmtab, c->msigma, c->mdelta, c->mq, c->mpartial, g->breach, lists_of(c));
    k_bwd_advance<<<1, 1, 0, c->stream>>>(c->bi);
}

static void drop_captures(axbc_ctx *c)
{
    for (int i = 0; i < 2; i++) {
        if (c->fwd_step_exec[i]) cudaGraphExecDestroy(c->fwd_step_exec[i]);
        if (c->bwd_step_exec[i]) cudaGraphExecDestroy(c->bwd_step_exec[i]);
        c->fwd_step_exec[i] = c->bwd_step_exec[i] = nullptr;
    }
}

// Capture one forward step and one backward step of width K as CUDA graphs;
// every argument is fixed for the context (levels come from device state).
template <int K> static int capture_steps(axbc_ctx *c, int sgrid)
{
    const int i = K - 1;
    if (c->fwd_step_exec[i] && c->bwd_step_exec[i]) return AXBC_OK;
    for (int which = 0; which < 2; which++) {
        cudaGraph_t gr = nullptr;
        CU(cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeThreadLocal));
        if (which == 0) fwd_step_kernels<K>(c, sgrid);
        else bwd_step_kernels<K>(c);
        cudaError_t e = cudaStreamEndCapture(c->stream, &gr);
        if (e != cudaSuccess) return axbc_cuda_fail(e, "capture level step", __FILE__, __LINE__);
        e = cudaGraphInstantiate(which == 0 ? &c->fwd_step_exec[i] : &c->bwd_step_exec[i], gr, 0);
        cudaGraphDestroy(gr);
        if (e != cudaSuccess) return axbc_cuda_fail(e, "instantiate level step", __FILE__, __LINE__);
    }
    return AXBC_OK;
}

// Forward levels and backward depths as launches of the step kernels: CUDA
// graph replays of one level step, in blocks (profiling and counting: each
// kernel launched on its own).  *L_out: the first level that discovered
// nothing.
template <int K> static int traverse_stepwise(axbc_ctx *c, int nsrc, int sgrid, int *L_out)
{
    axbc_graph *g = c->g;
    const uint64_t n = g->n;
    cudaStream_t s = c->stream;
    const bool prof = c->prof_on || c->count_on;
    unsigned long long *wc = c->count_on ? c->wcount : nullptr;
    const LevelLists ll = lists_of(c);
    const uint32_t lmax = list_max_of(c);
    const size_t ctl_off = offsetof(BatchInfo, cur);
    const size_t ctl_len = offsetof(BatchInfo, push_factor) - ctl_off;
    const size_t prof_first = c->prof.size();
    // forward steps launched before the first look at `alive`: one more than
    // the last batch needed, so a batch like it ends after one host round
    // trip; later groups double
    int launched = 0, B = std::max(4, std::min(256, c->last_batch_levels + 1));
    if (c->last_batch_levels == 0) B = 8;
    for (;;) {
        TRY(axbc_batch_levels_alloc(c, launched + B + 2));
        for (int i = 0; i < B; i++) {
            if (!prof) {
                CU(cudaGraphLaunch(c->fwd_step_exec[K - 1], s));
            } else {
                const int L = launched + i + 1;
                {
                    ProfScope ps(c, KP_FWD_PUSH, 0);
                    if (c->prof_on) c->prof.back().tag = L;
                    if (wc)
                        k_fwd_push_step<K, true><<<push_grid<K>(c), BATCH_TPB, 0, s>>>(
                            g->bfwd, c->bi, c->fmtab, c->seen, c->msigma, c->ctrs, ll, wc + KP_FWD_PUSH * WC_NFIELDS);
                    else
                        k_fwd_push_step<K, false><<<push_grid<K>(c), BATCH_TPB, 0, s>>>(
                            g->bfwd, c->bi, c->fmtab, c->seen, c->msigma, c->ctrs, ll, nullptr);
                }
                {
                    ProfScope ps(c, KP_FWD_PULL, 0);
                    if (c->prof_on) c->prof.back().tag = L;
                    if (wc)
                        k_fwd_pull_step<K, true><<<pull_grid<K>(c), BATCH_TPB, 0, s>>>(
                            g->brev, c->bi, c->fmtab, c->seen, c->msigma, c->ctrs, ll, wc + KP_FWD_PULL * WC_NFIELDS);
                    else
                        k_fwd_pull_step<K, false><<<pull_grid<K>(c), BATCH_TPB, 0, s>>>(
                            g->brev, c->bi, c->fmtab, c->seen, c->msigma, c->ctrs, ll, nullptr);
                }
                {
                    ProfScope ps(c, KP_LEVEL_STATS, 0);
                    if (c->prof_on) c->prof.back().tag = L;
                    k_stats_step<K><<<sgrid, BATCH_TPB, 0, s>>>(n, c->bi, c->fmtab, c->seen, g->bfwd.col,
                                                                g->brev.col, g->breach, ll);
                }
                k_level_advance<K><<<1, 32, 0, s>>>(c->bi, c->d_level_te, c->d_level_cnt, c->d_level_mode, ll,
                                                    c->lpool_cap, lmax);
                c->launches++;
            }
        }
        CU_LAUNCH("forward levels");
        if (!prof) c->launches += 4ull * B;
        launched += B;
        c->prev_lend = std::min(launched, (int)c->fmask.size() - 1);  // masks written so far
        CU(cudaMemcpyAsync((char *)c->bi_host + ctl_off, (char *)c->bi + ctl_off, ctl_len,
                           cudaMemcpyDeviceToHost, s));
        CU(cudaStreamSynchronize(s));
        if (!c->bi_host->alive) break;
        if (launched + 2 * B + 2 > AXBC_MAX_LEVELS) {
            axbc_set_error("traversal deeper than %d levels", AXBC_MAX_LEVELS - 2);
            return AXBC_ERR_RANGE;
        }
        B = std::min(2 * B, 256);
    }
    const int L = c->bi_host->lend, Dmax = c->bi_host->dmax;
    *L_out = L;

    // per-level totals for the byte model of the profiling hooks
    std::vector<unsigned long long> lte, lcnt;
    std::vector<int32_t> lmode;
    if (c->prof_on) {
        lte.resize(L + 1);
        lcnt.resize(L + 1);
        lmode.resize(L + 1);
        // one wait for the three per-level arrays and the depth-0 mask
        CU(cudaMemcpyAsync(lte.data(), c->d_level_te, (L + 1) * 8, cudaMemcpyDeviceToHost, s));
        CU(cudaMemcpyAsync(lcnt.data(), c->d_level_cnt, (L + 1) * 8, cudaMemcpyDeviceToHost, s));
        CU(cudaMemcpyAsync(lmode.data(), c->d_level_mode, (L + 1) * 4, cudaMemcpyDeviceToHost, s));
        CU(cudaMemcpyAsync(&c->bi_host->depth0mask, &c->bi->depth0mask, 8, cudaMemcpyDeviceToHost, s));
        CU(cudaStreamSynchronize(s));
        const double W = nsrc;
        for (size_t i = prof_first; i < c->prof.size(); i++) {
            ProfRec &r = c->prof[i];
            if (r.tag < 1 || r.tag > L) continue;  // steps past the last level: no work
            if (r.kind == KP_FWD_PUSH || r.kind == KP_FWD_PULL) {
                // the byte model goes to the direction that ran; the other launch returned at once
                const bool ran = (r.kind == KP_FWD_PUSH) == (lmode[r.tag] != 0);
                r.bytes = ran ? (double)lte[r.tag - 1] * (4.0 / W + 4.0) : 0.0;
            } else if (r.kind == KP_LEVEL_STATS) {
                r.bytes = (double)n * 16.0;
            }
        }
    }

    // backward: depths Dmax .. 0 (depth 0 only for pivots whose BFS ended at level 2)
    unsigned long long depth0 = 0;
    if (Dmax >= 0) {
        for (int d = Dmax; d >= 0; d--) {
            if (!prof) {
                CU(cudaGraphLaunch(c->bwd_step_exec[K - 1], s));
                c->launches += g->bfwd.n_heavy ? 3 : 2;
                continue;
            }
            if (d == Dmax && c->prof_on) depth0 = c->bi_host->depth0mask;
            const double W = nsrc;
            double bytes = 0.0;
            if (c->prof_on) {
                double te_d = (double)lte[d], cnt_d = (double)lcnt[d];
                if (d == 0) {
                    const double frac = (double)__builtin_popcountll(depth0) / W;
                    te_d *= frac;
                    cnt_d *= frac;
                }
                bytes = d == Dmax ? cnt_d * 4.0 : te_d * (4.0 / W + 8.0);
            }
            {
                ProfScope ps(c, KP_BWD, bytes);
                if (c->prof_on) c->prof.back().tag = d;
                if (wc)
                    k_bwd_step<K, true><<<dim3(bwd_grid<K>(c), K), BATCH_TPB, 0, s>>>(
                        g->bfwd, c->bi, c->fmtab, c->msigma, c->mdelta, c->mq, c->mpartial, g->breach, c->ctrs, ll,
                        wc + KP_BWD * WC_NFIELDS);
                else
                    k_bwd_step<K, false><<<dim3(bwd_grid<K>(c), K), BATCH_TPB, 0, s>>>(
                        g->bfwd, c->bi, c->fmtab, c->msigma, c->mdelta, c->mq, c->mpartial, g->breach, c->ctrs, ll,
                        nullptr);
            }
            if (g->bfwd.n_heavy) {
                ProfScope ps(c, KP_BWD_COMBINE, 0);
                k_bwd_combine_step<K><<<dim3((g->bfwd.n_heavy + 7) / 8, K), 256, 0, s>>>(
                    g->bfwd, c->bi, c->fmtab, c->msigma, c->mdelta, c->mq, c->mpartial, g->breach, ll);
            }
            k_bwd_advance<<<1, 1, 0, s>>>(c->bi);
            c->launches++;
        }
        CU_LAUNCH("backward levels");
    }
    return AXBC_OK;
}

// Whether this batch runs as one persistent launch: always or never when the
// context says so; otherwise for a batch of at most AXBC_PERSIST_AUTO_WIDTH
// pivots when the last batch was deep, or -- for the first batch -- when no
// vertex has more than 64 neighbours (meshes and road-like graphs, whose many
// levels are narrow).  Measured on the 1024^2 grid (wall clock, 32 pivots per
// run): width 1 41.8 -> 32.8 ms, width 4 32.2 -> 26.0, width 8 34.3 -> 30.2,
// width 16 42.1 -> 40.2, width 32 even; on shallow graphs the step kernels'
// fuller grids win.  Counting runs use the step kernels.
static bool use_persist(axbc_ctx *c, int nsrc)
{
    if (c->count_on || c->persist_mode < 0) return false;
    if (c->persist_mode > 0) return true;
    if (nsrc > AXBC_PERSIST_AUTO_WIDTH) return false;
    if (c->last_batch_levels > AXBC_PERSIST_AUTO_LEVELS) return true;
    return c->last_batch_levels == 0 && c->g->max_deg <= 64;
}

// The batch's levels in k_traverse_persist: a cooperative launch of every
// block that fits resident (at most persist_blocks_per_sm per SM).  Level masks
// are allocated up front for the last batch's depth and grown when the loop
// asks for more.  *L_out: the first level that discovered nothing.
template <int K> static int traverse_persistent(axbc_ctx *c, int *L_out)
{
    axbc_graph *g = c->g;
    cudaStream_t s = c->stream;
    ALLOC_MISSING(c->gsync, sizeof(GridSync), &c->bytes);
    int bps = 0;
    CU(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&bps, k_traverse_persist<K>, BATCH_TPB, 0));
    bps = std::min(bps, std::max(1, c->persist_blocks_per_sm));
    if (bps < 1) {
        axbc_set_error("persistent level loop: no block of it fits on an SM");
        return AXBC_ERR_CUDA;
    }
    int grid = (c->num_sms > 0 ? c->num_sms : 152) * bps;
    const LevelLists ll = lists_of(c);
    const uint32_t lmax_list = list_max_of(c);
    const uint32_t pool_cap = c->lpool_cap;
    const uint64_t n = g->n;
    long long budget = AXBC_BAR_BUDGET;
    int levels = std::max(16, c->last_batch_levels + 8);
    GridSync hs;
    for (;;) {
        levels = std::min(levels, AXBC_MAX_LEVELS - 2);
        TRY(axbc_batch_levels_alloc(c, levels));
        c->prev_lend = levels - 1;  // masks the loop may write, cleared before the next batch
        CU(cudaMemsetAsync(c->gsync, 0, sizeof(GridSync), s));
        int lmax = levels;
        void *args[] = {(void *)&g->bfwd, (void *)&g->brev, (void *)&c->bi, (void *)&c->fmtab,
                        (void *)&c->seen, (void *)&c->msigma, (void *)&c->mdelta, (void *)&c->mq,
                        (void *)&c->mpartial, (void *)&g->breach, (void *)&c->ctrs, (void *)&ll,
                        (void *)&c->d_level_te, (void *)&c->d_level_cnt, (void *)&c->d_level_mode,
                        (void *)&pool_cap, (void *)&lmax_list, (void *)&n, (void *)&lmax,
                        (void *)&c->gsync, (void *)&budget};
        {
            ProfScope ps(c, KP_PERSIST, 0);
            CU(cudaLaunchCooperativeKernel((const void *)k_traverse_persist<K>, grid, BATCH_TPB, args, 0, s));
        }
        CU_LAUNCH("k_traverse_persist");
        CU(cudaMemcpyAsync(&hs, c->gsync, sizeof(GridSync), cudaMemcpyDeviceToHost, s));
        CU(cudaStreamSynchronize(s));
        if (hs.err) {
            axbc_set_error("persistent level loop: a grid barrier wait ran out of its budget (site %d)", hs.err);
            return AXBC_ERR_TIMEOUT;
        }
        if (!hs.need) break;
        if (levels >= AXBC_MAX_LEVELS - 2) {
            axbc_set_error("traversal deeper than %d levels", AXBC_MAX_LEVELS - 2);
            return AXBC_ERR_RANGE;
        }
        levels *= 2;
    }
    const size_t ctl_off = offsetof(BatchInfo, cur);
    const size_t ctl_len = offsetof(BatchInfo, push_factor) - ctl_off;
    CU(cudaMemcpyAsync((char *)c->bi_host + ctl_off, (char *)c->bi + ctl_off, ctl_len, cudaMemcpyDeviceToHost, s));
    CU(cudaStreamSynchronize(s));
    *L_out = c->bi_host->lend;
    return AXBC_OK;
}

// Forward and backward passes of the batch of width K whose roots/p are in
// c->bi.  The host launches forward level steps in blocks (8, then doubling)
// and reads the level state once per block; steps past the last level do
// nothing.
template <int K> static int batch_traverse(axbc_ctx *c, int nsrc, int H)
{
    axbc_graph *g = c->g;
    const uint64_t n = g->n;
    cudaStream_t s = c->stream;
    const int sgrid = axbc_grid_for(c, BATCH_TPB, 8);
    TRY(occupancy<K>(c));
    // per-launch mode: profiling events around each kernel, or the counting builds
    const bool prof = c->prof_on || c->count_on;
    TRY(ensure_level_tables(c));
    TRY(axbc_batch_levels_alloc(c, 10));
    if (!prof) TRY(capture_steps<K>(c, sgrid));

    // the previous batch's level masks back to zero (in its own width), then a
    // larger list pool if that batch ran out of list space
    if (c->prev_lend >= 2) {
        if (c->last_batch_k == 2)
            k_clean_levels<2><<<axbc_grid_for(c, 256, 2), 256, 0, s>>>(c->fmtab, c->lpool, c->lstart, c->lcount,
                                                                     c->lcap, n, 2, c->prev_lend);
        else
            k_clean_levels<1><<<axbc_grid_for(c, 256, 2), 256, 0, s>>>(c->fmtab, c->lpool, c->lstart, c->lcount,
                                                                     c->lcap, n, 2, c->prev_lend);
        CU_LAUNCH("k_clean_levels");
        c->launches++;
    }
    c->prev_lend = 0;
    TRY(axbc_batch_settle(c));
    const uint64_t pool_limit = (uint64_t)AXBC_WMAX * n + 64;
    if (c->pool_short && c->lpool_cap < pool_limit) {
        // the larger pool is allocated before the old one goes, so a failed
        // allocation leaves the context with a usable (smaller) pool
        const uint32_t ncap = (uint32_t)std::min<uint64_t>(std::min<uint64_t>(4ull * c->lpool_cap, pool_limit),
                                                           0xffffffffull);
        uint32_t *np = nullptr;
        TRY(axbc_dalloc((void **)&np, (uint64_t)ncap * 4, &c->bytes));
        CU(cudaStreamSynchronize(s));
        axbc_dfree(c->lpool);
        c->lpool = np;
        c->lpool_cap = ncap;
        c->pool_short = false;
        drop_captures(c);
        if (!prof) TRY(capture_steps<K>(c, sgrid));
    }
    c->last_batch_k = K;
    CU(cudaMemsetAsync(c->seen, 0, n * 4 * K, s));
    CU(cudaMemsetAsync(c->fmask[0], 0, n * 4 * K, s));
    CU(cudaMemsetAsync(c->fmask[1], 0, n * 4 * K, s));
    CU(cudaMemsetAsync(c->msigma, 0, n * AXBC_W * K * 4, s));
    CU(cudaMemsetAsync(c->ctrs, 0, 2 * AXBC_WMAX / 32 * AXBC_MAX_LEVELS * 4, s));
    CU(cudaMemsetAsync(c->lcount, 0, AXBC_MAX_LEVELS * 4, s));
    CU(cudaMemsetAsync(c->lheavy, 0, AXBC_MAX_LEVELS * 4, s));
    const LevelLists ll = lists_of(c);
    const uint32_t lmax = list_max_of(c);
    {
        ProfScope ps(c, KP_LEVEL_STATS, 0);
        k_batch_init<K><<<1, 32, 0, s>>>(c->bi, nsrc, H, c->bc, c->fmask[0], c->seen, c->msigma, g->bfwd.col,
                                         g->brev.col, g->m, c->push_factor_batch,
                                         // a factor of 1e30 or more pulls every level
                                         c->push_factor_batch >= 1e30 ? 0ull : (unsigned long long)(n / 4),
                                         c->d_level_te, c->d_level_cnt, ll, c->lpool_cap, lmax, g->to_view);
    }
    CU_LAUNCH("k_batch_init");

    int L = 0;
    if (use_persist(c, nsrc)) TRY(traverse_persistent<K>(c, &L));
    else TRY(traverse_stepwise<K>(c, nsrc, sgrid, &L));
    // the per-pivot level counts and the list-pool flag arrive in the
    // background; the next batch (or a caller that reports them) waits for them
    if (!c->rb_ev) CU(cudaEventCreateWithFlags(&c->rb_ev, cudaEventDisableTiming));
    CU(cudaMemcpyAsync(c->bi_host->Ls, c->bi->Ls, sizeof(c->bi_host->Ls), cudaMemcpyDeviceToHost, s));
    CU(cudaMemcpyAsync(&c->bi_host->pool_short, &c->bi->pool_short, 4, cudaMemcpyDeviceToHost, s));
    CU(cudaEventRecord(c->rb_ev, s));
    c->rb_pending = true;
    c->last_batch_levels = L;
    c->last_batch_nsrc = nsrc;
    c->prev_lend = L;
    return AXBC_OK;
}

// A multi-source pass of nsrc <= 64 pivots: 32-bit masks up to 32 pivots,
// 64-bit masks above.
int axbc_batch_traverse(axbc_ctx *c, int nsrc, int H)
{
    if (nsrc < 1 || nsrc > AXBC_WMAX) {
        axbc_set_error("batched pass of %d pivots (1..%d)", nsrc, AXBC_WMAX);
        return AXBC_ERR_INVALID;
    }
    return width_k(nsrc) == 2 ? batch_traverse<2>(c, nsrc, H) : batch_traverse<1>(c, nsrc, H);
}

int axbc_batch_settle(axbc_ctx *c)
{
    if (!c->rb_pending) return AXBC_OK;
    CU(cudaEventSynchronize(c->rb_ev));
    c->rb_pending = false;
    c->pool_short = c->bi_host->pool_short != 0;
    for (int i = 0; i < AXBC_WMAX; i++) c->last_Ls[i] = i < c->last_batch_nsrc ? c->bi_host->Ls[i] : 0;
    return AXBC_OK;
}

// The update of the applied lanes into each lane's bc vector, then the last
// applied dependency vector of each lane segment [lane_lo[i], lane_hi[i]) into
// delta_out[i] (defaults: one segment of all lanes into the context's).
template <int K>
static int apply_lanes(axbc_ctx *c, float *const *delta_out, const int *lane_lo, const int *lane_hi, int nseg)
{
    axbc_graph *g = c->g;
    cudaStream_t s = c->stream;
    // a grid-stride loop: exactly the blocks that stay resident
    if (!c->upd_blocks_per_sm[K - 1]) {
        int b = 0;
        CU(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, k_update_m<K>, UPD_TPB(K), 0));
        c->upd_blocks_per_sm[K - 1] = std::max(1, b);
    }
    const int grid = axbc_grid_for(c, UPD_TPB(K), c->upd_blocks_per_sm[K - 1]);
    const bool one_seg = nseg == 1 && (!lane_lo || lane_lo[0] == 0) && (!lane_hi || lane_hi[0] >= AXBC_W * K);
    {
        ProfScope ps(c, KP_UPDATE, (double)g->n * c->last_batch_nsrc * 20.0);
        // one segment over all lanes: the update writes the last delta itself
        k_update_m<K><<<grid, UPD_TPB(K), 0, s>>>(c->mdelta, c->seen, g->breach, g->n, c->bi,
                                                  one_seg ? (delta_out ? delta_out[0] : c->delta_last) : nullptr,
                                                  g->from_view);
    }
    for (int i = 0; i < nseg && !one_seg; i++) {
        ProfScope ps(c, KP_UPDATE, 0);
        k_extract_delta<K><<<grid, 256, 0, s>>>(delta_out ? delta_out[i] : c->delta_last, c->mdelta, c->seen,
                                                g->breach, g->n, c->bi, lane_lo ? lane_lo[i] : 0,
                                                lane_hi ? lane_hi[i] : AXBC_WMAX, g->from_view);
    }
    CU_LAUNCH("update");
    c->delta_last_valid = true;
    return AXBC_OK;
}

int axbc_batch_apply_lanes(axbc_ctx *c, float *const *delta_out, const int *lane_lo,
                           const int *lane_hi, int nseg)
{
    return c->last_batch_k == 2 ? apply_lanes<2>(c, delta_out, lane_lo, lane_hi, nseg)
                                : apply_lanes<1>(c, delta_out, lane_lo, lane_hi, nseg);
}

// Per forward level of the last batch: vertices newly reached (over all
// pivots), their degree sum, the direction (1 push), and the level's vertex
// list (entries counted, capacity; count > capacity: the level was scanned).
extern "C" int axbc_ctx_level_stats(axbc_ctx *c, uint64_t *count, uint64_t *te, int32_t *push,
                                    uint32_t *list_count, uint32_t *list_cap, int max_levels,
                                    int *levels)
{
    CHECK_ARG(c && levels, "axbc_ctx_level_stats: null argument");
    const int L = std::min(c->last_batch_levels + 1, max_levels);
    *levels = c->last_batch_levels + 1;
    if (!c->d_level_cnt || L <= 0) return AXBC_OK;
    CU(cudaStreamSynchronize(c->stream));
    if (count) CU(cudaMemcpy(count, c->d_level_cnt, L * 8, cudaMemcpyDeviceToHost));
    if (te) CU(cudaMemcpy(te, c->d_level_te, L * 8, cudaMemcpyDeviceToHost));
    if (push) CU(cudaMemcpy(push, c->d_level_mode, L * 4, cudaMemcpyDeviceToHost));
    if (list_count) CU(cudaMemcpy(list_count, c->lcount, L * 4, cudaMemcpyDeviceToHost));
    if (list_cap) CU(cudaMemcpy(list_cap, c->lcap, L * 4, cudaMemcpyDeviceToHost));
    return AXBC_OK;
}

int axbc_batch_apply(axbc_ctx *c) { return axbc_batch_apply_lanes(c, nullptr, nullptr, nullptr, 1); }

__global__ void k_set_lane_targets(BatchInfo *bi, LaneTargets t)
{
    if (threadIdx.x < AXBC_WMAX) bi->lane_bc[threadIdx.x] = t.bc[threadIdx.x];
}

// bc_of_lane: AXBC_WMAX vectors, one per lane of the pass
int axbc_batch_set_targets(axbc_ctx *c, float *const *bc_of_lane)
{
    LaneTargets t;
    for (int i = 0; i < AXBC_WMAX; i++) t.bc[i] = bc_of_lane[i];
    k_set_lane_targets<<<1, AXBC_WMAX, 0, c->stream>>>(c->bi, t);
    CU_LAUNCH("k_set_lane_targets");
    return AXBC_OK;
}

extern "C" int axbc_run_batch(axbc_ctx *c, const uint32_t *v0, const double *p, int k, int H,
                              axbc_pivot_stats *stats)
{
    CHECK_ARG(c && v0 && p, "axbc_run_batch: null argument");
    CHECK_ARG(k >= 1 && k <= AXBC_MAX_BATCH, "axbc_run_batch: k must be in [1, 64]");
    CHECK_ARG(H == 0 || H == 1, "axbc_run_batch: H must be 0 or 1");
    for (int i = 0; i < k; i++) CHECK_ARG(v0[i] < c->g->n, "axbc_run_batch: pivot >= n");
    TRY(axbc_ensure_batch(c));
    cudaStream_t s = c->stream;
    for (int i = 0; i < k; i++) {
        c->bi_host->root[i] = v0[i];
        c->bi_host->p[i] = p[i];
    }
    CU(cudaMemcpyAsync(&c->bi->root, c->bi_host->root, sizeof(c->bi_host->root),
                       cudaMemcpyHostToDevice, s));
    CU(cudaMemcpyAsync(&c->bi->p, c->bi_host->p, sizeof(c->bi_host->p), cudaMemcpyHostToDevice, s));
    TRY(axbc_batch_traverse(c, k, H));
    TRY(axbc_batch_apply(c));
    TRY(axbc_batch_settle(c));
    if (stats) {
        CU(cudaMemcpyAsync(c->bi_host, c->bi, sizeof(BatchInfo), cudaMemcpyDeviceToHost, s));
        std::vector<uint32_t> rr(k);
        for (int i = 0; i < k; i++)
            CU(cudaMemcpyAsync(&rr[i], c->g->reach + v0[i], 4, cudaMemcpyDeviceToHost, s));
        CU(cudaStreamSynchronize(s));
        for (int i = 0; i < k; i++) {
            stats[i].nvisited = c->bi_host->nvis[i];
            stats[i].all = (H == 1 ? (uint32_t)c->bi_host->rsum[i] : 0u) + rr[i];
            stats[i].te = 2 * c->bi_host->te[i];
            stats[i].levels = c->last_Ls[i];
            stats[i].pad = 0;
        }
    }
    return AXBC_OK;
}

extern "C" int axbc_get_batch_source(axbc_ctx *c, int src, uint32_t *sigma_host, int32_t *lvl_host,
                                     float *delta_host)
{
    CHECK_ARG(c && c->seen, "axbc_get_batch_source: no batch has run");
    CHECK_ARG(src >= 0 && src < c->last_batch_nsrc, "axbc_get_batch_source: bad source index");
    const uint64_t n = c->g->n;
    cudaStream_t s = c->stream;
    const int levels = c->last_batch_levels + 1;
    uint32_t **d_fm = nullptr;
    uint32_t *sig = nullptr;
    int32_t *lvl = nullptr;
    float *dl = nullptr;
    TRY(axbc_dalloc((void **)&d_fm, levels * sizeof(uint32_t *), nullptr));
    TRY(axbc_dalloc((void **)&sig, n * 4, nullptr));
    TRY(axbc_dalloc((void **)&lvl, n * 4, nullptr));
    TRY(axbc_dalloc((void **)&dl, n * 4, nullptr));
    CU(cudaMemcpyAsync(d_fm, c->fmask.data(), levels * sizeof(uint32_t *), cudaMemcpyHostToDevice, s));
    unsigned long long depth0 = 0;
    CU(cudaMemcpyAsync(&depth0, &c->bi->depth0mask, 8, cudaMemcpyDeviceToHost, s));
    CU(cudaStreamSynchronize(s));
    if (c->last_batch_k == 2)
        k_source_view<2><<<axbc_grid_for(c, 256, 4), 256, 0, s>>>(src, levels, d_fm, c->seen, c->msigma, c->mdelta,
                                                                  c->g->breach, n, depth0, sig, lvl, dl,
                                                                  c->g->from_view);
    else
        k_source_view<1><<<axbc_grid_for(c, 256, 4), 256, 0, s>>>(src, levels, d_fm, c->seen, c->msigma, c->mdelta,
                                                                  c->g->breach, n, depth0, sig, lvl, dl,
                                                                  c->g->from_view);
    CU_LAUNCH("k_source_view");
    if (sigma_host) CU(cudaMemcpyAsync(sigma_host, sig, n * 4, cudaMemcpyDeviceToHost, s));
    if (lvl_host) CU(cudaMemcpyAsync(lvl_host, lvl, n * 4, cudaMemcpyDeviceToHost, s));
    if (delta_host) CU(cudaMemcpyAsync(delta_host, dl, n * 4, cudaMemcpyDeviceToHost, s));
    CU(cudaStreamSynchronize(s));
    axbc_dfree(d_fm);
    axbc_dfree(sig);
    axbc_dfree(lvl);
    axbc_dfree(dl);
    return AXBC_OK;
}

// ------------------------------------------------------------ self-test
// The update's fast float(double(x)/p) against the double divide on n
// generated (x, p) pairs: random magnitudes, random bit patterns, and x*p
// products chosen to land next to float rounding midpoints.
__device__ __forceinline__ uint64_t st_mix(uint64_t z)
{
    z += 0x9E3779B97F4A7C15ull;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

__global__ void k_selftest_div(uint64_t n, uint64_t seed, unsigned long long *bad,
                               unsigned long long *slow)
{
    unsigned long long nb = 0, ns = 0;
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n;
         i += (uint64_t)gridDim.x * blockDim.x) {
        const uint64_t h1 = st_mix(seed ^ (i * 3 + 1)), h2 = st_mix(seed ^ (i * 3 + 2));
        float x;
        double p;
        switch (i % 6) {
        case 0:  // pivot probabilities: 1/N-like and products of small integers
            x = (float)((h1 & 0xffffff) + 1) * ldexpf(1.0f, (int)((h1 >> 24) & 31) - 16);
            p = 1.0 / (double)((h2 & 0xffffff) + 1);
            break;
        case 1:  // random float bits (positive, normal), random double p in (0,1]
            x = __uint_as_float(((uint32_t)(h1 & 0x7fffffff) % 0x7f000000u) | 0x00800000u);
            p = (double)((h2 >> 11) + 1) * 0x1.0p-53;
            break;
        case 2: {  // near midpoints: x/p = m + half ulp(m) +- tiny
            const float m = (float)((h1 & 0xffffff) | 0x800000) * ldexpf(1.0f, (int)((h1 >> 24) & 15) - 8);
            p = (double)((h2 >> 11) + 1) * 0x1.0p-53 + 1e-9;
            const double target = ((double)m + (double)m * 0x1.0p-24) * (1.0 + ((int)(h2 & 7) - 3) * 0x1.0p-50);
            x = (float)(target * p);
            break;
        }
        case 3:  // integers times integers
            x = (float)((h1 & 0xfffff) + 1);
            p = (double)((h2 & 0xfff) + 1) / (double)((h2 >> 12 & 0xfffff) + 1);
            break;
        case 4:  // exact powers of two: small integers over p = 2^-k
            x = (float)((h1 & 15) + 1) * ldexpf(1.0f, (int)((h1 >> 4) & 15) - 8);
            p = ldexp(1.0, -(int)(h2 & 31));
            break;
        default: {  // just below a power of two, around the quarter-ulp boundary
            p = (double)((h2 >> 11) + 1) * 0x1.0p-53 + 1e-9;
            const double pw = ldexp(1.0, (int)(h1 & 31) - 8);
            const double target = pw * (1.0 - 0x1.0p-26 * (1.0 + ((int)((h1 >> 5) & 15) - 8) * 0x1.0p-20));
            x = (float)(target * p);
        }
        }
        if (!(x > 0.0f) || !(p > 0.0)) continue;
        const InvSplit iv = inv_split(p);
        const float f = div_to_float(x, p, iv);
        const float e = __double2float_rn(__ddiv_rn((double)x, p));
        if (__float_as_uint(f) != __float_as_uint(e)) nb++;
        // count how often the exact path decided
        const float a = __fmul_rn(x, iv.hi);
        const float ee = __fmaf_rn(x, iv.hi, -a);
        const float b = __fmaf_rn(x, iv.lo, ee);
        const float s = __fadd_rn(a, b);
        if (!iv.ok || __float_as_uint(s) != __float_as_uint(f)) ns++;
    }
    if (nb) atomicAdd(bad, nb);
    if (ns) atomicAdd(slow, ns);
}

extern "C" int axbc_selftest_division(uint64_t n, uint64_t seed, uint64_t *mismatches,
                                      uint64_t *exact_path)
{
    CHECK_ARG(mismatches, "axbc_selftest_division: null argument");
    unsigned long long *d = nullptr;
    TRY(axbc_dalloc((void **)&d, 16, nullptr));
    CU(cudaMemset(d, 0, 16));
    k_selftest_div<<<1024, 256>>>(n, seed, d, d + 1);
    CU_LAUNCH("k_selftest_div");
    unsigned long long h[2];
    CU(cudaMemcpy(h, d, 16, cudaMemcpyDeviceToHost));
    axbc_dfree(d);
    *mismatches = h[0];
    if (exact_path) *exact_path = h[1];
    return AXBC_OK;
}

// ------------------------------------------------ persistent loop controls
extern "C" int axbc_ctx_set_persistent(axbc_ctx *c, int mode, int blocks_per_sm)
{
    CHECK_ARG(c, "axbc_ctx_set_persistent: null context");
    CHECK_ARG(mode >= -1 && mode <= 1, "axbc_ctx_set_persistent: mode must be -1, 0 or 1");
    CHECK_ARG(blocks_per_sm >= 0 && blocks_per_sm <= 8, "axbc_ctx_set_persistent: blocks_per_sm must be in [0, 8]");
    if (mode > 0) {
        int dev = 0, coop = 0;
        CU(cudaGetDevice(&dev));
        CU(cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, dev));
        if (!coop) {
            axbc_set_error("axbc_ctx_set_persistent: the device has no cooperative launch");
            return AXBC_ERR_INVALID;
        }
    }
    c->persist_mode = mode;
    if (blocks_per_sm > 0) c->persist_blocks_per_sm = blocks_per_sm;
    return AXBC_OK;
}

extern "C" int axbc_selftest_grid_barrier(int blocks_per_sm, int rounds, long long budget_cycles,
                                          int absent_block, int *err_site, uint32_t *leads, float *ms)
{
    CHECK_ARG(err_site && leads, "axbc_selftest_grid_barrier: null argument");
    CHECK_ARG(rounds >= 1 && budget_cycles > 0, "axbc_selftest_grid_barrier: bad rounds or budget");
    int dev = 0, sms = 0, fit = 0;
    CU(cudaGetDevice(&dev));
    CU(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    CU(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&fit, k_barrier_selftest, BATCH_TPB, 0));
    CHECK_ARG(blocks_per_sm >= 1 && blocks_per_sm <= fit, "axbc_selftest_grid_barrier: blocks_per_sm does not fit");
    int grid = sms * blocks_per_sm;
    CHECK_ARG(absent_block < grid, "axbc_selftest_grid_barrier: absent_block beyond the grid");
    DBuf gs, out;
    TRY(gs.alloc(sizeof(GridSync)));
    TRY(out.alloc(4));
    CU(cudaMemset(gs.p, 0, sizeof(GridSync)));
    CU(cudaMemset(out.p, 0, 4));
    cudaEvent_t a, b;
    CU(cudaEventCreate(&a));
    CU(cudaEventCreate(&b));
    GridSync *gsp = gs.as<GridSync>();
    unsigned *outp = out.as<unsigned>();
    void *args[] = {(void *)&gsp, (void *)&rounds, (void *)&budget_cycles, (void *)&absent_block, (void *)&outp};
    CU(cudaEventRecord(a, 0));
    cudaError_t e = cudaLaunchCooperativeKernel((const void *)k_barrier_selftest, grid, BATCH_TPB, args, 0, 0);
    if (e == cudaSuccess) e = cudaEventRecord(b, 0);
    if (e == cudaSuccess) e = cudaEventSynchronize(b);
    float t = 0;
    if (e == cudaSuccess) e = cudaEventElapsedTime(&t, a, b);
    cudaEventDestroy(a);
    cudaEventDestroy(b);
    if (e != cudaSuccess) return axbc_cuda_fail(e, "k_barrier_selftest", __FILE__, __LINE__);
    GridSync h;
    CU(cudaMemcpy(&h, gs.p, sizeof(h), cudaMemcpyDeviceToHost));
    CU(cudaMemcpy(leads, out.p, 4, cudaMemcpyDeviceToHost));
    *err_site = h.err;
    if (ms) *ms = t;
    return AXBC_OK;
}
