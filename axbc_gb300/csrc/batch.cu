// Batched form: up to 32 pivots in one multi-source pass.  Lane s of a warp
// owns pivot s; every vertex carries one 32-bit mask per BFS level (bit s:
// the vertex is at that depth from pivot s), a `seen` mask, and per-pivot path
// counts / dependencies laid out [vertex][32] so the 32 lanes touch one
// 128-byte line.  Results equal those of the plain form bit for bit: path
// counts are integers, and each lane accumulates its dependency sum in the
// canonical order (32-position chunks summed as a tree in registers, chunks
// then spans left to right).
#include <algorithm>
#include <cstddef>
#include <vector>

#include "common.cuh"

#define BATCH_TPB 256

static __device__ __forceinline__ uint64_t row_base(uint64_t v) { return v * AXBC_W; }

// roots: depth 0, sigma 1 (set_mlp_cuda, src/cuda_kernels.cu:862-876)
__global__ void k_batch_init(BatchInfo *bi, int nsrc, int H, uint32_t *fmask0, uint32_t *seen,
                             uint32_t *msigma, const uint32_t *__restrict__ col,
                             const uint32_t *__restrict__ rcol, unsigned long long m)
{
    const int s = threadIdx.x;
    if (s == 0) {
        bi->nsrc = nsrc;
        bi->napply = nsrc;
        bi->srcmask = nsrc >= 32 ? FULL_MASK : ((1u << nsrc) - 1u);
        bi->depth0mask = 0;
        bi->H = H;
    }
    unsigned long long fd = 0, rd = 0;
    if (s < nsrc) {
        const uint32_t v = bi->root[s];
        atomicOr(&fmask0[v], 1u << s);
        atomicOr(&seen[v], 1u << s);
        msigma[row_base(v) + s] = 1;
        bi->nvis[s] = 1;
        bi->rsum[s] = 0;
        bi->te[s] = col[v + 1] - col[v];
        fd = col[v + 1] - col[v];
        rd = rcol[v + 1] - rcol[v];
    } else if (s < AXBC_W) {
        bi->nvis[s] = 0;
        bi->rsum[s] = 0;
        bi->te[s] = 0;
    }
    for (int o = 16; o; o >>= 1) {
        fd += __shfl_xor_sync(FULL_MASK, fd, o);
        rd += __shfl_xor_sync(FULL_MASK, rd, o);
    }
    if (s == 0) {
        bi->front_deg = fd;
        bi->unvis_deg = m - rd;
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

__host__ __device__ __forceinline__ uint64_t n_units(const Adj &a)
{
    return a.n_heavy_items + (a.n_ltask + LIGHT_PER_UNIT - 1) / LIGHT_PER_UNIT;
}

// Forward level L, push from the vertices of depth L-1: for each neighbour u
// and each pivot s with v at depth L-1 and u unseen, sigma_s[u] += sigma_s[v]
// and bit s joins u's level-L mask.  Atomics are fire-and-forget reductions.
__device__ __forceinline__ void push_span(const Adj &a, uint32_t v, uint32_t f, uint32_t b0,
                                          uint32_t b1, const uint32_t *__restrict__ seen,
                                          uint32_t *fcur, uint32_t *msigma)
{
    const unsigned lane = lane_id();
    const uint32_t sig = ((f >> lane) & 1u) ? msigma[row_base(v) + lane] : 0u;
    for (uint32_t base = b0; base < b1; base += 32) {
        const uint32_t e = base + lane;
        uint32_t u = 0, nm = 0;
        if (e < b1) {
            u = a.row[e];
            nm = f & ~seen[u];
        }
        if (nm) atomicOr(&fcur[u], nm);
        unsigned act = __ballot_sync(FULL_MASK, nm != 0);
        while (act) {
            const int j = __ffs(act) - 1;
            act &= act - 1;
            const uint32_t uj = __shfl_sync(FULL_MASK, u, j);
            const uint32_t mj = __shfl_sync(FULL_MASK, nm, j);
            if ((mj >> lane) & 1u) atomicAdd(&msigma[row_base(uj) + lane], sig);
        }
    }
}

__global__ void __launch_bounds__(BATCH_TPB) k_fwd_push_m(Adj a, const uint32_t *__restrict__ fprev,
                                                          uint32_t *fcur,
                                                          const uint32_t *__restrict__ seen,
                                                          uint32_t *msigma, uint32_t *ctr)
{
    const unsigned lane = lane_id();
    const uint64_t nhi = a.n_heavy_items, nu = n_units(a);
    for (;;) {
        const uint32_t t = grab_unit(ctr);
        if (t >= nu) break;
        if (t < nhi) {
            const uint32_t v = a.hitem_v[t];
            const uint32_t f = fprev[v];
            if (!f) continue;
            const uint32_t b0 = a.col[v] + a.hitem_k[t] * AXBC_SPAN;
            push_span(a, v, f, b0, min(a.col[v + 1], b0 + AXBC_SPAN), seen, fcur, msigma);
            continue;
        }
        const uint64_t l0 = (uint64_t)(t - nhi) * LIGHT_PER_UNIT;
        for (uint64_t lt = l0; lt < l0 + LIGHT_PER_UNIT && lt < a.n_ltask; lt++) {
            const uint32_t beg = a.ltask[lt], cnt = a.ltask[lt + 1] - beg;
            uint32_t v_l = 0, f_l = 0;
            if (lane < cnt) {
                v_l = a.order[beg + lane];
                f_l = fprev[v_l];
            }
            unsigned act = __ballot_sync(FULL_MASK, f_l != 0);
            while (act) {
                const int j = __ffs(act) - 1;
                act &= act - 1;
                const uint32_t v = __shfl_sync(FULL_MASK, v_l, j);
                const uint32_t f = __shfl_sync(FULL_MASK, f_l, j);
                push_span(a, v, f, a.col[v], a.col[v + 1], seen, fcur, msigma);
            }
        }
    }
}

// Forward level L, pull into vertex u for the pivots `ns` that have not seen
// it: sum sigma_s over every in-neighbour at depth L-1 from pivot s.  The
// positions of a 32-wide chunk are staged in shared memory and their gathers
// issued eight at a time before any is consumed.
__device__ __forceinline__ uint32_t pull_span(const Adj &rv, uint32_t ns, uint32_t b0, uint32_t b1,
                                              const uint32_t *__restrict__ fprev,
                                              const uint32_t *__restrict__ msigma, uint32_t *su,
                                              uint32_t *sg, uint32_t &acc)
{
    const unsigned lane = lane_id();
    bool found = false;
    acc = 0;
    for (uint32_t base = b0; base < b1; base += 32) {
        const uint32_t e = base + lane;
        uint32_t v = 0, fm = 0;
        if (e < b1) {
            v = rv.row[e];
            fm = fprev[v] & ns;
        }
        unsigned act = __ballot_sync(FULL_MASK, fm != 0);
        if (!act) continue;
        su[lane] = v;
        sg[lane] = fm;
        __syncwarp();
        while (act) {
            uint32_t x[8];
            bool h[8];
#pragma unroll
            for (int q = 0; q < 8; q++) {
                const int j = act ? __ffs(act) - 1 : 0;
                const bool ok = act != 0;
                act &= act - 1;
                h[q] = ok && ((sg[j] >> lane) & 1u);
                x[q] = h[q] ? msigma[row_base(su[j]) + lane] : 0u;
            }
#pragma unroll
            for (int q = 0; q < 8; q++) {
                acc += x[q];
                found |= h[q];
            }
        }
        __syncwarp();
    }
    return __ballot_sync(FULL_MASK, found);
}

__global__ void __launch_bounds__(BATCH_TPB) k_fwd_pull_m(Adj rv, uint32_t srcmask,
                                                          const uint32_t *__restrict__ fprev,
                                                          uint32_t *fcur,
                                                          const uint32_t *__restrict__ seen,
                                                          uint32_t *msigma, uint32_t *ctr)
{
    __shared__ uint32_t s_u[BATCH_TPB], s_g[BATCH_TPB];
    const unsigned lane = lane_id();
    uint32_t *su = s_u + (threadIdx.x & ~31u), *sg = s_g + (threadIdx.x & ~31u);
    const uint64_t nhi = rv.n_heavy_items, nu = n_units(rv);
    for (;;) {
        const uint32_t t = grab_unit(ctr);
        if (t >= nu) break;
        if (t < nhi) {
            const uint32_t u = rv.hitem_v[t];
            const uint32_t ns = srcmask & ~seen[u];
            if (!ns) continue;
            const uint32_t b0 = rv.col[u] + rv.hitem_k[t] * AXBC_SPAN;
            uint32_t acc;
            const uint32_t nm =
                pull_span(rv, ns, b0, min(rv.col[u + 1], b0 + AXBC_SPAN), fprev, msigma, su, sg, acc);
            if ((nm >> lane) & 1u) atomicAdd(&msigma[row_base(u) + lane], acc);
            if (lane == 0 && nm) atomicOr(&fcur[u], nm);
            continue;
        }
        const uint64_t l0 = (uint64_t)(t - nhi) * LIGHT_PER_UNIT;
        for (uint64_t lt = l0; lt < l0 + LIGHT_PER_UNIT && lt < rv.n_ltask; lt++) {
            const uint32_t beg = rv.ltask[lt], cnt = rv.ltask[lt + 1] - beg;
            uint32_t u_l = 0, ns_l = 0;
            if (lane < cnt) {
                u_l = rv.order[beg + lane];
                if (rv.col[u_l + 1] > rv.col[u_l]) ns_l = srcmask & ~seen[u_l];
            }
            unsigned act = __ballot_sync(FULL_MASK, ns_l != 0);
            uint32_t mine = 0;
            while (act) {
                const int j = __ffs(act) - 1;
                act &= act - 1;
                const uint32_t u = __shfl_sync(FULL_MASK, u_l, j);
                const uint32_t ns = __shfl_sync(FULL_MASK, ns_l, j);
                uint32_t acc;
                const uint32_t nm =
                    pull_span(rv, ns, rv.col[u], rv.col[u + 1], fprev, msigma, su, sg, acc);
                if ((nm >> lane) & 1u) msigma[row_base(u) + lane] = acc;
                if ((int)lane == j) mine = nm;
            }
            if (mine) fcur[u_l] = mine;
        }
    }
}

// After level L: fold the level mask into `seen` and count, per pivot, the
// vertices reached, their degree sum and their reach sum.
__global__ void __launch_bounds__(BATCH_TPB) k_level_stats(uint64_t n, uint32_t srcmask,
                                                           const uint32_t *__restrict__ fcur,
                                                           uint32_t *seen,
                                                           const uint32_t *__restrict__ col,
                                                           const uint32_t *__restrict__ rcol,
                                                           const uint32_t *__restrict__ reach,
                                                           BatchInfo *bi)
{
    const unsigned lane = lane_id();
    const uint64_t nblk = (n + 31) / 32;
    const uint64_t nw = (uint64_t)gridDim.x * blockDim.x / 32;
    unsigned long long cnt = 0, te = 0, rs = 0, fdeg = 0, udeg = 0;
    bool any = false;
    for (uint64_t t = (blockIdx.x * (uint64_t)blockDim.x + threadIdx.x) / 32; t < nblk; t += nw) {
        const uint64_t u = t * 32 + lane;
        uint32_t nm = 0, d = 0, r = 0;
        if (u < n) {
            nm = fcur[u];
            uint32_t sn = seen[u];
            if (nm) {
                any = true;
                sn |= nm;
                seen[u] = sn;
                d = col[u + 1] - col[u];
                r = reach[u];
                fdeg += d;
            }
            if (srcmask & ~sn) udeg += rcol[u + 1] - rcol[u];
        }
        unsigned act = __ballot_sync(FULL_MASK, nm != 0);
        while (act) {
            const int j = __ffs(act) - 1;
            act &= act - 1;
            const uint32_t mj = __shfl_sync(FULL_MASK, nm, j);
            const uint32_t dj = __shfl_sync(FULL_MASK, d, j);
            const uint32_t rj = __shfl_sync(FULL_MASK, r, j);
            if ((mj >> lane) & 1u) {
                cnt++;
                te += dj;
                rs += rj;
            }
        }
    }
    {
        unsigned long long tsum = te;
        for (int o = 16; o; o >>= 1) tsum += __shfl_xor_sync(FULL_MASK, tsum, o);
        if (lane == 0 && tsum) atomicAdd(&bi->lvl_te, tsum);
    }
    if (cnt) {
        atomicAdd(&bi->lvl_new[lane], cnt);
        atomicAdd(&bi->nvis[lane], cnt);
        atomicAdd(&bi->te[lane], te);
        atomicAdd(&bi->rsum[lane], rs);
    }
    for (int o = 16; o; o >>= 1) {
        fdeg += __shfl_xor_sync(FULL_MASK, fdeg, o);
        udeg += __shfl_xor_sync(FULL_MASK, udeg, o);
    }
    any = __any_sync(FULL_MASK, any);
    if (lane == 0) {
        if (fdeg) atomicAdd(&bi->front_deg, fdeg);
        if (udeg) atomicAdd(&bi->unvis_deg, udeg);
        if (any) atomicOr(&bi->any_new, 1u);
    }
}

// Sum of the 8 staged successor terms of one group as a balanced tree (pairs
// differing in the lowest position bit first).  mq_l points at lane l of row 0.
__device__ __forceinline__ float tree8(const uint4 *su4, const uint4 *sg4, int g,
                                       const float *__restrict__ mq_l, float sv, uint32_t lanebit)
{
    const uint4 ua = su4[2 * g], ub = su4[2 * g + 1];
    const uint4 ga = sg4[2 * g], gb = sg4[2 * g + 1];
    const uint32_t u[8] = {ua.x, ua.y, ua.z, ua.w, ub.x, ub.y, ub.z, ub.w};
    const uint32_t m[8] = {ga.x, ga.y, ga.z, ga.w, gb.x, gb.y, gb.z, gb.w};
    float t[8];
#pragma unroll
    for (int jj = 0; jj < 8; jj++) {
        const bool h = (m[jj] & lanebit) != 0u;
        const float q = h ? mq_l[(uint64_t)u[jj] * AXBC_W] : 0.0f;
        t[jj] = h ? __fmul_rn(q, sv) : 0.0f;
    }
    const float a = __fadd_rn(__fadd_rn(t[0], t[1]), __fadd_rn(t[2], t[3]));
    const float b = __fadd_rn(__fadd_rn(t[4], t[5]), __fadd_rn(t[6], t[7]));
    return __fadd_rn(a, b);
}

// Canonical dependency sum of vertex v over adjacency positions [b0,b1) for
// the pivots in f.  q[u][s] = (delta_s[u] + 1) / sigma_s[u] was stored when
// u's dependency was final, so a successor term is q * sigma_s[v], bit for bit
// the reference's ((delta + 1) / sigma[r]) * sigma[c].  The 32 positions of a
// chunk form four 8-position subtrees of the canonical tree; a subtree without
// successors sums to +0 and is skipped.
__device__ __forceinline__ float dep_span(const Adj &a, uint32_t f, float sv, uint32_t b0,
                                          uint32_t b1, const uint32_t *__restrict__ fnext,
                                          const float *__restrict__ mq, uint32_t *su, uint32_t *sg)
{
    const unsigned lane = lane_id();
    const uint32_t lanebit = 1u << lane;
    const float *mq_l = mq + lane;
    const uint4 *su4 = reinterpret_cast<const uint4 *>(su);
    const uint4 *sg4 = reinterpret_cast<const uint4 *>(sg);
    float P = 0.0f;
    for (uint32_t base = b0; base < b1; base += 32) {
        const uint32_t e = base + lane;
        uint32_t u = 0, gm = 0;
        if (e < b1) {
            u = a.row[e];
            gm = fnext[u] & f;
        }
        const unsigned pm = __ballot_sync(FULL_MASK, gm != 0);
        if (!pm) continue;
        su[lane] = u;
        sg[lane] = gm;
        __syncwarp();
        float g0 = 0.0f, g1 = 0.0f, g2 = 0.0f, g3 = 0.0f;
        if (pm & 0x000000ffu) g0 = tree8(su4, sg4, 0, mq_l, sv, lanebit);
        if (pm & 0x0000ff00u) g1 = tree8(su4, sg4, 1, mq_l, sv, lanebit);
        if (pm & 0x00ff0000u) g2 = tree8(su4, sg4, 2, mq_l, sv, lanebit);
        if (pm & 0xff000000u) g3 = tree8(su4, sg4, 3, mq_l, sv, lanebit);
        P = __fadd_rn(P, __fadd_rn(__fadd_rn(g0, g1), __fadd_rn(g2, g3)));
        __syncwarp();
    }
    return P;
}

// delta and q of vertex v for the pivots in f
__device__ __forceinline__ void write_dep(float *mdelta, float *mq, uint32_t v, uint32_t f,
                                          float delta, uint32_t sig)
{
    const unsigned lane = lane_id();
    if ((f >> lane) & 1u) {
        mdelta[row_base(v) + lane] = delta;
        mq[row_base(v) + lane] = __fdiv_rn(__fadd_rn(delta, 1.0f), __uint2float_rn(sig));
    }
}

// Backward depth d for the pivots in dmask.  With no_succ (the deepest depth)
// nothing lies below, so delta = reach.
__global__ void __launch_bounds__(BATCH_TPB) k_bwd_m(Adj a, uint32_t dmask, int no_succ,
                                                     const uint32_t *__restrict__ fd,
                                                     const uint32_t *__restrict__ fnext,
                                                     const uint32_t *__restrict__ msigma,
                                                     float *mdelta, float *mq, float *mpartial,
                                                     const uint32_t *__restrict__ reach,
                                                     uint32_t *ctr)
{
    __shared__ __align__(16) uint32_t s_u[BATCH_TPB];
    __shared__ __align__(16) uint32_t s_g[BATCH_TPB];
    const unsigned lane = lane_id();
    uint32_t *su = s_u + (threadIdx.x & ~31u), *sg = s_g + (threadIdx.x & ~31u);
    const uint64_t nhi = a.n_heavy_items, nu = n_units(a);
    for (;;) {
        const uint32_t t = grab_unit(ctr);
        if (t >= nu) break;
        if (t < nhi) {
            const uint32_t v = a.hitem_v[t];
            const uint32_t f = fd[v] & dmask;
            if (!f) continue;
            float P = 0.0f;
            if (!no_succ) {
                const float sv = __uint2float_rn(((f >> lane) & 1u) ? msigma[row_base(v) + lane] : 0u);
                const uint32_t b0 = a.col[v] + a.hitem_k[t] * AXBC_SPAN;
                P = dep_span(a, f, sv, b0, min(a.col[v + 1], b0 + AXBC_SPAN), fnext, mq, su, sg);
            }
            mpartial[(uint64_t)t * AXBC_W + lane] = P;
            continue;
        }
        const uint64_t l0 = (uint64_t)(t - nhi) * LIGHT_PER_UNIT;
        for (uint64_t lt = l0; lt < l0 + LIGHT_PER_UNIT && lt < a.n_ltask; lt++) {
            const uint32_t beg = a.ltask[lt], cnt = a.ltask[lt + 1] - beg;
            uint32_t v_l = 0, f_l = 0;
            if (lane < cnt) {
                v_l = a.order[beg + lane];
                f_l = fd[v_l] & dmask;
            }
            unsigned act = __ballot_sync(FULL_MASK, f_l != 0);
            while (act) {
                const int j = __ffs(act) - 1;
                act &= act - 1;
                const uint32_t v = __shfl_sync(FULL_MASK, v_l, j);
                const uint32_t f = __shfl_sync(FULL_MASK, f_l, j);
                const uint32_t sig = ((f >> lane) & 1u) ? msigma[row_base(v) + lane] : 0u;
                float P = 0.0f;
                if (!no_succ)
                    P = dep_span(a, f, __uint2float_rn(sig), a.col[v], a.col[v + 1], fnext, mq, su, sg);
                write_dep(mdelta, mq, v, f, __fadd_rn(__uint2float_rn(reach[v]), P), sig);
            }
        }
    }
}

__global__ void k_bwd_combine_m(Adj a, uint32_t dmask, const uint32_t *__restrict__ fd,
                                const uint32_t *__restrict__ msigma, float *mdelta, float *mq,
                                const float *__restrict__ mpartial,
                                const uint32_t *__restrict__ reach)
{
    const unsigned lane = lane_id();
    const uint64_t nw = (uint64_t)gridDim.x * blockDim.x / 32;
    for (uint64_t i = (blockIdx.x * (uint64_t)blockDim.x + threadIdx.x) / 32; i < a.n_heavy; i += nw) {
        const uint32_t v = a.heavy_v[i];
        const uint32_t f = fd[v] & dmask;
        if (!f) continue;
        float acc = __uint2float_rn(reach[v]);
        for (uint32_t k = a.heavy_first[i]; k < a.heavy_first[i + 1]; k++)
            acc = __fadd_rn(acc, mpartial[(uint64_t)k * AXBC_W + lane]);
        const uint32_t sig = ((f >> lane) & 1u) ? msigma[row_base(v) + lane] : 0u;
        write_dep(mdelta, mq, v, f, acc, sig);
    }
}

// bc update for pivots 0..napply-1 in order (update_bc, src/cuda_kernels.cu:
// 269-286).  A pivot that did not reach v contributes delta = reach[v].  Zero
// terms are skipped: x + float(0/p) == x for p > 0.
__global__ void __launch_bounds__(BATCH_TPB) k_update_m(float *bc, const float *__restrict__ mdelta,
                                                        const uint32_t *__restrict__ seen,
                                                        const uint32_t *__restrict__ reach,
                                                        uint64_t n, const BatchInfo *__restrict__ bi)
{
    __shared__ uint32_t s_root[AXBC_W], s_reach[AXBC_W];
    __shared__ double s_p[AXBC_W];
    __shared__ unsigned long long s_nvt[AXBC_W];
    __shared__ InvSplit s_iv[AXBC_W];
    const uint32_t napply = bi->napply;
    if (threadIdx.x < AXBC_W) {
        const int s = threadIdx.x;
        if (s < (int)napply) {
            const uint32_t r = bi->root[s];
            const uint32_t rv = reach[r];
            const uint32_t all = (bi->H == 1 ? (uint32_t)bi->rsum[s] : 0u) + rv;
            s_root[s] = r;
            s_reach[s] = rv;
            s_p[s] = bi->p[s];
            s_nvt[s] = bi->nvis[s] + all;
            s_iv[s] = inv_split(bi->p[s]);
        } else {
            s_root[s] = 0xffffffffu;
            s_reach[s] = 0;
            s_p[s] = 1.0;
            s_nvt[s] = 2;
            s_iv[s] = inv_split(1.0);
        }
    }
    __syncthreads();
    if (napply == 0) return;
    for (uint64_t v = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; v < n;
         v += (uint64_t)gridDim.x * blockDim.x) {
        const uint32_t sv = seen[v];
        const uint32_t rv = reach[v];
        if (sv == 0 && rv == 0) {
            // unreached by every pivot with delta 0: only a root term could
            // apply, and roots are reached
            continue;
        }
        const float rf = __uint2float_rn(rv);
        const float4 *row = reinterpret_cast<const float4 *>(mdelta + row_base(v));
        float b = bc[v];
        for (int q = 0; q < AXBC_W / 4; q++) {
            if (4 * q >= (int)napply) break;
            float4 x = make_float4(rf, rf, rf, rf);
            if ((sv >> (4 * q)) & 0xfu) x = row[q];
            const float dq[4] = {x.x, x.y, x.z, x.w};
#pragma unroll
            for (int k = 0; k < 4; k++) {
                const int s = 4 * q + k;
                if (s >= (int)napply) break;
                if ((uint32_t)v == s_root[s]) {
                    if (s_reach[s] > 0) b = __fadd_rn(b, bc_root_term(s_reach[s], s_nvt[s]));
                    continue;
                }
                const float dv = ((sv >> s) & 1u) ? dq[k] : rf;
                if (dv == 0.0f && s_p[s] > 0.0) continue;
                b = __fadd_rn(b, bc_term_fast(dv, s_reach[s], s_p[s], s_iv[s]));
            }
        }
        bc[v] = b;
    }
}

// the last applied pivot's dependencies as a plain n-vector
__global__ void k_extract_delta(float *out, const float *__restrict__ mdelta,
                                const uint32_t *__restrict__ seen,
                                const uint32_t *__restrict__ reach, uint64_t n,
                                const BatchInfo *__restrict__ bi)
{
    const uint32_t napply = bi->napply;
    if (napply == 0) return;
    const int s = napply - 1;
    const uint32_t root = bi->root[s];
    const bool root_done = (bi->depth0mask >> s) & 1u;
    for (uint64_t v = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; v < n;
         v += (uint64_t)gridDim.x * blockDim.x) {
        bool have = (seen[v] >> s) & 1u;
        if (v == root) have = root_done;
        out[v] = have ? mdelta[row_base(v) + s] : __uint2float_rn(reach[v]);
    }
}

// one pivot of the last batch: path counts, depths, dependencies
__global__ void k_source_view(int s, int levels, uint32_t *const *fm, const uint32_t *__restrict__ seen,
                              const uint32_t *__restrict__ msigma, const float *__restrict__ mdelta,
                              const uint32_t *__restrict__ reach, uint64_t n, uint32_t depth0,
                              uint32_t *sig, int32_t *lvl, float *dl)
{
    for (uint64_t v = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; v < n;
         v += (uint64_t)gridDim.x * blockDim.x) {
        int L = -1;
        if ((seen[v] >> s) & 1u) {
            for (int l = 0; l < levels; l++)
                if ((fm[l][v] >> s) & 1u) {
                    L = l;
                    break;
                }
        }
        lvl[v] = L;
        sig[v] = L >= 0 ? msigma[row_base(v) + s] : 0u;
        bool have = L > 0 || (L == 0 && ((depth0 >> s) & 1u));
        dl[v] = have ? mdelta[row_base(v) + s] : __uint2float_rn(reach[v]);
    }
}

int axbc_batch_levels_alloc(axbc_ctx *c, int levels)
{
    while ((int)c->fmask.size() < levels) {
        uint32_t *p = nullptr;
        TRY(axbc_dalloc((void **)&p, c->g->n * 4, &c->bytes));
        c->fmask.push_back(p);
    }
    return AXBC_OK;
}

int axbc_ensure_batch(axbc_ctx *c)
{
    if (c->seen) return AXBC_OK;
    const uint64_t n = c->g->n;
    TRY(axbc_dalloc((void **)&c->seen, n * 4, &c->bytes));
    TRY(axbc_dalloc((void **)&c->msigma, n * AXBC_W * 4, &c->bytes));
    TRY(axbc_dalloc((void **)&c->mdelta, n * AXBC_W * 4, &c->bytes));
    TRY(axbc_dalloc((void **)&c->mq, n * AXBC_W * 4, &c->bytes));
    TRY(axbc_dalloc((void **)&c->task_ctr, 64, &c->bytes));
    TRY(axbc_dalloc((void **)&c->mpartial, (c->g->fwd.n_heavy_items + 1) * AXBC_W * 4, &c->bytes));
    TRY(axbc_dalloc((void **)&c->bi, sizeof(BatchInfo), &c->bytes));
    CU(cudaMallocHost((void **)&c->bi_host, sizeof(BatchInfo)));
    CU(cudaMemset(c->bi, 0, sizeof(BatchInfo)));
    TRY(axbc_batch_levels_alloc(c, 8));
    return AXBC_OK;
}

// Forward and backward passes of the batch whose roots/p are in c->bi.
int axbc_batch_traverse(axbc_ctx *c, int nsrc, int H)
{
    axbc_graph *g = c->g;
    const uint64_t n = g->n;
    cudaStream_t s = c->stream;
    const int grid = axbc_grid_for(c, BATCH_TPB, 8);
    // dynamic kernels: as many blocks as stay resident; work comes from a counter
    if (!c->dyn_blocks_per_sm) {
        int a = 0, b = 0, d = 0;
        CU(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&a, k_fwd_push_m, BATCH_TPB, 0));
        CU(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, k_fwd_pull_m, BATCH_TPB, 0));
        CU(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&d, k_bwd_m, BATCH_TPB, 0));
        c->dyn_blocks_per_sm = std::max(1, std::min(a, std::min(b, d)));
    }
    const int dgrid = axbc_grid_for(c, BATCH_TPB, c->dyn_blocks_per_sm);
    const size_t lvl_off = offsetof(BatchInfo, lvl_new);
    const size_t lvl_len = offsetof(BatchInfo, task_ctr) - lvl_off;
    const uint32_t srcmask = nsrc >= 32 ? FULL_MASK : ((1u << nsrc) - 1u);

    CU(cudaMemsetAsync(c->seen, 0, n * 4, s));
    CU(cudaMemsetAsync(c->fmask[0], 0, n * 4, s));
    CU(cudaMemsetAsync(c->msigma, 0, n * AXBC_W * 4, s));
    {
        ProfScope ps(c, KP_LEVEL_STATS, 0);
        k_batch_init<<<1, 32, 0, s>>>(c->bi, nsrc, H, c->fmask[0], c->seen, c->msigma, g->fwd.col,
                                      g->rev.col, g->m);
    }
    CU_LAUNCH("k_batch_init");
    CU(cudaMemcpyAsync((char *)c->bi_host + lvl_off, (char *)c->bi + lvl_off, lvl_len,
                       cudaMemcpyDeviceToHost, s));
    CU(cudaStreamSynchronize(s));
    uint64_t front = c->bi_host->front_deg, unvis = c->bi_host->unvis_deg;
    // per depth: degree sum over (vertex, pivot) pairs and pair count, for
    // the traversed-edge byte model of the profiling hooks
    std::vector<double> dte(1, (double)front), dcnt(1, (double)nsrc);
    const double W = nsrc;

    int Ls[AXBC_W];
    for (int i = 0; i < AXBC_W; i++) Ls[i] = 0;
    uint32_t alive = srcmask;
    int L = 0;
    for (;;) {
        L++;
        TRY(axbc_batch_levels_alloc(c, L + 2));
        uint32_t *fprev = c->fmask[L - 1], *fcur = c->fmask[L];
        CU(cudaMemsetAsync(fcur, 0, n * 4, s));
        CU(cudaMemsetAsync((char *)c->bi + lvl_off, 0, lvl_len, s));
        const bool push = (double)front * c->push_factor_batch < (double)unvis;
        {
            ProfScope ps(c, push ? KP_FWD_PUSH : KP_FWD_PULL, dte[L - 1] * (4.0 / W + 4.0));
            CU(cudaMemsetAsync(c->task_ctr, 0, 4, s));
            if (push)
                k_fwd_push_m<<<dgrid, BATCH_TPB, 0, s>>>(g->fwd, fprev, fcur, c->seen, c->msigma,
                                                        c->task_ctr);
            else
                k_fwd_pull_m<<<dgrid, BATCH_TPB, 0, s>>>(g->rev, srcmask, fprev, fcur, c->seen,
                                                        c->msigma, c->task_ctr);
        }
        {
            ProfScope ps(c, KP_LEVEL_STATS, (double)n * 16.0);
            k_level_stats<<<grid, BATCH_TPB, 0, s>>>(n, srcmask, fcur, c->seen, g->fwd.col,
                                                     g->rev.col, g->reach, c->bi);
        }
        CU_LAUNCH("forward level");
        CU(cudaMemcpyAsync((char *)c->bi_host + lvl_off, (char *)c->bi + lvl_off, lvl_len,
                           cudaMemcpyDeviceToHost, s));
        CU(cudaStreamSynchronize(s));
        for (int i = 0; i < nsrc; i++) {
            if (((alive >> i) & 1u) && c->bi_host->lvl_new[i] == 0) {
                Ls[i] = L;
                alive &= ~(1u << i);
            }
        }
        front = c->bi_host->front_deg;
        unvis = c->bi_host->unvis_deg;
        double cnt = 0;
        for (int i = 0; i < nsrc; i++) cnt += (double)c->bi_host->lvl_new[i];
        dte.push_back((double)c->bi_host->lvl_te);
        dcnt.push_back(cnt);
        if (!c->bi_host->any_new) break;
    }
    // every pivot's frontier is empty at level L; its deepest depth is Ls-1
    const int Dmax = L - 1;
    uint32_t depth0 = 0;
    for (int i = 0; i < nsrc; i++)
        if (Ls[i] == 2) depth0 |= 1u << i;
    CU(cudaMemcpyAsync(&c->bi->depth0mask, &depth0, 4, cudaMemcpyHostToDevice, s));

    for (int d = Dmax; d >= 0; d--) {
        const uint32_t dmask = d >= 1 ? srcmask : depth0;
        if (!dmask) continue;
        double te_d = dte[d], cnt_d = dcnt[d];
        if (d == 0) {
            const double frac = (double)__builtin_popcount(dmask) / W;
            te_d *= frac;
            cnt_d *= frac;
        }
        const double bytes = d == Dmax ? cnt_d * 4.0 : te_d * (4.0 / W + 8.0);
        {
            ProfScope ps(c, KP_BWD, bytes);
            CU(cudaMemsetAsync(c->task_ctr, 0, 4, s));
            k_bwd_m<<<dgrid, BATCH_TPB, 0, s>>>(g->fwd, dmask, d == Dmax, c->fmask[d],
                                                c->fmask[d + 1], c->msigma, c->mdelta, c->mq,
                                                c->mpartial, g->reach, c->task_ctr);
        }
        if (g->fwd.n_heavy) {
            ProfScope ps(c, KP_BWD_COMBINE, 0);
            k_bwd_combine_m<<<(g->fwd.n_heavy + 7) / 8, 256, 0, s>>>(
                g->fwd, dmask, c->fmask[d], c->msigma, c->mdelta, c->mq, c->mpartial, g->reach);
        }
        CU_LAUNCH("backward level");
    }
    c->last_batch_levels = L;
    c->last_batch_nsrc = nsrc;
    for (int i = 0; i < AXBC_W; i++) c->last_Ls[i] = i < nsrc ? Ls[i] : 0;
    return AXBC_OK;
}

int axbc_batch_apply(axbc_ctx *c)
{
    axbc_graph *g = c->g;
    cudaStream_t s = c->stream;
    const int grid = axbc_grid_for(c, BATCH_TPB, 8);
    {
        ProfScope ps(c, KP_UPDATE, (double)g->n * c->last_batch_nsrc * 20.0);
        k_update_m<<<grid, BATCH_TPB, 0, s>>>(c->bc, c->mdelta, c->seen, g->reach, g->n, c->bi);
    }
    {
        ProfScope ps(c, KP_UPDATE, 0);
        k_extract_delta<<<grid, 256, 0, s>>>(c->delta_last, c->mdelta, c->seen, g->reach, g->n, c->bi);
    }
    CU_LAUNCH("update");
    c->delta_last_valid = true;
    return AXBC_OK;
}

extern "C" int axbc_run_batch(axbc_ctx *c, const uint32_t *v0, const double *p, int k, int H,
                              axbc_pivot_stats *stats)
{
    CHECK_ARG(c && v0 && p, "axbc_run_batch: null argument");
    CHECK_ARG(k >= 1 && k <= AXBC_MAX_BATCH, "axbc_run_batch: k must be in [1, 32]");
    CHECK_ARG(H == 0 || H == 1, "axbc_run_batch: H must be 0 or 1");
    for (int i = 0; i < k; i++) {
        CHECK_ARG(v0[i] < c->g->n, "axbc_run_batch: pivot >= n");
        for (int j = 0; j < i; j++) CHECK_ARG(v0[i] != v0[j], "axbc_run_batch: repeated pivot");
    }
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
    uint32_t depth0 = 0;
    CU(cudaMemcpyAsync(&depth0, &c->bi->depth0mask, 4, cudaMemcpyDeviceToHost, s));
    CU(cudaStreamSynchronize(s));
    k_source_view<<<axbc_grid_for(c, 256, 4), 256, 0, s>>>(src, levels, d_fm, c->seen, c->msigma,
                                                           c->mdelta, c->g->reach, n, depth0, sig,
                                                           lvl, dl);
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
        switch (i & 3) {
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
        default:  // integers times integers
            x = (float)((h1 & 0xfffff) + 1);
            p = (double)((h2 & 0xfff) + 1) / (double)((h2 >> 12 & 0xfffff) + 1);
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
