// Pivot sampling on the device: the seven heuristics of -z, the drand48
// stream, the rejection of already-drawn pivots, the degree-0 skip, the
// bad-sample limit and Bader's stop test -- the loop of src/axbc2d.c:
// 2729-3156 on one rank -- plus the driver that alternates sampling with the
// batched Brandes pass.
//
// Float-weighted distributions (LCC, bc, delta, 1/(1+bc)) are sampled from a
// hierarchical double prefix (block-local running sums plus a running sum of
// block totals) instead of the reference's float running sum; the integer
// degree^2 distribution keeps the reference's uint32 wrap-around.
#include <algorithm>
#include <cstring>

#include "common.cuh"
#include "sampled.cuh"

struct SamplerState {
    uint64_t rng;
    uint64_t ui, nbfs, N;
    int32_t z;
    uint32_t dist_mix;
    uint32_t lim;
    uint32_t bader_c;
    uint32_t nchecks;
    int32_t W;
    int32_t done, stopped;
    uint64_t nrounds, skipped, dropped, te;
    uint64_t nrounds_snap;
    // this batch
    int32_t nb;
    uint32_t napply;
    uint64_t skipped_run;
    uint32_t v0[AXBC_MAX_WIDTH];
    double p[AXBC_MAX_WIDTH];
    uint64_t skip_before[AXBC_MAX_WIDTH];
};

struct SamplerDists {
    // static
    const uint32_t *col, *row, *deg2p, *seg_end, *sdn;
    uint32_t n_seg, sum_deg;
    const float *lcc;
    const double *lcc_local, *lcc_csum;
    // dynamic (this batch's snapshot)
    const float *bc, *delta_last;
    const double *bc_local, *bc_csum;  // prefix of bc (z 3, 6) or 1/(1+bc) (z 5)
    const double *d_local, *d_csum;    // prefix of the last delta (z 4, 6)
};

// ------------------------------------------------------------ drand48
__device__ __forceinline__ int64_t d_lrand48(uint64_t &x)
{
    x = (0x5DEECE66DULL * x + 0xBULL) & 0xFFFFFFFFFFFFULL;
    return (int64_t)(x >> 17);
}
// uniform_int(max, min) in uint32 arithmetic (src/axbc2d.c:2155-2164), of the
// lrand48 value r
__device__ __forceinline__ uint32_t d_int_of(int64_t r, uint32_t max, uint32_t min)
{
    const uint32_t mod = max - min + 1u;
    if (mod == 0) return (uint32_t)r + min;
    return (uint32_t)(r % (int64_t)mod) + min;
}
__device__ __forceinline__ uint32_t d_uniform_int(uint64_t &x, uint32_t max, uint32_t min)
{
    return d_int_of(d_lrand48(x), max, min);
}
// uniform01 (src/axbc2d.c:2172-2176): lrand48() / RAND_MAX
__device__ __forceinline__ double d_01_of(int64_t r) { return __ddiv_rn((double)r, 2147483647.0); }
__device__ __forceinline__ double d_uniform01(uint64_t &x) { return d_01_of(d_lrand48(x)); }

// ------------------------------------------------- hierarchical prefix
// The prefix of a float weight vector in double, two-level at both scales so
// that no chain of dependent double additions is long (double adds are slow
// on this part and a left-to-right sum of millions of terms cannot run in
// parallel):
//  - a block of AXBC_SAMPLE_BLOCK (1024) weights is 32 runs of 32; s = running
//    sum inside a run, P = running sum of the finished runs' totals,
//    local[i] = P + s; the block total is P after the last run;
//  - blocks form groups of 32: L = running sum of block totals inside the
//    group, G = running sum of the finished groups' totals, csum[b] = G + L.
// Every sum is left to right; the oracle computes the same values.
#define HP_WARPS 4
__device__ __forceinline__ float hp_weight(const float *__restrict__ w, uint64_t i, int mode)
{
    const float x = __ldg(w + i);
    // mode 1: the weight 1/(1+bc) of heuristic 5 (src/axbc2d.c:2025-2058)
    return mode == 1 ? __fdiv_rn(1.0f, __fadd_rn(1.0f, x)) : x;
}

// one warp per block: lane l owns run l; the run prefixes are staged in shared
// memory so the stores of local[] are coalesced
__global__ void __launch_bounds__(32 * HP_WARPS) k_hprefix_local(const float *__restrict__ w, uint64_t n,
                                                               double *__restrict__ local,
                                                               double *__restrict__ bsum, int mode,
                                                               const SamplerState *ss)
{
    if (ss && (ss->done || ss->nrounds_snap == 0)) return;
    __shared__ double sd[HP_WARPS][32 * 33];
    const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
    const uint64_t nb = (n + AXBC_SAMPLE_BLOCK - 1) / AXBC_SAMPLE_BLOCK;
    for (uint64_t b = (uint64_t)blockIdx.x * HP_WARPS + wib; b < nb; b += (uint64_t)gridDim.x * HP_WARPS) {
        const uint64_t base = b * AXBC_SAMPLE_BLOCK, i0 = base + 32 * (uint64_t)lane;
        const int cnt = i0 >= n ? 0 : (int)min((uint64_t)32, n - i0);
        double s = 0.0;
        for (int k = 0; k < cnt; k++) s = __dadd_rn(s, (double)hp_weight(w, i0 + k, mode));
        // P before run l; c ends as the block total (absent runs add +0)
        double c = 0.0, pex = 0.0;
#pragma unroll
        for (int k = 0; k < 32; k++) {
            const double t = __shfl_sync(FULL_MASK, s, k);
            if (lane == k) pex = c;
            c = __dadd_rn(c, t);
        }
        double r = 0.0;
        for (int k = 0; k < cnt; k++) {
            r = __dadd_rn(r, (double)hp_weight(w, i0 + k, mode));
            sd[wib][lane * 33 + k] = __dadd_rn(pex, r);
        }
        __syncwarp();
        for (int it = 0; it < 32; it++) {
            const uint64_t i = base + 32 * (uint64_t)it + lane;
            if (i < n) local[i] = sd[wib][it * 33 + lane];
        }
        __syncwarp();
        if (lane == 0) bsum[b] = c;
    }
}

// csum holds the block totals on entry and their prefix on exit.  One block of
// 1024 threads; groups are handled in chunks of 1024.
__global__ void __launch_bounds__(1024, 1) k_hprefix_csum(double *csum, uint64_t nb, const SamplerState *ss)
{
    if (ss && (ss->done || ss->nrounds_snap == 0)) return;
    __shared__ double s_G[1024];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    const uint64_t ng = (nb + 31) / 32;
    double G = 0.0;  // warp 0's running sum of group totals
    for (uint64_t g0 = 0; g0 < ng; g0 += 1024) {
        const uint64_t gend = min(ng, g0 + 1024);
        // in-group running sums, in place
        for (uint64_t g = g0 + wid; g < gend; g += 32) {
            const uint64_t b = g * 32 + lane;
            const double x = b < nb ? csum[b] : 0.0;
            double c = 0.0, mine = 0.0;
#pragma unroll
            for (int k = 0; k < 32; k++) {
                c = __dadd_rn(c, __shfl_sync(FULL_MASK, x, k));
                if (lane == k) mine = c;
            }
            if (b < nb) csum[b] = mine;
        }
        __syncthreads();
        // G before each group of the chunk (warp 0)
        if (wid == 0) {
            for (uint64_t gb = g0; gb < gend; gb += 32) {
                const uint64_t g = gb + lane;
                const double tot = g < gend ? csum[min(g * 32 + 31, nb - 1)] : 0.0;
#pragma unroll
                for (int k = 0; k < 32; k++) {
                    if (lane == k && g < gend) s_G[g - g0] = G;
                    G = __dadd_rn(G, __shfl_sync(FULL_MASK, tot, k));
                }
            }
        }
        __syncthreads();
        for (uint64_t b = g0 * 32 + threadIdx.x; b < min(nb, gend * 32); b += 1024)
            csum[b] = __dadd_rn(s_G[b / 32 - g0], csum[b]);
        __syncthreads();
    }
}

int axbc_hprefix_launch(const float *w, uint64_t n, double *local, double *csum, cudaStream_t s)
{
    const uint64_t nb = (n + AXBC_SAMPLE_BLOCK - 1) / AXBC_SAMPLE_BLOCK;
    k_hprefix_local<<<(unsigned)min((uint64_t)65535, (nb + HP_WARPS - 1) / HP_WARPS), 32 * HP_WARPS, 0, s>>>(
        w, n, local, csum, 0, nullptr);
    k_hprefix_csum<<<1, 1024, 0, s>>>(csum, nb, nullptr);
    CU_LAUNCH("hprefix");
    return AXBC_OK;
}

// first index whose prefix reaches r; *found = 0 if the total is NaN or < r
__device__ uint64_t d_hsearch(const double *local, const double *csum, uint64_t n, double r,
                              int *found)
{
    const uint64_t B = AXBC_SAMPLE_BLOCK, nb = (n + B - 1) / B;
    *found = 0;
    if (n == 0) return 0;
    const double tot = csum[nb - 1];
    if (isnan(tot) || !(tot >= r)) return n - 1;
    uint64_t lo = 0, hi = nb;
    while (lo < hi) {
        const uint64_t mid = (lo + hi) / 2;
        if (csum[mid] >= r) hi = mid;
        else lo = mid + 1;
    }
    const uint64_t b = lo;
    const double rr = __dsub_rn(r, b > 0 ? csum[b - 1] : 0.0);
    const uint64_t e = min((b + 1) * B, n);
    lo = b * B;
    hi = e;
    while (lo < hi) {
        const uint64_t mid = (lo + hi) / 2;
        if (local[mid] >= rr) hi = mid;
        else lo = mid + 1;
    }
    *found = 1;
    return lo < e ? lo : e - 1;
}

// The same search run by all SAMPLER_TPB threads of a block together (every
// thread calls it with the same arguments): each step tests SAMPLER_TPB evenly
// spaced positions at once and keeps the gap holding the first position >= r,
// so a search of n entries takes a few steps instead of log2(n) dependent loads.
#define SAMPLER_TPB 256
__device__ uint64_t blk_first_ge(const double *a, uint64_t lo, uint64_t hi, double r)
{
    while (lo < hi) {
        const uint64_t step = (hi - lo + SAMPLER_TPB - 1) / SAMPLER_TPB;
        const uint64_t p = lo + (uint64_t)threadIdx.x * step;
        const int below = __syncthreads_count(p < hi && !(a[p] >= r));
        if (below == 0) return lo;
        const uint64_t nhi = min(hi, lo + (uint64_t)below * step);
        lo = lo + (uint64_t)(below - 1) * step + 1;
        hi = nhi;
    }
    return hi;
}

__device__ uint64_t blk_hsearch(const double *local, const double *csum, uint64_t n, double r, int *found)
{
    const uint64_t B = AXBC_SAMPLE_BLOCK, nb = (n + B - 1) / B;
    *found = 0;
    if (n == 0) return 0;
    const double tot = csum[nb - 1];
    if (isnan(tot) || !(tot >= r)) return n - 1;
    const uint64_t b = blk_first_ge(csum, 0, nb, r);
    const double rr = __dsub_rn(r, b > 0 ? csum[b - 1] : 0.0);
    const uint64_t e = min((b + 1) * B, n);
    const uint64_t lo = blk_first_ge(local, b * B, e, rr);
    *found = 1;
    return lo < e ? lo : e - 1;
}

// first index of a wrapping uint32 prefix with prefix >= r, searched run by
// run (findsample_LOCINT, src/axbc2d.c:2188-2198)
__device__ uint64_t d_find_u32(const uint32_t *p, const uint32_t *seg_end, uint32_t n_seg, uint32_t r,
                               int *found)
{
    uint32_t start = 0;
    *found = 0;
    for (uint32_t k = 0; k < n_seg; k++) {
        const uint32_t end = seg_end[k];
        if (end > start && p[end - 1] >= r) {
            uint32_t lo = start, hi = end;
            while (lo < hi) {
                const uint32_t mid = (lo + hi) >> 1;
                if (p[mid] >= r) hi = mid;
                else lo = mid + 1;
            }
            *found = 1;
            return lo;
        }
        start = end;
    }
    return 0;
}

__device__ bool d_bader(const float *bc, const uint32_t *checks, uint32_t x, uint64_t N, uint32_t c)
{
    const double lim = (double)((uint64_t)c * N);
    for (uint32_t i = 0; i < x; i++) {
        const double b = checks[i] < N ? (double)bc[checks[i]] : 0.0;
        if (__ddiv_rn(b, 2.0) < lim) return false;
    }
    return true;
}

// init_rand + the check vertices + the heuristic's set-up draws
// (src/axbc2d.c:2736-2760, 2793-2795)
__global__ void k_sampler_init(SamplerState *ss, uint32_t *checks, int64_t seed, int z, uint64_t nbfs,
                               uint64_t N, uint32_t bader_c, uint32_t nchecks, int W)
{
    uint64_t x = (((uint64_t)seed & 0xffffffffULL) << 16) | 0x330EULL;
    for (uint32_t i = 0; i < nchecks; i++) checks[i] = d_uniform_int(x, (uint32_t)N, 0);
    uint32_t dist_mix = (uint32_t)z;
    if (z == 0) (void)d_uniform_int(x, (uint32_t)N, 0);
    else if (z == 6) dist_mix = d_uniform_int(x, 4, 0);
    ss->rng = x;
    ss->ui = 0;
    ss->nbfs = nbfs < N ? nbfs : N;
    ss->N = N;
    ss->z = z;
    ss->dist_mix = dist_mix;
    ss->lim = (uint32_t)(N * N);  // int LIMxSAMPLE = N*N, truncated (src/axbc2d.c:2835)
    ss->bader_c = bader_c;
    ss->nchecks = nchecks;
    ss->W = W;
    ss->done = ss->nbfs == 0;
    ss->stopped = 0;
    ss->nrounds = ss->skipped = ss->dropped = ss->te = ss->nrounds_snap = 0;
    ss->nb = 0;
    ss->napply = 0;
    ss->skipped_run = 0;
}

// The draws that take one lrand48 value: the pivot and its probability from
// the value r, for the effective heuristic k in {0, 2, 3, 4, 5}.
// COOP: called by every thread of a SAMPLER_TPB block with the same
// arguments, searching together (blk_hsearch); else one thread searches alone.
template <bool COOP>
__device__ __forceinline__ uint64_t hsearch_of(const double *local, const double *csum, uint64_t n, double r,
                                               int *found)
{
    return COOP ? blk_hsearch(local, csum, n, r, found) : d_hsearch(local, csum, n, r, found);
}

template <bool COOP>
__device__ void d_map_one(int64_t r, int k, uint64_t N, const SamplerDists &D, bool snap0,
                          double S_bc, double S_d, double S_lcc, uint32_t &v0, double &prob)
{
    int found;
    if (k == 0 || snap0 && (k == 3 || k == 4 || k == 5)) {
        v0 = d_int_of(r, (uint32_t)N, 0);
        prob = __ddiv_rn(1.0, (double)N);
    } else if (k == 2) {
        // LCC (src/axbc2d.c:2919-2937)
        const double rr = __dmul_rn(d_01_of(r), S_lcc);
        uint64_t h = hsearch_of<COOP>(D.lcc_local, D.lcc_csum, N, rr, &found);
        if (!found) h = N - 1;
        v0 = (uint32_t)h;
        prob = __ddiv_rn((double)D.lcc[v0], S_lcc);
    } else if (k == 4) {
        // delta of the last pivot (src/axbc2d.c:2970-2991)
        const double rr = __dmul_rn(d_01_of(r), S_d);
        uint64_t h = hsearch_of<COOP>(D.d_local, D.d_csum, N, rr, &found);
        if (!found) h = N - 1;
        v0 = (uint32_t)h;
        prob = __ddiv_rn((double)D.delta_last[v0], S_d);
    } else {
        // bc (src/axbc2d.c:2941-2969) or 1/(1+bc) (2995-3022)
        const double rr = __dmul_rn(d_01_of(r), S_bc);
        uint64_t h = hsearch_of<COOP>(D.bc_local, D.bc_csum, N, rr, &found);
        if (!found) h = N - 1;
        v0 = (uint32_t)h;
        if (k == 3) prob = __ddiv_rn((double)D.bc[v0], S_bc);
        else prob = __ddiv_rn(__ddiv_rn(1.0, __dadd_rn((double)D.bc[v0], 1.0)), S_bc);
    }
}

// One draw of heuristic z (dist_mix: the -z 6 mixture state, equal to z for
// the others): v0 and its probability, the reference's rules of
// src/axbc2d.c:2873-3051.  snap0: no pivot applied yet (the dynamic heuristics
// then draw uniformly).
template <bool COOP>
__device__ void d_draw_one(uint64_t &x, uint32_t &dist_mix, int z, uint64_t N, const SamplerDists &D,
                           bool snap0, double S_bc, double S_d, double S_lcc, uint32_t &v0,
                           double &prob)
{
    const int k = z == 6 ? (int)dist_mix : z;  // the distribution this draw uses
    prob = 0;
    if (k == 1) {
        // high-degree neighbourhood (src/axbc2d.c:2890-2917): one or two values
        int found;
        const uint32_t r = d_uniform_int(x, D.sum_deg, 0);
        uint64_t h = d_find_u32(D.deg2p, D.seg_end, D.n_seg, r, &found);
        if (!found) h = N - 1;
        const uint32_t dh = D.col[h + 1] - D.col[h];
        if (dh > 0) {
            uint32_t kk = 0;
            if (dh != 1) kk = d_uniform_int(x, dh - 1, 0);
            h = D.row[D.col[h] + kk];
        }
        v0 = (uint32_t)h;
        prob = __ddiv_rn((double)D.sdn[v0], (double)D.sum_deg);
    } else {
        d_map_one<COOP>(d_lrand48(x), k, N, D, snap0, S_bc, S_d, S_lcc, v0, prob);
    }
    if (z == 6) {
        // mixture probability (src/axbc2d.c:3026-3051)
        prob = __ddiv_rn(1.0, (double)N);
        if (snap0) {
            prob = __dadd_rn(prob, __ddiv_rn(1.0, (double)N));
            prob = __dadd_rn(prob, __ddiv_rn(1.0, (double)N));
        } else if (v0 < N) {
            prob = __dadd_rn(prob, __ddiv_rn((double)D.bc[v0], S_bc));
            prob = __dadd_rn(prob, __ddiv_rn((double)D.delta_last[v0], S_d));
        }
        if (v0 < N) {
            prob = __dadd_rn(prob, __ddiv_rn((double)D.sdn[v0], (double)D.sum_deg));
            prob = __dadd_rn(prob, __ddiv_rn((double)D.lcc[v0], S_lcc));
            prob = __ddiv_rn(prob, 5.0);
        }
        dist_mix = d_uniform_int(x, 2, 0);
    }
}

// Draw the rounds of one batch: up to W accepted pivots.  Every thread of the
// block runs the same sequential loop on the same values (stores by thread 0);
// for the heuristics that take one lrand48 value per draw, a streak of
// rejected draws (pivot already used) is searched SAMPLER_TPB draws at a time:
// thread t evaluates the draw t steps ahead (drand48 skip-ahead: x -> A_t x +
// C_t mod 2^48) and the first acceptable one wins, with the state and the
// rejection count advanced exactly as the sequential loop would.
// rejections in a row before the block searches draws in parallel
#ifndef AXBC_SAMPLER_STREAK
#define AXBC_SAMPLER_STREAK 4
#endif

// The used-pivot flags are set by thread 0 between two barriers: after every
// thread has tested the round's draws against them, before any thread tests
// the next round's.
__device__ __forceinline__ bool is_used(const uint8_t *used, uint32_t v) { return used[v] != 0; }
__device__ __forceinline__ void set_used(uint8_t *used, uint32_t v) { used[v] = 1; }
__global__ void __launch_bounds__(SAMPLER_TPB) k_sampler(SamplerState *ss, SamplerDists D, uint8_t *used,
                                                       const uint32_t *checks, double S_lcc)
{
    __shared__ uint64_t s_A[SAMPLER_TPB + 1], s_C[SAMPLER_TPB + 1];
    __shared__ int s_best;
    __shared__ uint32_t s_v0;
    __shared__ double s_prob;
    const int t = threadIdx.x;
    const bool lead = t == 0;
    const bool done = ss->done != 0;
    __syncthreads();
    if (lead) {
        ss->nb = 0;
        ss->napply = 0;
        ss->skipped_run = 0;
    }
    if (done) return;
    const uint64_t N = ss->N;
    if (ss->bader_c > 0 && d_bader(D.bc, checks, ss->nchecks, N, ss->bader_c)) {
        if (lead) {
            ss->stopped = 1;
            ss->done = 1;
        }
        return;
    }
    uint64_t x = ss->rng;
    uint32_t dist_mix = ss->dist_mix;
    const int z = ss->z;
    const uint32_t LIM = ss->lim;
    const bool snap0 = ss->nrounds_snap == 0;
    const int W = ss->W;
    const uint64_t nbfs = ss->nbfs;
    const uint64_t nbB = (N + AXBC_SAMPLE_BLOCK - 1) / AXBC_SAMPLE_BLOCK;
    double S_bc = 0, S_d = 0;
    if (!snap0) {
        if (D.bc_csum) S_bc = D.bc_csum[nbB - 1];
        if (D.d_csum) S_d = D.d_csum[nbB - 1];
    }
    const bool one_value = z == 0 || z == 2 || z == 3 || z == 4 || z == 5;
    if (one_value && lead) {
        const uint64_t M = 0xFFFFFFFFFFFFULL;
        uint64_t A = 1, C = 0;
        s_A[0] = 1;
        s_C[0] = 0;
        for (int k = 1; k <= SAMPLER_TPB; k++) {
            A = (A * 0x5DEECE66DULL) & M;
            C = (C * 0x5DEECE66DULL + 0xBULL) & M;
            s_A[k] = A;
            s_C[k] = C;
        }
    }
    __syncthreads();
    int nb = 0;
    uint64_t ui = ss->ui, skipped_run = 0, dropped = 0;
    while (nb < W && ui < nbfs) {
        uint32_t v0 = 0;
        double prob = 0;
        uint32_t BSM = 0;
        bool good = false;
        while (!good) {
            if (BSM > LIM) break;
            if (one_value && BSM >= AXBC_SAMPLER_STREAK) {
                // candidates allowed before the bad-sample limit
                const uint64_t allow = min((uint64_t)SAMPLER_TPB, (uint64_t)LIM - BSM + 1);
                uint32_t v = 0;
                double pr = 0;
                bool acc = false;
                if ((uint64_t)t < allow) {
                    const uint64_t xt = (s_A[t + 1] * x + s_C[t + 1]) & 0xFFFFFFFFFFFFULL;
                    d_map_one<false>((int64_t)(xt >> 17), z, N, D, snap0, S_bc, S_d, S_lcc, v, pr);
                    acc = !(v < N && is_used(used, v));
                }
                if (lead) s_best = SAMPLER_TPB;
                __syncthreads();
                if (acc) atomicMin(&s_best, t);
                __syncthreads();
                const int j = s_best;
                if (j < SAMPLER_TPB) {
                    if (t == j) {
                        s_v0 = v;
                        s_prob = pr;
                    }
                    __syncthreads();
                    v0 = s_v0;
                    prob = s_prob;
                    x = (s_A[j + 1] * x + s_C[j + 1]) & 0xFFFFFFFFFFFFULL;
                    BSM += (uint32_t)j;
                    good = true;
                } else {
                    x = (s_A[allow] * x + s_C[allow]) & 0xFFFFFFFFFFFFULL;
                    BSM += (uint32_t)allow;
                }
                __syncthreads();
                continue;
            }
            d_draw_one<true>(x, dist_mix, z, N, D, snap0, S_bc, S_d, S_lcc, v0, prob);
            if (v0 < N && is_used(used, v0)) BSM++;
            else good = true;
        }
        if (!good) {  // round dropped (src/axbc2d.c:3072-3077)
            dropped++;
            ui++;
            continue;
        }
        // every thread has tested this round's draws against the flags
        // before thread 0 sets the new one
        __syncthreads();
        if (v0 >= N || D.col[v0 + 1] == D.col[v0]) {  // degree-0 root (3095-3111)
            skipped_run++;
            if (v0 < N && lead) set_used(used, v0);
            __syncthreads();
            ui++;
            continue;
        }
        if (lead) {
            set_used(used, v0);
            ss->v0[nb] = v0;
            ss->p[nb] = prob;
            ss->skip_before[nb] = skipped_run;
        }
        __syncthreads();
        skipped_run = 0;
        nb++;
        ui++;
    }
    if (lead) {
        ss->rng = x;
        ss->dist_mix = dist_mix;
        ss->ui = ui;
        ss->nb = nb;
        ss->skipped_run = skipped_run;
        ss->dropped += dropped;
    }
}

// Pivots [off, off + count) of a drawn round become lanes lane0 + 0.. of one
// pass (count = min(nb - off, AXBC_WMAX - lane0)).
__global__ void k_load_pass(const SamplerState *ss, BatchInfo *bi, int off, int lane0, int cnt)
{
    const int s = threadIdx.x;
    const int count = min(min(ss->nb - off, AXBC_WMAX - lane0), cnt);
    if (s < count) {
        bi->root[lane0 + s] = ss->v0[off + s];
        bi->p[lane0 + s] = ss->p[off + s];
    }
}

// After a pass (the drawn pivots [off, off + cnt)): replay Bader's test
// between its pivots, fix how many are applied, and account rounds, skips and
// traversed edges.  The pass that ends the round also settles the degree-0
// draws after its last pivot.
__global__ void k_sampler_post(SamplerState *ss, BatchInfo *bi, const float *__restrict__ bc,
                               const float *__restrict__ mdelta, const uint32_t *__restrict__ seen,
                               const uint32_t *__restrict__ reach, const uint32_t *__restrict__ checks,
                               float *b, uint32_t *hist_v, double *hist_p, uint64_t hist_cap,
                               int off, int lane0, int cnt, int K, const uint32_t *__restrict__ to_view)
{
    if (ss->done && ss->nb == 0) return;
    const int nb = max(0, min(min(ss->nb - off, AXBC_WMAX - lane0), cnt));
    const bool last = off + nb >= ss->nb;
    const uint64_t N = ss->N;
    const uint32_t c = ss->bader_c;
    const double lim = (double)((uint64_t)c * N);
    int stop = nb;
    // check-vertex values through the batch, in the order the update applies
    const uint32_t x = ss->nchecks;
    const bool track = c > 0;
    if (track)
        for (uint32_t i = 0; i < x; i++) b[i] = checks[i] < N ? bc[checks[i]] : 0.0f;
    for (int s = 0; s < nb; s++) {
        if (c > 0 && off + s > 0) {
            bool sat = true;
            for (uint32_t i = 0; i < x && sat; i++) {
                const float bv = track ? b[i] : 0.0f;
                if (__ddiv_rn((double)bv, 2.0) < lim) sat = false;
            }
            if (sat) {
                stop = s;
                break;
            }
        }
        if (!track) continue;
        const int l = lane0 + s;
        const uint32_t r = bi->root[l];
        const uint32_t rr = reach[r];
        const uint32_t all = (bi->H == 1 ? (uint32_t)bi->rsum[l] : 0u) + rr;
        const unsigned long long nvt = bi->nvis[l] + all;
        const double p = bi->p[l];
        for (uint32_t i = 0; i < x; i++) {
            if (checks[i] >= N) continue;
            // the pass runs in the graph's view (roots, masks, rows, reach)
            const uint32_t v = to_view ? to_view[checks[i]] : checks[i];
            if (v == r) {
                if (rr > 0) b[i] = __fadd_rn(b[i], bc_root_term(rr, nvt));
                continue;
            }
            // the pass's layout: K mask words and 32 K row values per vertex
            const bool reached = (seen[(uint64_t)v * K + l / 32] >> (l % 32)) & 1u;
            const float dv = reached ? mdelta[(uint64_t)v * (AXBC_W * K) + l] : __uint2float_rn(reach[v]);
            if (dv == 0.0f && p > 0.0) continue;
            b[i] = __fadd_rn(b[i], bc_term(dv, rr, p));
        }
    }
    // lanes [lane0, lane0 + nb) of the pass: the first `stop` are applied
    const unsigned long long seg = (nb >= 64 ? ~0ull : ((1ull << nb) - 1ull)) << lane0;
    const unsigned long long app = (stop >= 64 ? ~0ull : ((1ull << stop) - 1ull)) << lane0;
    bi->applymask = (bi->applymask & ~seg) | app;
    ss->napply = stop;
    for (int s = 0; s < stop; s++) {
        if (ss->nrounds < hist_cap) {
            hist_v[ss->nrounds] = ss->v0[off + s];
            hist_p[ss->nrounds] = ss->p[off + s];
        }
        ss->nrounds++;
        ss->skipped += ss->skip_before[off + s];
        ss->te += 2 * bi->te[lane0 + s];
    }
    if (stop < nb) {
        ss->stopped = 1;
        ss->done = 1;
    } else if (last) {
        if (ss->skipped_run) {
            bool sat = false;
            if (c > 0 && nb > 0) {
                sat = true;
                for (uint32_t i = 0; i < x && sat; i++) {
                    const float bv = track ? b[i] : 0.0f;
                    if (__ddiv_rn((double)bv, 2.0) < lim) sat = false;
                }
            }
            if (sat) {
                ss->stopped = 1;
                ss->done = 1;
            } else {
                ss->skipped += ss->skipped_run;
            }
        }
        if (ss->ui >= ss->nbfs) ss->done = 1;
    }
    ss->nrounds_snap = ss->nrounds;
}

// ------------------------------------------------------------ sampled runs
// Device state of one sampled run lives in a SampledRun (sampled.cuh): the
// context's own buffers for axbc_run_sampled, or buffers of its own for a
// request of the server.

uint64_t sr_bytes(uint64_t n, const axbc_run_params *prm)
{
    const uint64_t nb = (n + AXBC_SAMPLE_BLOCK - 1) / AXBC_SAMPLE_BLOCK;
    const uint64_t nbfs = prm->nbfs < n ? prm->nbfs : n;
    uint64_t b = sizeof(SamplerState) + n * 4 * 2 + n + (prm->nchecks + 1) * 8 + (nbfs + 1) * 12;
    const int z = prm->z;
    if (z == 3 || z == 5 || z == 6) b += n * 8 + nb * 8;
    if (z == 4 || z == 6) b += n * 8 + nb * 8;
    return b;
}

static void sr_release(SampledRun *r, bool own)
{
    if (own) {
        axbc_dfree(r->ss);
        if (r->ss_host) cudaFreeHost(r->ss_host);
        axbc_dfree(r->bc);
        axbc_dfree(r->delta_last);
        axbc_dfree(r->used);
        axbc_dfree(r->checks);
        axbc_dfree(r->checkval);
        axbc_dfree(r->dyn_local);
        axbc_dfree(r->dyn_csum);
        axbc_dfree(r->dyn_local2);
        axbc_dfree(r->dyn_csum2);
    }
    axbc_dfree(r->hist_v);
    axbc_dfree(r->hist_p);
    r->hist_v = nullptr;
    r->hist_p = nullptr;
}

void sr_free(SampledRun *r) { sr_release(r, true); }

static int sr_alloc_hist(SampledRun *r, uint64_t n)
{
    const uint64_t nbfs = r->prm.nbfs < n ? r->prm.nbfs : n;
    r->hist_cap = nbfs + 1;
    TRY(axbc_dalloc((void **)&r->hist_v, r->hist_cap * 4, nullptr));
    TRY(axbc_dalloc((void **)&r->hist_p, r->hist_cap * 8, nullptr));
    return AXBC_OK;
}

int sr_alloc(axbc_graph *g, const axbc_run_params *prm, SampledRun *r)
{
    const uint64_t n = g->n;
    memset(r, 0, sizeof(*r));
    r->prm = *prm;
    const uint64_t nb = (n + AXBC_SAMPLE_BLOCK - 1) / AXBC_SAMPLE_BLOCK;
    int st = AXBC_OK;
#define SR_TRY(x)                   \
    do {                            \
        if ((st = (x)) != AXBC_OK) { \
            sr_release(r, true);    \
            return st;              \
        }                           \
    } while (0)
    SR_TRY(axbc_dalloc((void **)&r->ss, sizeof(SamplerState), nullptr));
    if (cudaMallocHost((void **)&r->ss_host, sizeof(SamplerState)) != cudaSuccess) {
        sr_release(r, true);
        axbc_set_error("sampled run: pinned host allocation failed");
        return AXBC_ERR_NOMEM;
    }
    SR_TRY(axbc_dalloc((void **)&r->bc, n * 4, nullptr));
    SR_TRY(axbc_dalloc((void **)&r->delta_last, n * 4, nullptr));
    SR_TRY(axbc_dalloc((void **)&r->used, n, nullptr));
    SR_TRY(axbc_dalloc((void **)&r->checks, (prm->nchecks + 1) * 4, nullptr));
    SR_TRY(axbc_dalloc((void **)&r->checkval, (prm->nchecks + 1) * 4, nullptr));
    const int z = prm->z;
    if (z == 3 || z == 5 || z == 6) {
        SR_TRY(axbc_dalloc((void **)&r->dyn_local, n * 8, nullptr));
        SR_TRY(axbc_dalloc((void **)&r->dyn_csum, nb * 8, nullptr));
    }
    if (z == 4 || z == 6) {
        SR_TRY(axbc_dalloc((void **)&r->dyn_local2, n * 8, nullptr));
        SR_TRY(axbc_dalloc((void **)&r->dyn_csum2, nb * 8, nullptr));
    }
    SR_TRY(sr_alloc_hist(r, n));
#undef SR_TRY
    return AXBC_OK;
}

int sr_check_params(const axbc_graph *g, const axbc_run_params *prm, int max_width)
{
    CHECK_ARG(prm->z >= 0 && prm->z <= 6, "sampled run: heuristic must be in [0,6]");
    CHECK_ARG(prm->H == 0 || prm->H == 1, "sampled run: H must be 0 or 1");
    CHECK_ARG(prm->batch_width >= 1 && prm->batch_width <= max_width,
              max_width == AXBC_W ? "sampled run: batch_width must be in [1, 32]"
                                  : "sampled run: batch_width must be in [1, 64]");
    CHECK_ARG(prm->nchecks <= g->n, "sampled run: more check vertices than vertices");
    return AXBC_OK;
}

// reset the run's vectors and draw its check vertices (on the context's stream)
int sr_begin(axbc_ctx *c, SampledRun *r)
{
    axbc_graph *g = c->g;
    const uint64_t n = g->n;
    cudaStream_t s = c->stream;
    const int z = r->prm.z;
    if (z == 1 || z == 6) TRY(axbc_build_deg_dist(g, s));
    if (z == 2 || z == 6) TRY(axbc_build_lcc(g, s));
    CU(cudaMemsetAsync(r->bc, 0, n * 4, s));
    CU(cudaMemsetAsync(r->delta_last, 0, n * 4, s));
    CU(cudaMemsetAsync(r->used, 0, n, s));
    {
        ProfScope ps(c, KP_SAMPLER, 0);
        k_sampler_init<<<1, 1, 0, s>>>(r->ss, r->checks, r->prm.seed, z, r->prm.nbfs, n,
                                       (uint32_t)r->prm.bader_c, r->prm.nchecks, r->prm.batch_width);
    }
    CU_LAUNCH("k_sampler_init");
    r->batches = 0;
    return AXBC_OK;
}

// draw the run's next round from its current bc / last delta; the sampler
// state is copied to the pinned mirror (read it after the stream syncs)
int sr_draw(axbc_ctx *c, SampledRun *r)
{
    axbc_graph *g = c->g;
    const uint64_t n = g->n;
    cudaStream_t s = c->stream;
    const int z = r->prm.z;
    SamplerDists D;
    memset(&D, 0, sizeof(D));
    D.col = g->fwd.col;
    D.row = g->fwd.row;
    D.deg2p = g->deg2p;
    D.seg_end = g->seg_end;
    D.sdn = g->sdn;
    D.n_seg = g->n_seg;
    D.sum_deg = g->sum_deg;
    D.lcc = g->lcc;
    D.lcc_local = g->lcc_local;
    D.lcc_csum = g->lcc_csum;
    D.bc = r->bc;
    D.delta_last = r->delta_last;
    const bool dyn_bc = z == 3 || z == 5 || z == 6;
    const bool dyn_d = z == 4 || z == 6;
    const uint64_t nbB = (n + AXBC_SAMPLE_BLOCK - 1) / AXBC_SAMPLE_BLOCK;
    const unsigned hb = (unsigned)min((uint64_t)65535, (nbB + HP_WARPS - 1) / HP_WARPS);
    if (dyn_bc) {
        D.bc_local = r->dyn_local;
        D.bc_csum = r->dyn_csum;
        {
            ProfScope ps(c, KP_SAMPLER, (double)n * 12.0);
            k_hprefix_local<<<hb, 32 * HP_WARPS, 0, s>>>(r->bc, n, r->dyn_local, r->dyn_csum, z == 5 ? 1 : 0, r->ss);
        }
        {
            ProfScope ps(c, KP_SAMPLER, 0);
            k_hprefix_csum<<<1, 1024, 0, s>>>(r->dyn_csum, nbB, r->ss);
        }
    }
    if (dyn_d) {
        D.d_local = r->dyn_local2;
        D.d_csum = r->dyn_csum2;
        {
            ProfScope ps(c, KP_SAMPLER, (double)n * 12.0);
            k_hprefix_local<<<hb, 32 * HP_WARPS, 0, s>>>(r->delta_last, n, r->dyn_local2, r->dyn_csum2, 0, r->ss);
        }
        {
            ProfScope ps(c, KP_SAMPLER, 0);
            k_hprefix_csum<<<1, 1024, 0, s>>>(r->dyn_csum2, nbB, r->ss);
        }
    }
    {
        ProfScope ps(c, KP_SAMPLER, 0);
        k_sampler<<<1, SAMPLER_TPB, 0, s>>>(r->ss, D, r->used, r->checks, g->S_lcc);
    }
    CU_LAUNCH("k_sampler");
    CU(cudaMemcpyAsync(r->ss_host, r->ss, sizeof(SamplerState), cudaMemcpyDeviceToHost, s));
    return AXBC_OK;
}

int sr_nb(const SampledRun *r) { return r->ss_host->nb; }
bool sr_done(const SampledRun *r) { return r->ss_host->done != 0; }
bool sr_finished(const SampledRun *r)
{
    return r->ss_host->done && r->ss_host->nb == 0 && r->ss_host->skipped_run == 0;
}

// Bader's test between two passes of one round, before the next pivot is
// traversed: the replay's test at that pivot (stop there, nothing applied).
__global__ void k_sampler_stop_test(SamplerState *ss, const float *__restrict__ bc,
                                    const uint32_t *__restrict__ checks)
{
    if (ss->done || ss->bader_c == 0) return;
    if (d_bader(bc, checks, ss->nchecks, ss->N, ss->bader_c)) {
        ss->stopped = 1;
        ss->done = 1;
    }
}

int sr_stop_test(axbc_ctx *c, SampledRun *r)
{
    {
        ProfScope ps(c, KP_SAMPLER, 0);
        k_sampler_stop_test<<<1, 1, 0, c->stream>>>(r->ss, r->bc, r->checks);
    }
    CU_LAUNCH("k_sampler_stop_test");
    CU(cudaMemcpyAsync(&r->ss_host->done, &r->ss->done, sizeof(int32_t), cudaMemcpyDeviceToHost, c->stream));
    return AXBC_OK;
}

int sr_load(axbc_ctx *c, SampledRun *r, int off, int lane0, int cnt)
{
    k_load_pass<<<1, AXBC_WMAX, 0, c->stream>>>(r->ss, c->bi, off, lane0, cnt);
    CU_LAUNCH("k_load_pass");
    return AXBC_OK;
}

int sr_post(axbc_ctx *c, SampledRun *r, int off, int lane0, int cnt)
{
    {
        ProfScope ps(c, KP_SAMPLER, 0);
        k_sampler_post<<<1, 1, 0, c->stream>>>(r->ss, c->bi, r->bc, c->mdelta, c->seen, c->g->breach,
                                               r->checks, r->checkval, r->hist_v, r->hist_p,
                                               r->hist_cap, off, lane0, cnt, c->last_batch_k,
                                               c->g->to_view);
    }
    CU_LAUNCH("k_sampler_post");
    return AXBC_OK;
}

// final counters, pivot history and check vertices of a finished run
int sr_result(axbc_ctx *c, SampledRun *r, axbc_run_result *res, std::vector<uint32_t> *piv,
              std::vector<double> *probs, std::vector<uint32_t> *checks)
{
    CU(cudaMemcpyAsync(r->ss_host, r->ss, sizeof(SamplerState), cudaMemcpyDeviceToHost, c->stream));
    CU(cudaStreamSynchronize(c->stream));
    const SamplerState &S = *r->ss_host;
    res->nrounds = S.nrounds;
    res->skipped = S.skipped;
    res->dropped = S.dropped;
    res->rounds = S.ui;
    res->te = S.te;
    res->stopped = S.stopped;
    res->batches = r->batches;
    const uint64_t k = std::min<uint64_t>(S.nrounds, r->hist_cap);
    if (piv) {
        piv->resize(k);
        if (k) CU(cudaMemcpy(piv->data(), r->hist_v, k * 4, cudaMemcpyDeviceToHost));
    }
    if (probs) {
        probs->resize(k);
        if (k) CU(cudaMemcpy(probs->data(), r->hist_p, k * 8, cudaMemcpyDeviceToHost));
    }
    if (checks) {
        checks->resize(r->prm.nchecks);
        if (r->prm.nchecks)
            CU(cudaMemcpy(checks->data(), r->checks, r->prm.nchecks * 4, cudaMemcpyDeviceToHost));
    }
    return AXBC_OK;
}

// the context's own sampler buffers, grown on demand
static int ensure_sampler(axbc_ctx *c, uint32_t nchecks)
{
    const uint64_t n = c->g->n;
    TRY(axbc_ensure_batch(c));
    if (!c->sampler_ready) {
        ALLOC_MISSING(c->ss, sizeof(SamplerState), &c->bytes);
        if (!c->ss_host) CU(cudaMallocHost((void **)&c->ss_host, sizeof(SamplerState)));
        ALLOC_MISSING(c->used, n, &c->bytes);
        const uint64_t nb = (n + AXBC_SAMPLE_BLOCK - 1) / AXBC_SAMPLE_BLOCK;
        ALLOC_MISSING(c->dyn_local, n * 8, &c->bytes);
        ALLOC_MISSING(c->dyn_csum, nb * 8, &c->bytes);
        ALLOC_MISSING(c->dyn_local2, n * 8, &c->bytes);
        ALLOC_MISSING(c->dyn_csum2, nb * 8, &c->bytes);
        c->sampler_ready = true;
    }
    if (!c->checks || !c->checkval || nchecks > c->nchecks_cap) {
        // both new buffers first: a failure keeps the old pair
        DBuf nc, nv;
        TRY(nc.alloc((nchecks + 1) * 4));
        TRY(nv.alloc((nchecks + 1) * 4));
        axbc_dfree(c->checks);
        axbc_dfree(c->checkval);
        c->checks = nc.as<uint32_t>();
        c->checkval = nv.as<float>();
        nc.p = nv.p = nullptr;
        c->bytes += 2 * (uint64_t)(nchecks + 1) * 4;
        c->nchecks_cap = nchecks;
    }
    return AXBC_OK;
}

// One drawn round of one run: its pivots in one pass (widths up to 64); the
// Bader replay between the pass's pivots decides how many are applied.  The
// first round of a run with Bader's stop goes in passes of 1, 1, 2, 4, ...
// pivots instead: with no bc yet the stop may come after any of its pivots,
// and the pivots of a pass past the stop are traversed for nothing.  Passes
// split a round without changing it: its pivots were all drawn before it, and
// each vertex's bc gets their terms in the same order.
static int sr_round_alone(axbc_ctx *c, SampledRun *r)
{
    const int nb = sr_nb(r);
    const bool ramp = r->prm.bader_c > 0 && r->batches == 0;
    int want = ramp ? 1 : AXBC_WMAX;
    for (int off = 0; off == 0 || off < nb;) {
        const int cnt = std::min(nb - off, want);
        if (cnt > 0) {
            TRY(sr_load(c, r, off, 0, cnt));
            TRY(axbc_batch_traverse(c, cnt, r->prm.H));
            r->batches++;
            float *tg[AXBC_WMAX];
            for (int i = 0; i < AXBC_WMAX; i++) tg[i] = r->bc;
            TRY(axbc_batch_set_targets(c, tg));
        }
        TRY(sr_post(c, r, off, 0, std::max(cnt, 0)));
        if (cnt > 0) {
            float *dout[1] = {r->delta_last};
            const int lo[1] = {0}, hi[1] = {AXBC_WMAX};
            TRY(axbc_batch_apply_lanes(c, dout, lo, hi, 1));
        }
        if (off + cnt < nb) {
            // a later pass runs only if Bader's test did not stop the round,
            // at or before its first pivot
            TRY(sr_stop_test(c, r));
            CU(cudaStreamSynchronize(c->stream));
            if (r->ss_host->done) break;
        }
        off += std::max(cnt, 1);
        if (ramp && off > 1) want = std::min(2 * want, AXBC_WMAX);
    }
    return AXBC_OK;
}

extern "C" int axbc_run_sampled(axbc_ctx *c, const axbc_run_params *prm, axbc_run_result *res)
{
    CHECK_ARG(c && prm && res, "axbc_run_sampled: null argument");
    TRY(sr_check_params(c->g, prm, AXBC_MAX_WIDTH));
    TRY(ensure_sampler(c, prm->nchecks));
    // a view of the context's buffers
    SampledRun r;
    memset(&r, 0, sizeof(r));
    r.prm = *prm;
    r.ss = c->ss;
    r.ss_host = c->ss_host;
    r.bc = c->bc;
    r.delta_last = c->delta_last;
    r.used = c->used;
    r.checks = c->checks;
    r.checkval = c->checkval;
    r.dyn_local = c->dyn_local;
    r.dyn_csum = c->dyn_csum;
    r.dyn_local2 = c->dyn_local2;
    r.dyn_csum2 = c->dyn_csum2;
    int st = sr_alloc_hist(&r, c->g->n);
    if (st == AXBC_OK) st = sr_begin(c, &r);
    while (st == AXBC_OK) {
        if ((st = sr_draw(c, &r)) != AXBC_OK) break;
        if (cudaStreamSynchronize(c->stream) != cudaSuccess) {
            st = axbc_cuda_fail(cudaGetLastError(), "sampler", __FILE__, __LINE__);
            break;
        }
        if (sr_finished(&r)) break;
        st = sr_round_alone(c, &r);
    }
    if (st == AXBC_OK) st = sr_result(c, &r, res, &c->run_pivots, &c->run_probs, &c->run_checks);
    sr_release(&r, false);
    return st;
}

// ------------------------------------------------- single draws, stop test
__global__ void k_sample_one(SamplerDists D, int z, uint64_t N, int first, double S_lcc,
                             uint64_t *state, uint32_t *out_v, double *out_p)
{
    uint64_t x = state[0];
    uint32_t mix = (uint32_t)state[1];
    const uint64_t nbB = (N + AXBC_SAMPLE_BLOCK - 1) / AXBC_SAMPLE_BLOCK;
    double S_bc = 0, S_d = 0;
    if (!first) {
        if (D.bc_csum) S_bc = D.bc_csum[nbB - 1];
        if (D.d_csum) S_d = D.d_csum[nbB - 1];
    }
    uint32_t v0 = 0;
    double prob = 0;
    d_draw_one<false>(x, mix, z, N, D, first != 0, S_bc, S_d, S_lcc, v0, prob);
    state[0] = x;
    state[1] = mix;
    *out_v = v0;
    *out_p = prob;
}

extern "C" uint64_t axbc_srand48(int64_t seed)
{
    return (((uint64_t)seed & 0xffffffffULL) << 16) | 0x330EULL;
}

extern "C" int axbc_sample(axbc_ctx *c, int z, uint64_t *rng, uint32_t *mix, int first, uint32_t *v0,
                           double *p)
{
    CHECK_ARG(c && rng && mix && v0 && p, "axbc_sample: null argument");
    CHECK_ARG(z >= 0 && z <= 6, "axbc_sample: heuristic must be in [0,6]");
    CHECK_ARG(z != 6 || *mix <= 4, "axbc_sample: mixture state must be in [0,4]");
    TRY(ensure_sampler(c, 0));
    axbc_graph *g = c->g;
    const uint64_t n = g->n;
    cudaStream_t s = c->stream;
    if (z == 1 || z == 6) TRY(axbc_build_deg_dist(g, s));
    if (z == 2 || z == 6) TRY(axbc_build_lcc(g, s));
    SamplerDists D;
    memset(&D, 0, sizeof(D));
    D.col = g->fwd.col;
    D.row = g->fwd.row;
    D.deg2p = g->deg2p;
    D.seg_end = g->seg_end;
    D.sdn = g->sdn;
    D.n_seg = g->n_seg;
    D.sum_deg = g->sum_deg;
    D.lcc = g->lcc;
    D.lcc_local = g->lcc_local;
    D.lcc_csum = g->lcc_csum;
    D.bc = c->bc;
    D.delta_last = c->delta_last;
    const uint64_t nbB = (n + AXBC_SAMPLE_BLOCK - 1) / AXBC_SAMPLE_BLOCK;
    const unsigned hb = (unsigned)min((uint64_t)65535, (nbB + HP_WARPS - 1) / HP_WARPS);
    if (!first && (z == 3 || z == 5 || z == 6)) {
        D.bc_local = c->dyn_local;
        D.bc_csum = c->dyn_csum;
        k_hprefix_local<<<hb, 32 * HP_WARPS, 0, s>>>(c->bc, n, c->dyn_local, c->dyn_csum, z == 5 ? 1 : 0, nullptr);
        k_hprefix_csum<<<1, 1024, 0, s>>>(c->dyn_csum, nbB, nullptr);
    }
    if (!first && (z == 4 || z == 6)) {
        D.d_local = c->dyn_local2;
        D.d_csum = c->dyn_csum2;
        k_hprefix_local<<<hb, 32 * HP_WARPS, 0, s>>>(c->delta_last, n, c->dyn_local2, c->dyn_csum2, 0, nullptr);
        k_hprefix_csum<<<1, 1024, 0, s>>>(c->dyn_csum2, nbB, nullptr);
    }
    // state, v0, p through the check-value scratch of the context
    uint64_t *dstate = nullptr;
    TRY(axbc_dalloc((void **)&dstate, 32, nullptr));
    // the reference keeps dist_mix = z outside the -z 6 mixture
    uint64_t h[4] = {*rng, z == 6 ? *mix : (uint32_t)z, 0, 0};
    cudaError_t e = cudaMemcpyAsync(dstate, h, 16, cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess) {
        k_sample_one<<<1, 1, 0, s>>>(D, z, n, first, g->S_lcc, dstate, (uint32_t *)(dstate + 2),
                                     (double *)(dstate + 3));
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaMemcpyAsync(h, dstate, 32, cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    axbc_dfree(dstate);
    if (e != cudaSuccess) return axbc_cuda_fail(e, "axbc_sample", __FILE__, __LINE__);
    *rng = h[0];
    if (z == 6) *mix = (uint32_t)h[1];
    *v0 = (uint32_t)h[2];
    memcpy(p, &h[3], 8);
    return AXBC_OK;
}

__global__ void k_bader_check(const float *bc, const uint32_t *checks, uint32_t x, uint64_t N, uint32_t c,
                              int *out)
{
    *out = d_bader(bc, checks, x, N, c) ? 1 : 0;
}

extern "C" int axbc_bader_check(axbc_ctx *c, const uint32_t *checks, uint32_t x, uint32_t bader_c,
                                int *satisfied)
{
    CHECK_ARG(c && satisfied && (checks || x == 0), "axbc_bader_check: null argument");
    TRY(ensure_sampler(c, x));
    cudaStream_t s = c->stream;
    if (x) CU(cudaMemcpyAsync(c->checks, checks, x * 4, cudaMemcpyHostToDevice, s));
    int *d = nullptr;
    TRY(axbc_dalloc((void **)&d, 4, nullptr));
    k_bader_check<<<1, 1, 0, s>>>(c->bc, c->checks, x, c->g->n, bader_c, d);
    int h = 0;
    cudaError_t e = cudaGetLastError();
    if (e == cudaSuccess) e = cudaMemcpyAsync(&h, d, 4, cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    axbc_dfree(d);
    if (e != cudaSuccess) return axbc_cuda_fail(e, "axbc_bader_check", __FILE__, __LINE__);
    *satisfied = h;
    return AXBC_OK;
}

extern "C" int axbc_get_pivots(const axbc_ctx *c, uint32_t *v0, double *p, uint64_t cap,
                               uint64_t *count)
{
    CHECK_ARG(c, "axbc_get_pivots: null context");
    const uint64_t k = std::min<uint64_t>(cap, c->run_pivots.size());
    for (uint64_t i = 0; i < k; i++) {
        if (v0) v0[i] = c->run_pivots[i];
        if (p) p[i] = c->run_probs[i];
    }
    if (count) *count = c->run_pivots.size();
    return AXBC_OK;
}

extern "C" int axbc_get_checks(const axbc_ctx *c, uint32_t *checks, uint32_t cap)
{
    CHECK_ARG(c && checks, "axbc_get_checks: null argument");
    for (uint32_t i = 0; i < cap && i < c->run_checks.size(); i++) checks[i] = c->run_checks[i];
    return AXBC_OK;
}
