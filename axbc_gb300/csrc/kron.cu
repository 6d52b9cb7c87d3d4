/* Parts of this file follow the Graph500 generator, which carries this notice:
 *
 * Copyright (C) 2009-2010 The Trustees of Indiana University.
 * Use, modification and distribution is subject to the Boost Software
 * License, Version 1.0.  Authors: Jeremiah Willcock, Andrew Lumsdaine.
 *
 * Boost Software License - Version 1.0 - August 17th, 2003
 *
 * Permission is hereby granted, free of charge, to any person or organization
 * obtaining a copy of the software and accompanying documentation covered by
 * this license (the "Software") to use, reproduce, display, distribute,
 * execute, and transmit the Software, and to prepare derivative works of the
 * Software, and to permit third-parties to whom the Software is furnished to
 * do so, all subject to the following:
 *
 * The copyright notices in the Software and this entire statement, including
 * the above license grant, this restriction and the following disclaimer,
 * must be included in all copies of the Software, in whole or in part, and
 * all derivative works of the Software, unless such copies or derivative
 * works are solely in the form of machine-executable object code generated by
 * a source language processor.
 *
 * THE SOFTWARE IS PROVIDED "AS IS", WITHOUT WARRANTY OF ANY KIND, EXPRESS OR
 * IMPLIED, INCLUDING BUT NOT LIMITED TO THE WARRANTIES OF MERCHANTABILITY,
 * FITNESS FOR A PARTICULAR PURPOSE, TITLE AND NON-INFRINGEMENT. IN NO EVENT
 * SHALL THE COPYRIGHT HOLDERS OR ANYONE DISTRIBUTING THE SOFTWARE BE LIABLE
 * FOR ANY DAMAGES OR OTHER LIABILITY, WHETHER IN CONTRACT, TORT OR OTHERWISE,
 * ARISING FROM, OUT OF OR IN CONNECTION WITH THE SOFTWARE OR THE USE OR OTHER
 * DEALINGS IN THE SOFTWARE.
 */

// The Graph500 Kronecker generator on the device, edge for edge.
//
// The reference builds its synthetic graphs with the Graph500 generator it
// vendors (generator/, called by gen_graph, src/axbc2d.c:518-527: initiator
// .57/.19/.19/.05, seeds 23 and 24, 2^scale * edgefactor edges).  This file
// produces the same edge list on the GPU:
//
//  - random numbers: the order-5 multiple recursive generator modulo 2^31-1,
//    x_n = 107374182 x_{n-1} + 104480 x_{n-5} (generator/splittable_mrg.c:
//    18-50, 154-165, 282-292).  A skip by e = hi 2^128 + mid 2^64 + lo steps
//    multiplies the state by A^e (splittable_mrg.c:169-184); here the 192
//    matrices A^(2^k) are made on the host by repeated squaring and one is
//    applied per set bit of e.
//  - the edge split (generator/graph_generator.c:147-278) runs level by level
//    instead of recursively: a node is one block of the adjacency matrix at
//    one level {first edge index, edge count, source base, target base}, and
//    its random state is a skip from the root state by its position alone, so
//    the nodes of a level are independent threads.  Nodes with one edge walk
//    down to a single cell (make_one_edge, graph_generator.c:98-145); nodes of
//    the last level write their cell count times; the others draw the counts
//    of their four quadrants (make_square_counts, graph_generator.c:50-83)
//    with binomial variates (BTRD for n p >= 10, geometric waiting times
//    below; generator/btrd_binomial_distribution.c:43-153) and fold the lower
//    diagonal quadrant into the upper one (clip-and-flip).  Self-loops and
//    repeated edges are kept, as the generator's settings ask
//    (graph_generator.h:60-85).
//  - the vertex permutation and the edge scramble (generator/permutation_gen.c
//    :149-228, scramble_edges.c:35-59, make_graph.c:35-105): every element
//    draws a key, a stable radix sort orders elements by key (equal keys by
//    element index, as the reference's selection sort leaves them), and each
//    group of equal keys is shuffled by Fisher-Yates with its own skipped
//    state.
//
// This file is compiled without floating-point contraction (-fmad=false):
// every product and sum of the binomial draws rounds on its own, as in the
// reference's host build.  Logarithms come from CUDA's math library; a result
// one unit in the last place away from the host's can only change an outcome
// when a uniform variate lands within that unit of a decision threshold.
#include <cub/cub.cuh>

#include <cmath>
#include <cstring>
#include <vector>

#include "common.cuh"

namespace {

constexpr uint64_t KP = 0x7FFFFFFFull;
constexpr uint64_t KMUL1 = 107374182ull;
constexpr uint64_t KMUL5 = 104480ull;
// weights of the two outputs that make one double: 1/(2^31-1), 1/(2^31-1)^2
constexpr double KW1 = .000000000465661287524579692;
constexpr double KW2 = .0000000000000000002168404346990492787;
constexpr int KBITS = 192;
constexpr int KRETRY = 1 << 20;  // bound on rejection loops (expected: a few)

struct KState {
    uint32_t z[5];  // z[0] is the newest output
};

struct KIni {
    double p[4];
};

struct KNode {
    long long fei, cnt;  // first edge index, edge count
    uint32_t bs, bt;     // source and target base of the block
};

__host__ __device__ __forceinline__ uint32_t kmod(uint64_t x)
{
    x = (x & KP) + (x >> 31);
    x = (x & KP) + (x >> 31);
    return (uint32_t)(x >= KP ? x - KP : x);
}

// ---------------------------------------------------------------- host side
struct KTable {
    uint32_t m[KBITS][25];  // A^(2^k), row-major 5x5
};

void kt_mul(uint32_t *r, const uint32_t *a, const uint32_t *b)
{
    uint32_t t[25];
    for (int i = 0; i < 5; i++)
        for (int j = 0; j < 5; j++) {
            uint32_t acc = 0;
            for (int k = 0; k < 5; k++) acc = kmod((uint64_t)acc + (uint64_t)a[5 * i + k] * b[5 * k + j]);
            t[5 * i + j] = acc;
        }
    memcpy(r, t, sizeof(t));
}

KTable make_ktable()
{
    KTable t;
    memset(&t, 0, sizeof(t));
    t.m[0][0] = (uint32_t)KMUL1;
    t.m[0][4] = (uint32_t)KMUL5;
    for (int i = 1; i < 5; i++) t.m[0][5 * i + i - 1] = 1;
    for (int k = 1; k < KBITS; k++) kt_mul(t.m[k], t.m[k - 1], t.m[k - 1]);
    return t;
}

const KTable &ktable()
{
    static const KTable t = make_ktable();
    return t;
}

void kh_apply(KState &s, const uint32_t *m)
{
    uint32_t o[5];
    for (int i = 0; i < 5; i++) {
        uint32_t acc = 0;
        for (int k = 0; k < 5; k++) acc = kmod((uint64_t)acc + (uint64_t)m[5 * i + k] * s.z[k]);
        o[i] = acc;
    }
    memcpy(s.z, o, sizeof(o));
}

void kh_skip(KState &s, uint64_t hi, uint64_t mid, uint64_t lo)
{
    const KTable &t = ktable();
    for (int b = 0; b < 64; b++) {
        if ((lo >> b) & 1) kh_apply(s, t.m[b]);
        if ((mid >> b) & 1) kh_apply(s, t.m[64 + b]);
        if ((hi >> b) & 1) kh_apply(s, t.m[128 + b]);
    }
}

KState kh_seed(uint64_t s1, uint64_t s2)
{
    // make_mrg_seed, generator/utils.c:82-88
    KState s;
    s.z[0] = (uint32_t)((s1 & 0x3FFFFFFF) + 1);
    s.z[1] = (uint32_t)(((s1 >> 30) & 0x3FFFFFFF) + 1);
    s.z[2] = (uint32_t)((s2 & 0x3FFFFFFF) + 1);
    s.z[3] = (uint32_t)(((s2 >> 30) & 0x3FFFFFFF) + 1);
    s.z[4] = (uint32_t)(((s2 >> 60) << 4) + (s1 >> 60) + 1);
    return s;
}

// ---------------------------------------------------------------- device side
__device__ __forceinline__ void kd_apply(KState &s, const uint32_t *__restrict__ m)
{
    uint32_t o[5];
#pragma unroll
    for (int i = 0; i < 5; i++) {
        const uint32_t *r = m + 5 * i;
        // three products < 3 * 2^62, then the fold plus two more < 2^64
        uint64_t a = (uint64_t)__ldg(r) * s.z[0] + (uint64_t)__ldg(r + 1) * s.z[1] +
                     (uint64_t)__ldg(r + 2) * s.z[2];
        uint64_t b = (uint64_t)kmod(a) + (uint64_t)__ldg(r + 3) * s.z[3] + (uint64_t)__ldg(r + 4) * s.z[4];
        o[i] = kmod(b);
    }
#pragma unroll
    for (int i = 0; i < 5; i++) s.z[i] = o[i];
}

__device__ __forceinline__ void kd_skip(KState &s, const uint32_t *__restrict__ tab, uint64_t hi,
                                        uint64_t mid, uint64_t lo)
{
    for (uint64_t w = lo; w; w &= w - 1) kd_apply(s, tab + 25 * (__ffsll((long long)w) - 1));
    for (uint64_t w = mid; w; w &= w - 1) kd_apply(s, tab + 25 * (64 + __ffsll((long long)w) - 1));
    for (uint64_t w = hi; w; w &= w - 1) kd_apply(s, tab + 25 * (128 + __ffsll((long long)w) - 1));
}

__device__ __forceinline__ uint32_t kd_uint(KState &s)
{
    uint32_t nz = kmod(KMUL1 * s.z[0] + KMUL5 * s.z[4]);
    s.z[4] = s.z[3];
    s.z[3] = s.z[2];
    s.z[2] = s.z[1];
    s.z[1] = s.z[0];
    s.z[0] = nz;
    return nz;
}

__device__ __forceinline__ double kd_double(KState &s)
{
    double a = (double)kd_uint(s);  // the first output takes the larger weight
    double b = (double)kd_uint(s);
    return __dadd_rn(__dmul_rn(a, KW1), __dmul_rn(b, KW2));
}

// unbiased integer in [0, n) by rejection, generator/utils.c:50-78
__device__ uint64_t kd_upto(KState &s, uint64_t n, int *err)
{
    if (n <= 1) return 0;
    if (n <= 0x7FFFFFFFull) {
        const uint64_t lim = (0x7FFFFFFFull / n) * n;
        for (int t = 0; t < KRETRY; t++) {
            uint64_t a = kd_uint(s);
            if (a < lim) return a % n;
        }
    } else {
        const uint64_t lim = (0x3FFFFFFF00000001ull / n) * n;
        for (int t = 0; t < KRETRY; t++) {
            uint64_t a = (uint64_t)kd_uint(s) * 0x7FFFFFFFull;
            a += kd_uint(s);
            if (a < lim) return a % n;
        }
    }
    atomicExch(err, 1);
    return 0;
}

// Stirling-series correction log(k!) - [(k+1/2) log(k+1) - (k+1) + log(2 pi)/2]:
// Hoermann's table for k <= 9, the series above
__device__ double kd_fc(int k)
{
    switch (k) {
    case 0: return .08106146679532726;
    case 1: return .04134069595540929;
    case 2: return .02767792568499834;
    case 3: return .02079067210376509;
    case 4: return .01664469118982119;
    case 5: return .01387612882307075;
    case 6: return .01189670994589177;
    case 7: return .01041126526197209;
    case 8: return .009255462182712733;
    case 9: return .008330563433362871;
    default: break;
    }
    double r = 1. / (k + 1);
    return (1. / 12 - (1. / 360 - 1. / 1260 * r * r) * r * r) * r;
}

// binomial(n0, p) for p <= .5, n0 <= 10^9 (btrd_binomial_distribution.c:43-153)
__device__ long long kd_binom_half(long long n0, double p, KState &s, int *err)
{
    if ((double)n0 * p < 10) {
        // waiting times of a geometric variate; ln(1-p) by the series
        // 2/r (1 + 1/(3 r^2) + 1/(5 r^4) + 1/(7 r^6)), r = 1 - 2/p
        double r = 1. - 2. / p;
        double ir = 1. / r, ir2 = ir * ir, ir4 = ir2 * ir2, ir6 = ir4 * ir2;
        double l1p = 2. * ir * (1 + ir2 / 3. + ir4 / 5. + ir6 / 7.);
        double il = 1. / l1p;
        int x = 0, sum = 0;
        for (int t = 0; t < KRETRY; t++) {
            sum += (int)ceil(log(kd_double(s)) * il);
            ++x;
            if ((unsigned long long)sum > (unsigned long long)n0) return x - 1;
        }
        atomicExch(err, 1);
        return 0;
    }
    const int n = (int)n0;
    const int m = (int)floor((n + 1) * p);
    const double r = p / (1. - p);
    const double nr = (n + 1) * r;
    const double npq = n * p * (1. - p);
    const double snpq = sqrt(npq);
    const double b = 1.15 + 2.53 * snpq;
    const double a = -.0873 + .0248 * b + .01 * p;
    const double c = n * p + .5;
    const double alpha = (2.83 + 5.1 / b) * snpq;
    const double vr = .92 - 4.2 / b;
    const double urvr = .86 * vr;
    for (int t = 0; t < KRETRY; t++) {
        double v = kd_double(s), u, us;
        if (v <= urvr) {
            u = v / vr - .43;
            return (int)floor((2 * a / (.5 + fabs(u)) + b) * u + c);
        }
        const double w = kd_double(s);
        if (v >= vr) {
            u = w - .5;
        } else {
            u = v / vr - .93;
            u = (u > 0. ? 1. : u < 0. ? -1. : 0.) * .5 - u;
            v = vr * w;
        }
        us = .5 - fabs(u);
        const int k = (int)floor((2 * a / us + b) * u + c);
        if (k < 0 || k > n) continue;
        v *= alpha / (a / (us * us) + b);
        const int km = k >= m ? k - m : m - k;
        if (km > 15) {
            const double rho = (km / npq) * (((km / 3 + .625) * km + 1. / 6) / npq + .5);
            const double tt = -km * km / (2 * npq);
            v = log(v);
            if (v < tt - rho) return k;
            if (v > tt + rho) continue;
            const int nm = n - m + 1;
            const double h = (m + .5) * log((m + 1) / (r * nm)) + kd_fc(m) + kd_fc(n - m);
            const int nk = n - k + 1;
            const double thr = h + (n + 1) * log((double)nm / nk) + (k + .5) * log(nk * r / (k + 1)) -
                               kd_fc(k) - kd_fc(n - k);
            if (v <= thr) return k;
        } else {
            double f = 1.;
            if (m < k) {
                for (int i = m; i != k; ++i) f *= nr / i - r;
            } else if (m > k) {
                for (int i = k; i != m; ++i) v *= nr / i + r;
            }
            if (v <= f) return k;
        }
    }
    atomicExch(err, 1);
    return 0;
}

__device__ long long kd_binom(long long n0, double p, KState &s, int *err)
{
    if (p == 0.) return 0;
    if (p > .5) {
        const double q = 1. - p;
        return n0 - (q == 0. ? 0 : kd_binom_half(n0, q, s, err));
    }
    return kd_binom_half(n0, p, s, err);
}

__device__ __forceinline__ int kd_quad(KState &s, const KIni &ini)
{
    double r = kd_double(s);
#pragma unroll
    for (int j = 0; j < 3; j++) {
        if (r < ini.p[j]) return j;
        r -= ini.p[j];
    }
    return 3;
}

__device__ __forceinline__ uint64_t kpack(uint32_t s, uint32_t t) { return ((uint64_t)s << 32) | t; }

// One level of the edge split: node i of level d covers a block of side
// 2^(scale-d).  Children are appended to `out` (warp-aggregated), finished
// edges written to `edges` at their edge index.
__global__ void k_kron_level(const KNode *__restrict__ in, unsigned long long nin, int d, int scale,
                             KState root, KIni ini, const uint32_t *__restrict__ tab,
                             KNode *__restrict__ out, unsigned long long *__restrict__ nout,
                             uint64_t *__restrict__ edges, int *__restrict__ err)
{
    const int lane = threadIdx.x & 31;
    const int sh = scale - d;
    for (unsigned long long base = (unsigned long long)blockIdx.x * blockDim.x; base < nin;
         base += (unsigned long long)gridDim.x * blockDim.x) {
        const unsigned long long i = base + threadIdx.x;
        KNode ch[4];
        int nch = 0;
        if (i < nin) {
            const KNode nd = in[i];
            KState s = root;
            kd_skip(s, tab, 0, (uint64_t)(nd.bs >> sh) + (1ull << d), (uint64_t)(nd.bt >> sh) + (1ull << d));
            if (sh == 0) {
                const uint64_t e = kpack(nd.bs, nd.bt);
                for (long long c = 0; c < nd.cnt; c++) edges[nd.fei + c] = e;
            } else if (nd.cnt == 1) {
                uint32_t bs = nd.bs, bt = nd.bt;
                for (int l = sh; l > 0; l--) {
                    const int q = kd_quad(s, ini);
                    uint32_t so = q >> 1, to = q & 1;
                    if (bs == bt && so > to) {
                        so = 0;
                        to = 1;
                    }
                    bs += so << (l - 1);
                    bt += to << (l - 1);
                }
                edges[nd.fei] = kpack(bs, bt);
            } else {
                long long sq[4] = {0, 0, 0, 0};
                if (nd.cnt <= 20) {
                    for (long long e = 0; e < nd.cnt; e++) {
                        double r = kd_double(s);
                        int j = 0;
                        for (; j < 3; j++) {
                            if (r < ini.p[j]) break;
                            r -= ini.p[j];
                        }
                        sq[j]++;
                    }
                } else {
                    long long left = nd.cnt;
                    double dv = 1.;
                    for (int j = 0; j < 3; j++) {
                        sq[j] = kd_binom(left, ini.p[j] / dv, s, err);
                        left -= sq[j];
                        dv -= ini.p[j];
                    }
                    sq[3] = left;
                }
                if (nd.bs == nd.bt) {  // clip-and-flip
                    sq[1] += sq[2];
                    sq[2] = 0;
                }
                const uint32_t h = 1u << (sh - 1);
                long long fei = nd.fei;
                for (int q = 0; q < 4; q++) {
                    if (!sq[q]) continue;
                    ch[nch].fei = fei;
                    ch[nch].cnt = sq[q];
                    ch[nch].bs = nd.bs + h * (uint32_t)(q >> 1);
                    ch[nch].bt = nd.bt + h * (uint32_t)(q & 1);
                    nch++;
                    fei += sq[q];
                }
            }
        }
        // every lane of the warp reaches here in the same iteration
        int incl = nch;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const int y = __shfl_up_sync(FULL_MASK, incl, o);
            if (lane >= o) incl += y;
        }
        unsigned long long at = 0;
        const int tot = __shfl_sync(FULL_MASK, incl, 31);
        if (lane == 31 && tot) at = atomicAdd(nout, (unsigned long long)tot);
        at = __shfl_sync(FULL_MASK, at, 31) + (unsigned long long)(incl - nch);
        for (int c = 0; c < nch; c++) out[at + c] = ch[c];
    }
}

// keys of a keyed bucket sort: element i draws from `base` skipped by i 2^64
__global__ void k_perm_keys(KState base, uint64_t n, uint64_t T, const uint32_t *__restrict__ tab,
                            uint32_t *__restrict__ keys, uint32_t *__restrict__ vals, int *__restrict__ err)
{
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n;
         i += (uint64_t)gridDim.x * blockDim.x) {
        KState s = base;
        kd_skip(s, tab, 0, i, 0);
        keys[i] = (uint32_t)kd_upto(s, T, err);
        vals[i] = (uint32_t)i;
    }
}

// shuffle each run of equal sorted keys with `st` skipped by 2^128 + key 2^64 + 100
__global__ void k_perm_groups(const uint32_t *__restrict__ keys, uint32_t *__restrict__ vals, uint64_t n,
                              KState st, const uint32_t *__restrict__ tab, int *__restrict__ err)
{
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n;
         i += (uint64_t)gridDim.x * blockDim.x) {
        const uint32_t k = keys[i];
        if (i > 0 && keys[i - 1] == k) continue;
        if (i + 1 >= n || keys[i + 1] != k) continue;
        uint64_t e = i + 2;
        while (e < n && keys[e] == k) e++;
        KState s = st;
        kd_skip(s, tab, 1, k, 100);
        for (uint64_t j = e - i - 1; j > 0; j--) {
            const uint64_t r = kd_upto(s, j + 1, err);
            if (r != j) {
                const uint32_t t = vals[i + j];
                vals[i + j] = vals[i + r];
                vals[i + r] = t;
            }
        }
    }
}

// vertex permutation of every edge, stored as (min, max)
__global__ void k_perm_apply(uint64_t *__restrict__ edges, uint64_t m, const uint32_t *__restrict__ perm)
{
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < m;
         i += (uint64_t)gridDim.x * blockDim.x) {
        const uint64_t e = edges[i];
        const uint32_t a = perm[e >> 32], b = perm[(uint32_t)e];
        edges[i] = a < b ? kpack(a, b) : kpack(b, a);
    }
}

__global__ void k_gather_edges(const uint64_t *__restrict__ in, const uint32_t *__restrict__ idx, uint64_t m,
                               uint64_t *__restrict__ out)
{
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < m;
         i += (uint64_t)gridDim.x * blockDim.x)
        out[i] = in[idx[i]];
}

__global__ void k_edges_to_int64(const uint64_t *__restrict__ in, uint64_t m, long long *__restrict__ out)
{
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < m;
         i += (uint64_t)gridDim.x * blockDim.x) {
        const uint64_t e = in[i];
        out[2 * i] = (long long)(e >> 32);
        out[2 * i + 1] = (long long)(uint32_t)e;
    }
}

// adjacency keys of the mirrored edge list: (u,v) and, for u != v, (v,u)
__global__ void k_edges_to_keys(const uint64_t *__restrict__ in, uint64_t m, uint64_t *__restrict__ keys)
{
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < m;
         i += (uint64_t)gridDim.x * blockDim.x) {
        const uint64_t e = in[i];
        const uint32_t u = (uint32_t)(e >> 32), v = (uint32_t)e;
        keys[2 * i] = ((uint64_t)v << 32) | u;
        keys[2 * i + 1] = u == v ? ~0ull : (((uint64_t)u << 32) | v);
    }
}

int grid_for(uint64_t n, int tpb)
{
    int dev = 0, sms = 152;
    if (cudaGetDevice(&dev) == cudaSuccess) cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    uint64_t g = (n + tpb - 1) / tpb;
    uint64_t cap = (uint64_t)sms * 16;
    return (int)(g < 1 ? 1 : (g > cap ? cap : g));
}

int check_err(const int *d_err, const char *what)
{
    int e = 0;
    CU(cudaMemcpy(&e, d_err, sizeof(int), cudaMemcpyDeviceToHost));
    if (e) {
        axbc_set_error("%s: a rejection loop ran past its bound", what);
        return AXBC_ERR_CUDA;
    }
    return AXBC_OK;
}

// keyed bucket sort of 0..n-1 into `perm` (n < 2^31 elements)
int rand_perm(const KState &st, uint64_t n, const uint32_t *d_tab, int *d_err, uint32_t *perm)
{
    if (n == 0) return AXBC_OK;
    const uint64_t T = 2 * n + 128;
    KState base = st;
    kh_skip(base, 1, 0, 0);
    DBuf keys, keys2, vals, tmp;
    TRY(axbc_dalloc(&keys.p, n * 4, nullptr));
    TRY(axbc_dalloc(&keys2.p, n * 4, nullptr));
    TRY(axbc_dalloc(&vals.p, n * 4, nullptr));
    k_perm_keys<<<grid_for(n, 256), 256>>>(base, n, T, d_tab, keys.as<uint32_t>(), vals.as<uint32_t>(), d_err);
    CU_LAUNCH("k_perm_keys");
    int end_bit = 1;
    while (end_bit < 32 && (T - 1) >> end_bit) end_bit++;
    size_t tb = 0;
    cub::DeviceRadixSort::SortPairs(nullptr, tb, keys.as<uint32_t>(), keys2.as<uint32_t>(), vals.as<uint32_t>(),
                                    perm, (int64_t)n, 0, end_bit);
    TRY(axbc_dalloc(&tmp.p, tb, nullptr));
    cub::DeviceRadixSort::SortPairs(tmp.p, tb, keys.as<uint32_t>(), keys2.as<uint32_t>(), vals.as<uint32_t>(),
                                    perm, (int64_t)n, 0, end_bit);
    CU_LAUNCH("radix sort of permutation keys");
    k_perm_groups<<<grid_for(n, 256), 256>>>(keys2.as<uint32_t>(), perm, n, st, d_tab, d_err);
    CU_LAUNCH("k_perm_groups");
    return check_err(d_err, "permutation keys");
}

}  // namespace

// Generate the edge list on the device: stage 0 as split (generator order),
// 1 with the vertex permutation applied ((min, max) pairs), 2 scrambled
// (make_graph's output).  *d_edges receives m packed (source << 32 | target)
// entries allocated with axbc_dalloc.
int axbc_kron_device(int scale, int edgefactor, uint64_t seed1, uint64_t seed2, const double *initiator,
                     int stage, uint64_t **d_edges, uint64_t *m_out)
{
    CHECK_ARG(d_edges && m_out, "kronecker: null output");
    CHECK_ARG(scale >= 1 && scale <= 30, "kronecker: scale must be in [1,30]");
    CHECK_ARG(edgefactor >= 1 && edgefactor <= 1024, "kronecker: edgefactor must be in [1,1024]");
    CHECK_ARG(stage >= 0 && stage <= 2, "kronecker: stage must be 0, 1 or 2");
    const uint64_t N = 1ull << scale, M = N * (uint64_t)edgefactor;
    CHECK_ARG(M <= 1000000000ull,
              "kronecker: at most 10^9 edges (the binomial draws of larger counts split them)");
    KIni ini;
    const double g500[4] = {.57, .19, .19, .05};
    for (int j = 0; j < 4; j++) ini.p[j] = initiator ? initiator[j] : g500[j];
    *d_edges = nullptr;
    *m_out = 0;

    const KTable &tab = ktable();
    DBuf d_tab, d_err, d_n, nodes_a, nodes_b, edges;
    TRY(axbc_dalloc(&d_tab.p, sizeof(KTable), nullptr));
    CU(cudaMemcpy(d_tab.p, &tab, sizeof(KTable), cudaMemcpyHostToDevice));
    TRY(axbc_dalloc(&d_err.p, sizeof(int), nullptr));
    CU(cudaMemset(d_err.p, 0, sizeof(int)));
    TRY(axbc_dalloc(&d_n.p, 8, nullptr));
    TRY(axbc_dalloc(&edges.p, M * 8, nullptr));
    // a level's nodes hold at least one edge each: M bounds every level
    TRY(axbc_dalloc(&nodes_a.p, M * sizeof(KNode), nullptr));
    TRY(axbc_dalloc(&nodes_b.p, M * sizeof(KNode), nullptr));

    const KState root = kh_seed(seed1, seed2);
    KNode top{0, (long long)M, 0, 0};
    CU(cudaMemcpy(nodes_a.p, &top, sizeof(top), cudaMemcpyHostToDevice));
    unsigned long long nin = 1;
    KNode *in = nodes_a.as<KNode>(), *out = nodes_b.as<KNode>();
    for (int d = 0; d <= scale && nin; d++) {
        CU(cudaMemset(d_n.p, 0, 8));
        k_kron_level<<<grid_for(nin, 128), 128>>>(in, nin, d, scale, root, ini, d_tab.as<uint32_t>(), out,
                                                  d_n.as<unsigned long long>(), edges.as<uint64_t>(),
                                                  d_err.as<int>());
        CU_LAUNCH("k_kron_level");
        CU(cudaMemcpy(&nin, d_n.p, 8, cudaMemcpyDeviceToHost));
        KNode *t = in;
        in = out;
        out = t;
    }
    TRY(check_err(d_err.as<int>(), "kronecker edge split"));
    nodes_a.release();
    nodes_b.release();

    if (stage >= 1) {
        DBuf perm;
        TRY(axbc_dalloc(&perm.p, N * 4, nullptr));
        TRY(rand_perm(root, N, d_tab.as<uint32_t>(), d_err.as<int>(), perm.as<uint32_t>()));
        k_perm_apply<<<grid_for(M, 256), 256>>>(edges.as<uint64_t>(), M, perm.as<uint32_t>());
        CU_LAUNCH("k_perm_apply");
    }
    if (stage >= 2) {
        KState st = root;
        kh_skip(st, 5, 0, 0);
        DBuf eperm, scr;
        TRY(axbc_dalloc(&eperm.p, M * 4, nullptr));
        TRY(rand_perm(st, M, d_tab.as<uint32_t>(), d_err.as<int>(), eperm.as<uint32_t>()));
        TRY(axbc_dalloc(&scr.p, M * 8, nullptr));
        k_gather_edges<<<grid_for(M, 256), 256>>>(edges.as<uint64_t>(), eperm.as<uint32_t>(), M,
                                                  scr.as<uint64_t>());
        CU_LAUNCH("k_gather_edges");
        std::swap(edges.p, scr.p);
    }
    CU(cudaDeviceSynchronize());
    *d_edges = edges.as<uint64_t>();
    edges.p = nullptr;
    *m_out = M;
    return AXBC_OK;
}

extern "C" int axbc_kron_edges(int scale, int edgefactor, uint64_t seed1, uint64_t seed2,
                               const double *initiator, int stage, int64_t *edges_host)
{
    CHECK_ARG(edges_host, "axbc_kron_edges: null output");
    uint64_t *d = nullptr, m = 0;
    TRY(axbc_kron_device(scale, edgefactor, seed1, seed2, initiator, stage, &d, &m));
    DBuf e, w;
    e.p = d;
    TRY(axbc_dalloc(&w.p, 2 * m * 8, nullptr));
    k_edges_to_int64<<<grid_for(m, 256), 256>>>(e.as<uint64_t>(), m, w.as<long long>());
    CU_LAUNCH("k_edges_to_int64");
    CU(cudaMemcpy(edges_host, w.p, 2 * m * 8, cudaMemcpyDeviceToHost));
    return AXBC_OK;
}

extern "C" int axbc_graph_generate_kronecker(int scale, int edgefactor, uint64_t seed1, uint64_t seed2,
                                             const double *initiator, int H, axbc_graph **g)
{
    CHECK_ARG(g, "axbc_graph_generate_kronecker: null output");
    CHECK_ARG(H == 0 || H == 1, "axbc_graph_generate_kronecker: H must be 0 or 1");
    uint64_t *d = nullptr, m = 0;
    // the CSC does not depend on the order of the edges: no scramble
    TRY(axbc_kron_device(scale, edgefactor, seed1, seed2, initiator, 1, &d, &m));
    DBuf e, keys;
    e.p = d;
    TRY(axbc_dalloc(&keys.p, 2 * m * 8, nullptr));
    k_edges_to_keys<<<grid_for(m, 256), 256>>>(e.as<uint64_t>(), m, keys.as<uint64_t>());
    CU_LAUNCH("k_edges_to_keys");
    e.release();
    return axbc_keys_to_graph(keys.as<uint64_t>(), 2 * m, 1ull << scale, 1, H, g);
}
