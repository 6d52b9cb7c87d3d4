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

/* Test infrastructure: a plain-C restatement of the Graph500 Kronecker
 * generator that the reference links (generator/, called by gen_graph,
 * src/axbc2d.c:518-527), used as the checker of the library's device
 * generator.  It is checked in turn against the reference generator compiled
 * from its own sources (oracle/_ref) and against the committed fixtures.
 *
 * Pieces, each following the reference file named:
 *   - MRG: L'Ecuyer-Blouin-Couture multiple recursive generator, modulus
 *     2^31-1, order 5, x_n = 107374182 x_{n-1} + 104480 x_{n-5}
 *     (generator/splittable_mrg.c:18-50, 154-165); a skip by e steps applies
 *     A^e to the state vector, e a 192-bit number high:middle:low
 *     (splittable_mrg.c:169-184); here A^(2^k) for k < 192 by repeated
 *     squaring instead of the reference's byte tables;
 *   - uniform double from two outputs (splittable_mrg.c:282-292);
 *   - unbiased integer in [0, n) by rejection (generator/utils.c:50-78);
 *   - seed spreading (utils.c:82-88);
 *   - binomial variates: BTRD (Hoermann, "The generation of binomial random
 *     variates", 1993) for n p >= 10, a geometric waiting-time method below
 *     (generator/btrd_binomial_distribution.c:43-153);
 *   - the recursive edge split over the 2x2 initiator with clip-and-flip,
 *     self-loops and duplicates kept (generator/graph_generator.c:36-83,
 *     98-145, 147-278; settings graph_generator.h:60-85);
 *   - the vertex permutation and the edge scramble by a keyed bucket sort
 *     whose equal-key groups are sorted and then shuffled
 *     (generator/permutation_gen.c:149-228, scramble_edges.c:35-59);
 *   - make_graph's sequential driver (generator/make_graph.c:35-105).
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#define KP 0x7FFFFFFFull
#define KMUL1 107374182ull
#define KMUL5 104480ull

/* 1/(2^31-1) and 1/(2^31-1)^2, the weights of the two outputs of a double */
static const double KW1 = .000000000465661287524579692;
static const double KW2 = .0000000000000000002168404346990492787;

typedef struct {
    uint32_t z[5]; /* z[0] newest output */
} kst;

static uint32_t kmod(uint64_t x) /* x < 2^63 */
{
    x = (x & KP) + (x >> 31);
    x = (x & KP) + (x >> 31);
    return (uint32_t)(x >= KP ? x - KP : x);
}

static uint32_t kpow_tab[192][5][5];
static int kpow_ready = 0;

static void kmatmul(uint32_t r[5][5], uint32_t a[5][5], uint32_t b[5][5])
{
    uint32_t t[5][5];
    for (int i = 0; i < 5; i++)
        for (int j = 0; j < 5; j++) {
            uint32_t acc = 0;
            for (int k = 0; k < 5; k++) acc = kmod((uint64_t)acc + (uint64_t)a[i][k] * b[k][j]);
            t[i][j] = acc;
        }
    memcpy(r, t, sizeof(t));
}

static void kpow_init(void)
{
    if (kpow_ready) return;
    memset(kpow_tab, 0, sizeof(kpow_tab));
    kpow_tab[0][0][0] = (uint32_t)KMUL1;
    kpow_tab[0][0][4] = (uint32_t)KMUL5;
    for (int i = 1; i < 5; i++) kpow_tab[0][i][i - 1] = 1;
    for (int k = 1; k < 192; k++) kmatmul(kpow_tab[k], kpow_tab[k - 1], kpow_tab[k - 1]);
    kpow_ready = 1;
}

static void kapply(kst *s, uint32_t m[5][5])
{
    uint32_t o[5];
    for (int i = 0; i < 5; i++) {
        uint32_t acc = 0;
        for (int k = 0; k < 5; k++) acc = kmod((uint64_t)acc + (uint64_t)m[i][k] * s->z[k]);
        o[i] = acc;
    }
    memcpy(s->z, o, sizeof(o));
}

static void kskip(kst *s, uint64_t hi, uint64_t mid, uint64_t lo)
{
    kpow_init();
    for (int b = 0; b < 64; b++) {
        if ((lo >> b) & 1) kapply(s, kpow_tab[b]);
        if ((mid >> b) & 1) kapply(s, kpow_tab[64 + b]);
        if ((hi >> b) & 1) kapply(s, kpow_tab[128 + b]);
    }
}

static uint32_t kuint(kst *s)
{
    uint32_t nz = kmod(KMUL1 * s->z[0] + KMUL5 * s->z[4]);
    s->z[4] = s->z[3];
    s->z[3] = s->z[2];
    s->z[2] = s->z[1];
    s->z[1] = s->z[0];
    s->z[0] = nz;
    return nz;
}

static double kdouble(kst *s)
{
    double a = (double)kuint(s);
    double b = (double)kuint(s);
    return a * KW1 + b * KW2;
}

static uint64_t kupto(kst *s, uint64_t n)
{
    if (n <= 1) return 0;
    if (n <= 0x7FFFFFFFull) {
        uint64_t lim = (0x7FFFFFFFull / n) * n;
        for (;;) {
            uint64_t a = kuint(s);
            if (a < lim) return a % n;
        }
    }
    uint64_t lim = (0x3FFFFFFF00000001ull / n) * n;
    for (;;) {
        uint64_t a = (uint64_t)kuint(s) * 0x7FFFFFFFull;
        a += kuint(s);
        if (a < lim) return a % n;
    }
}

static void kseed(uint64_t s1, uint64_t s2, kst *s)
{
    s->z[0] = (uint32_t)((s1 & 0x3FFFFFFF) + 1);
    s->z[1] = (uint32_t)(((s1 >> 30) & 0x3FFFFFFF) + 1);
    s->z[2] = (uint32_t)((s2 & 0x3FFFFFFF) + 1);
    s->z[3] = (uint32_t)(((s2 >> 30) & 0x3FFFFFFF) + 1);
    s->z[4] = (uint32_t)(((s2 >> 60) << 4) + (s1 >> 60) + 1);
}

/* Stirling-series correction log(k!) - [(k+1/2) log(k+1) - (k+1) + log(2 pi)/2],
 * tabulated for k <= 9 (values of Hoermann's BTRD table), series above */
static double kfc(unsigned k)
{
    static const double t[10] = {.08106146679532726, .04134069595540929, .02767792568499834,
                                 .02079067210376509, .01664469118982119, .01387612882307075,
                                 .01189670994589177, .01041126526197209, .009255462182712733,
                                 .008330563433362871};
    if (k <= 9) return t[k];
    double r = 1. / (k + 1);
    return (1. / 12 - (1. / 360 - 1. / 1260 * r * r) * r * r) * r;
}

static uint64_t kbinom(uint64_t n0, double p, kst *s)
{
    if (p == 0.) return 0;
    if (p > .5) return n0 - kbinom(n0, 1. - p, s);
    if (n0 * p < 10) {
        /* geometric waiting times; ln(1-p) by the series 2/r (1 + 1/(3r^2) +
         * 1/(5r^4) + 1/(7r^6)), r = 1 - 2/p */
        double r = 1. - 2. / p;
        double ir = 1. / r, ir2 = ir * ir, ir4 = ir2 * ir2, ir6 = ir4 * ir2;
        double l1p = 2. * ir * (1 + ir2 / 3. + ir4 / 5. + ir6 / 7.);
        double il = 1. / l1p;
        int x = 0, sum = 0;
        do {
            sum += (int)ceil(log(kdouble(s)) * il);
            ++x;
        } while ((uint64_t)sum <= n0);
        return (uint64_t)(x - 1);
    }
    if (n0 > 1000000000ull)
        return kbinom(1000000000ull, p, s) + kbinom(n0 - 1000000000ull, p, s);
    int n = (int)n0;
    int m = (int)floor((n + 1) * p);
    double r = p / (1. - p);
    double nr = (n + 1) * r;
    double npq = n * p * (1. - p);
    double snpq = sqrt(npq);
    double b = 1.15 + 2.53 * snpq;
    double a = -.0873 + .0248 * b + .01 * p;
    double c = n * p + .5;
    double alpha = (2.83 + 5.1 / b) * snpq;
    double vr = .92 - 4.2 / b;
    double urvr = .86 * vr;
    for (;;) {
        double v = kdouble(s), u, us;
        if (v <= urvr) {
            u = v / vr - .43;
            return (uint64_t)(int)floor((2 * a / (.5 + fabs(u)) + b) * u + c);
        }
        double w = kdouble(s);
        if (v >= vr) {
            u = w - .5;
        } else {
            u = v / vr - .93;
            u = (u > 0. ? 1. : u < 0. ? -1. : 0.) * .5 - u;
            v = vr * w;
        }
        us = .5 - fabs(u);
        int k = (int)floor((2 * a / us + b) * u + c);
        if (k < 0 || k > n) continue;
        v *= alpha / (a / (us * us) + b);
        int km = k >= m ? k - m : m - k;
        if (km > 15) {
            double rho = (km / npq) * (((km / 3 + .625) * km + 1. / 6) / npq + .5);
            double t = -km * km / (2 * npq);
            v = log(v);
            if (v < t - rho) return (uint64_t)k;
            if (v > t + rho) continue;
            int nm = n - m + 1;
            double h = (m + .5) * log((m + 1) / (r * nm)) + kfc(m) + kfc(n - m);
            int nk = n - k + 1;
            double thr = h + (n + 1) * log((double)nm / nk) + (k + .5) * log(nk * r / (k + 1)) -
                         kfc(k) - kfc(n - k);
            if (v <= thr) return (uint64_t)k;
        } else {
            double f = 1.;
            if (m < k) {
                for (int i = m; i != k; ++i) f *= nr / i - r;
            } else if (m > k) {
                for (int i = k; i != m; ++i) v *= nr / i + r;
            }
            if (v <= f) return (uint64_t)k;
        }
    }
}

typedef struct {
    double ini[4];
    int64_t N;
    kst root;
    int64_t *out;
} kgen;

static int kquad(const kgen *g, kst *s)
{
    double r = kdouble(s);
    for (int j = 0; j < 3; j++) {
        if (r < g->ini[j]) return j;
        r -= g->ini[j];
    }
    return 3;
}

static void knode(const kgen *g, int64_t fei, int64_t cnt, int64_t nv, int64_t bs, int64_t bt)
{
    kst s = g->root;
    kskip(&s, 0, (uint64_t)((bs + g->N) / nv), (uint64_t)((bt + g->N) / nv));
    if (nv == 1) {
        for (int64_t i = 0; i < cnt; i++) {
            g->out[2 * (fei + i)] = bs;
            g->out[2 * (fei + i) + 1] = bt;
        }
        return;
    }
    if (cnt == 1) {
        while (nv > 1) {
            int q = kquad(g, &s);
            int so = q / 2, to = q % 2;
            if (bs == bt && so > to) {
                int t = so;
                so = to;
                to = t;
            }
            nv /= 2;
            bs += nv * so;
            bt += nv * to;
        }
        g->out[2 * fei] = bs;
        g->out[2 * fei + 1] = bt;
        return;
    }
    int64_t sq[4] = {0, 0, 0, 0};
    if (cnt <= 20) {
        for (int64_t e = 0; e < cnt; e++) {
            double r = kdouble(&s);
            for (int j = 0; j < 4; j++) {
                if (r < g->ini[j] || j == 3) {
                    sq[j]++;
                    break;
                }
                r -= g->ini[j];
            }
        }
    } else {
        int64_t left = cnt;
        double div = 1.;
        for (int i = 0; i < 3; i++) {
            sq[i] = (int64_t)kbinom((uint64_t)left, g->ini[i] / div, &s);
            left -= sq[i];
            div -= g->ini[i];
        }
        sq[3] = left;
    }
    if (bs == bt) { /* clip-and-flip: the diagonal block keeps its upper half */
        sq[1] += sq[2];
        sq[2] = 0;
    }
    int64_t h = nv / 2;
    for (int i = 0; i < 4; i++) {
        if (!sq[i]) continue;
        knode(g, fei, sq[i], h, bs + h * (i / 2), bt + h * (i % 2));
        fei += sq[i];
    }
}

/* keyed bucket sort of 0..n-1 (permutation_gen.c:149-228): element i draws a
 * key in [0, 2n+128) from the state skipped by 2^128 + i 2^64; elements with
 * equal keys are taken in increasing order and shuffled (Fisher-Yates) with the
 * state skipped by 2^128 + key 2^64 + 100 */
static int krandperm(const kst *st, int64_t n, int64_t *res)
{
    uint64_t T = 2 * (uint64_t)n + 128;
    uint64_t *key = (uint64_t *)malloc((n ? n : 1) * sizeof(uint64_t));
    uint64_t *cnt = (uint64_t *)calloc(T + 1, sizeof(uint64_t));
    if (!key || !cnt) {
        free(key);
        free(cnt);
        return -1;
    }
    for (int64_t i = 0; i < n; i++) {
        kst s = *st;
        kskip(&s, 1, (uint64_t)i, 0);
        key[i] = kupto(&s, T);
        cnt[key[i] + 1]++;
    }
    for (uint64_t k = 0; k < T; k++) cnt[k + 1] += cnt[k];
    for (int64_t i = 0; i < n; i++) res[cnt[key[i]]++] = i; /* stable: ties by i */
    /* cnt[k] is now the end of bucket k */
    uint64_t start = 0;
    for (uint64_t k = 0; k < T; k++) {
        uint64_t end = cnt[k], bi = end - start;
        if (bi > 1) {
            kst s = *st;
            kskip(&s, 1, k, 100);
            for (uint64_t i = bi - 1; i > 0; i--) {
                uint64_t j = kupto(&s, i + 1);
                if (i != j) {
                    int64_t t = res[start + i];
                    res[start + i] = res[start + j];
                    res[start + j] = t;
                }
            }
        }
        start = end;
    }
    free(key);
    free(cnt);
    return 0;
}

/* make_graph, sequential form.  stage 0: the generator's edges (before the
 * vertex permutation); 1: permuted, each edge as (min, max); 2: and scrambled
 * (make_graph's output).  out holds 2 * 2^scale * edgef int64 values.
 * Returns the edge count, or -1 when memory runs out. */
int64_t orc_kron_edges(int scale, int edgef, uint64_t seed1, uint64_t seed2, const double ini[4],
                       int stage, int64_t *out)
{
    kgen g;
    int64_t N = (int64_t)1 << scale, M = N * edgef;
    memcpy(g.ini, ini, sizeof(g.ini));
    g.N = N;
    kseed(seed1, seed2, &g.root);
    g.out = out;
    if (M > 0) knode(&g, 0, M, N, 0, 0);
    if (stage == 0) return M;
    int64_t *perm = (int64_t *)malloc(N * sizeof(int64_t));
    if (!perm) return -1;
    if (krandperm(&g.root, N, perm)) {
        free(perm);
        return -1;
    }
    for (int64_t i = 0; i < M; i++) {
        int64_t a = perm[out[2 * i]], b = perm[out[2 * i + 1]];
        out[2 * i] = a < b ? a : b;
        out[2 * i + 1] = a < b ? b : a;
    }
    free(perm);
    if (stage == 1) return M;
    kst s = g.root;
    kskip(&s, 5, 0, 0);
    int64_t *ep = (int64_t *)malloc((M ? M : 1) * sizeof(int64_t));
    int64_t *tmp = (int64_t *)malloc((M ? 2 * M : 1) * sizeof(int64_t));
    if (!ep || !tmp || krandperm(&s, M, ep)) {
        free(ep);
        free(tmp);
        return -1;
    }
    for (int64_t i = 0; i < M; i++) {
        tmp[2 * i] = out[2 * ep[i]];
        tmp[2 * i + 1] = out[2 * ep[i] + 1];
    }
    memcpy(out, tmp, 2 * M * sizeof(int64_t));
    free(ep);
    free(tmp);
    return M;
}

/* the key of element i of a keyed bucket sort, for the device tests */
uint64_t orc_kron_perm_key(uint64_t seed1, uint64_t seed2, uint64_t skip_hi, uint64_t i, uint64_t T)
{
    kst s;
    kseed(seed1, seed2, &s);
    if (skip_hi == 5) kskip(&s, 5, 0, 0);
    kskip(&s, 1, i, 0);
    return kupto(&s, T);
}
