// Graphs on the device: upload of the reference's CSC, heavy-vertex work
// items, transpose for directed inputs, device-side synthetic generators and
// the static pivot distributions (degree^2 prefix, neighbour-degree sums,
// local clustering coefficients).
#include <cub/cub.cuh>

#include <algorithm>
#include <atomic>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <unordered_map>
#include <vector>

#include "common.cuh"

// failure injection for tests: the next n device allocations fail; or, armed
// with a skip count, the allocation after the next `skip` fails
static std::atomic<int> g_fail_allocs{0};
static std::atomic<int> g_fail_after{-1};

extern "C" void axbc_inject_alloc_failures(int n) { g_fail_allocs.store(n < 0 ? 0 : n); }
extern "C" void axbc_inject_alloc_failure_after(int skip) { g_fail_after.store(skip < 0 ? -1 : skip); }

// device bytes the library holds, for leak checks
static std::mutex g_live_mu;
static std::unordered_map<void *, size_t> g_live;
static uint64_t g_live_bytes = 0;

extern "C" uint64_t axbc_device_bytes_live(void)
{
    std::lock_guard<std::mutex> lk(g_live_mu);
    return g_live_bytes;
}

static bool injected_failure()
{
    for (int k = g_fail_allocs.load(); k > 0; k = g_fail_allocs.load())
        if (g_fail_allocs.compare_exchange_weak(k, k - 1)) return true;
    for (int k = g_fail_after.load(); k >= 0; k = g_fail_after.load())
        if (g_fail_after.compare_exchange_weak(k, k - 1)) return k == 0;
    return false;
}

int axbc_dalloc(void **p, size_t bytes, uint64_t *acct)
{
    *p = nullptr;
    if (bytes == 0) bytes = 16;
    if (injected_failure()) {
        axbc_set_error("device allocation of %zu bytes refused (injected failure)", bytes);
        return AXBC_ERR_NOMEM;
    }
    cudaError_t e = cudaMalloc(p, bytes);
    if (e != cudaSuccess) {
        (void)cudaGetLastError();
        *p = nullptr;
        axbc_set_error("cudaMalloc(%zu bytes) failed: %s", bytes, cudaGetErrorString(e));
        return AXBC_ERR_NOMEM;
    }
    {
        std::lock_guard<std::mutex> lk(g_live_mu);
        g_live[*p] = bytes;
        g_live_bytes += bytes;
    }
    if (acct) *acct += bytes;
    return AXBC_OK;
}

void axbc_dfree(void *p)
{
    if (!p) return;
    {
        std::lock_guard<std::mutex> lk(g_live_mu);
        auto it = g_live.find(p);
        if (it != g_live.end()) {
            g_live_bytes -= it->second;
            g_live.erase(it);
        }
    }
    cudaFree(p);
}

// ------------------------------------------------------------------ upload

static void heavy_lists(const uint32_t *col, uint64_t n, std::vector<uint32_t> &hv,
                        std::vector<uint32_t> &hfirst, std::vector<uint32_t> &iv,
                        std::vector<uint32_t> &ik, uint32_t *maxdeg)
{
    uint32_t md = 0;
    for (uint64_t v = 0; v < n; v++) {
        uint32_t d = col[v + 1] - col[v];
        md = std::max(md, d);
        if (d > AXBC_SPAN) {
            hv.push_back((uint32_t)v);
            hfirst.push_back((uint32_t)iv.size());
            uint32_t spans = (d + AXBC_SPAN - 1) / AXBC_SPAN;
            for (uint32_t k = 0; k < spans; k++) {
                iv.push_back((uint32_t)v);
                ik.push_back(k);
            }
        }
    }
    if (maxdeg) *maxdeg = std::max(*maxdeg, md);
}

// Vertices by degree, descending (counting sort, ties by id), and light tasks
// of at most 32 vertices and about one span of adjacency each.
static void task_tables(const uint32_t *col, uint64_t n, std::vector<uint32_t> &order,
                        std::vector<uint32_t> &ltask, uint64_t n_heavy)
{
    uint32_t md = 0;
    for (uint64_t v = 0; v < n; v++) md = std::max(md, col[v + 1] - col[v]);
    std::vector<uint64_t> cnt((size_t)md + 2, 0);
    for (uint64_t v = 0; v < n; v++) cnt[md - (col[v + 1] - col[v])]++;
    uint64_t acc = 0;
    for (auto &c : cnt) {
        uint64_t t = c;
        c = acc;
        acc += t;
    }
    order.resize(n);
    for (uint64_t v = 0; v < n; v++) order[cnt[md - (col[v + 1] - col[v])]++] = (uint32_t)v;
    // light tasks: weight = degree + 8 per vertex, budget one span
    ltask.clear();
    uint64_t i = n_heavy;
    while (i < n) {
        ltask.push_back((uint32_t)i);
        uint64_t w = 0, k = 0;
        while (i < n && k < 32) {
            const uint64_t d = col[order[i] + 1] - col[order[i]];
            if (k > 0 && w + d + 8 > AXBC_SPAN) break;
            w += d + 8;
            k++;
            i++;
        }
    }
    ltask.push_back((uint32_t)n);
}

// heavy-vertex span items and light-vertex tasks of an adjacency whose col
// (host copy: col) is on the device
static int adj_tables(Adj &a, const uint32_t *col, uint64_t n, uint64_t *acct, uint32_t *maxdeg)
{
    std::vector<uint32_t> hv, hf, iv, ik;
    heavy_lists(col, n, hv, hf, iv, ik, maxdeg);
    a.n_heavy = (uint32_t)hv.size();
    a.n_heavy_items = iv.size();
    TRY(axbc_dalloc((void **)&a.heavy_v, hv.size() * 4, acct));
    TRY(axbc_dalloc((void **)&a.heavy_first, (hf.size() + 1) * 4, acct));
    TRY(axbc_dalloc((void **)&a.hitem_v, iv.size() * 4, acct));
    TRY(axbc_dalloc((void **)&a.hitem_k, ik.size() * 4, acct));
    hf.push_back((uint32_t)iv.size());
    if (!hv.empty()) CU(cudaMemcpy(a.heavy_v, hv.data(), hv.size() * 4, cudaMemcpyHostToDevice));
    CU(cudaMemcpy(a.heavy_first, hf.data(), hf.size() * 4, cudaMemcpyHostToDevice));
    if (!iv.empty()) {
        CU(cudaMemcpy(a.hitem_v, iv.data(), iv.size() * 4, cudaMemcpyHostToDevice));
        CU(cudaMemcpy(a.hitem_k, ik.data(), ik.size() * 4, cudaMemcpyHostToDevice));
    }
    std::vector<uint32_t> order, ltask;
    task_tables(col, n, order, ltask, a.n_heavy);
    a.n_ltask = ltask.size() - 1;
    TRY(axbc_dalloc((void **)&a.order, n * 4, acct));
    TRY(axbc_dalloc((void **)&a.ltask, ltask.size() * 4, acct));
    CU(cudaMemcpy(a.order, order.data(), n * 4, cudaMemcpyHostToDevice));
    CU(cudaMemcpy(a.ltask, ltask.data(), ltask.size() * 4, cudaMemcpyHostToDevice));
    return AXBC_OK;
}

static int upload_adj(Adj &a, const uint32_t *col, const uint32_t *row, uint64_t n, uint64_t m,
                      uint64_t *acct, uint32_t *maxdeg)
{
    a.n = n;
    a.m = m;
    a.owns = true;
    TRY(axbc_dalloc((void **)&a.col, (n + 1) * 4, acct));
    TRY(axbc_dalloc((void **)&a.row, m * 4, acct));
    CU(cudaMemcpy(a.col, col, (n + 1) * 4, cudaMemcpyHostToDevice));
    if (m) CU(cudaMemcpy(a.row, row, m * 4, cudaMemcpyHostToDevice));
    return adj_tables(a, col, n, acct, maxdeg);
}

// ------------------------------------------------------------ batch view

// view adjacency: the list of view vertex i is the list of vertex order[i],
// in its own order, its entries renumbered (one warp per vertex)
__global__ void k_view_rows(const uint32_t *__restrict__ col, const uint32_t *__restrict__ row,
                            const uint32_t *__restrict__ order, const uint32_t *__restrict__ to_view,
                            const uint32_t *__restrict__ vcol, uint32_t *__restrict__ vrow, uint64_t n)
{
    const unsigned lane = threadIdx.x & 31;
    const uint64_t nw = (uint64_t)gridDim.x * blockDim.x / 32;
    for (uint64_t i = (blockIdx.x * (uint64_t)blockDim.x + threadIdx.x) / 32; i < n; i += nw) {
        const uint32_t v = order[i];
        const uint32_t b = col[v], d = col[v + 1] - b, o = vcol[i];
        for (uint32_t k = lane; k < d; k += 32) vrow[o + k] = to_view[row[b + k]];
    }
}

__global__ void k_view_gather(const uint32_t *__restrict__ src, const uint32_t *__restrict__ order,
                              uint32_t *__restrict__ dst, uint64_t n)
{
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n;
         i += (uint64_t)gridDim.x * blockDim.x)
        dst[i] = src[order[i]];
}

// src (on the device, host copy of its col: col) in view numbering
static int view_adj(Adj &dst, const Adj &src, const uint32_t *col, const std::vector<uint32_t> &order,
                    const uint32_t *d_order, const uint32_t *d_to_view, uint64_t *acct)
{
    const uint64_t n = src.n, m = src.m;
    std::vector<uint32_t> vcol(n + 1);
    vcol[0] = 0;
    for (uint64_t i = 0; i < n; i++) vcol[i + 1] = vcol[i] + (col[order[i] + 1] - col[order[i]]);
    dst.n = n;
    dst.m = m;
    dst.owns = true;
    TRY(axbc_dalloc((void **)&dst.col, (n + 1) * 4, acct));
    TRY(axbc_dalloc((void **)&dst.row, m * 4, acct));
    CU(cudaMemcpy(dst.col, vcol.data(), (n + 1) * 4, cudaMemcpyHostToDevice));
    if (m) {
        k_view_rows<<<2048, 256>>>(src.col, src.row, d_order, d_to_view, dst.col, dst.row, n);
        CU_LAUNCH("k_view_rows");
    }
    return adj_tables(dst, vcol.data(), n, acct, nullptr);
}

// The batched passes' view (see axbc_graph): renumbered by descending degree
// when the largest degree exceeds AXBC_RENUMBER_MIN_DEG, else the graph itself.
static int build_view(axbc_graph *g, const uint32_t *col, const uint32_t *tcol)
{
    const uint64_t n = g->n;
    if (g->max_deg <= AXBC_RENUMBER_MIN_DEG || n < 2) {
        g->bfwd = g->fwd;
        g->bfwd.owns = false;
        g->brev = g->rev;
        g->brev.owns = false;
        g->breach = g->reach;
        g->renumbered = false;
        return AXBC_OK;
    }
    g->renumbered = true;
    // descending degree, ties by id (counting sort)
    uint32_t md = 0;
    for (uint64_t v = 0; v < n; v++) md = std::max(md, col[v + 1] - col[v]);
    std::vector<uint64_t> cnt((size_t)md + 2, 0);
    for (uint64_t v = 0; v < n; v++) cnt[md - (col[v + 1] - col[v])]++;
    uint64_t acc = 0;
    for (auto &c : cnt) {
        const uint64_t t = c;
        c = acc;
        acc += t;
    }
    std::vector<uint32_t> order(n), to_view(n);
    for (uint64_t v = 0; v < n; v++) order[cnt[md - (col[v + 1] - col[v])]++] = (uint32_t)v;
    for (uint64_t i = 0; i < n; i++) to_view[order[i]] = (uint32_t)i;
    TRY(axbc_dalloc((void **)&g->from_view, n * 4, &g->bytes));
    TRY(axbc_dalloc((void **)&g->to_view, n * 4, &g->bytes));
    TRY(axbc_dalloc((void **)&g->breach, n * 4, &g->bytes));
    CU(cudaMemcpy(g->from_view, order.data(), n * 4, cudaMemcpyHostToDevice));
    CU(cudaMemcpy(g->to_view, to_view.data(), n * 4, cudaMemcpyHostToDevice));
    k_view_gather<<<1024, 256>>>(g->reach, g->from_view, g->breach, n);
    CU_LAUNCH("k_view_gather");
    TRY(view_adj(g->bfwd, g->fwd, col, order, g->from_view, g->to_view, &g->bytes));
    if (g->symmetric) {
        g->brev = g->bfwd;
        g->brev.owns = false;
    } else {
        TRY(view_adj(g->brev, g->rev, tcol, order, g->from_view, g->to_view, &g->bytes));
    }
    CU(cudaDeviceSynchronize());
    return AXBC_OK;
}

static void free_adj(Adj &a)
{
    if (!a.owns) {
        a = Adj();
        return;
    }
    axbc_dfree(a.col);
    axbc_dfree(a.row);
    axbc_dfree(a.heavy_v);
    axbc_dfree(a.heavy_first);
    axbc_dfree(a.hitem_v);
    axbc_dfree(a.hitem_k);
    axbc_dfree(a.order);
    axbc_dfree(a.ltask);
    a = Adj();
}

// transpose of a CSC: column r of the result lists, ascending, the columns c
// whose list contains r
static void transpose_host(const uint32_t *col, const uint32_t *row, uint64_t n, uint64_t m,
                           std::vector<uint32_t> &tcol, std::vector<uint32_t> &trow)
{
    tcol.assign(n + 1, 0);
    trow.resize(m);
    for (uint64_t e = 0; e < m; e++) tcol[row[e] + 1]++;
    for (uint64_t v = 0; v < n; v++) tcol[v + 1] += tcol[v];
    std::vector<uint32_t> pos(tcol.begin(), tcol.end() - 1);
    for (uint64_t c = 0; c < n; c++)
        for (uint32_t e = col[c]; e < col[c + 1]; e++) trow[pos[row[e]]++] = (uint32_t)c;
}

static int graph_from_host(const uint32_t *col, const uint32_t *row, uint64_t n, uint64_t m,
                           const uint32_t *reach, int known_symmetric, axbc_graph **out)
{
    axbc_graph *g = new axbc_graph();
    CU(cudaGetDevice(&g->device));
    g->n = n;
    g->m = m;
    int rc = upload_adj(g->fwd, col, row, n, m, &g->bytes, &g->max_deg);
    if (rc) {
        axbc_graph_destroy(g);
        return rc;
    }
    bool sym = known_symmetric != 0;
    std::vector<uint32_t> tcol, trow;
    if (!sym) {
        transpose_host(col, row, n, m, tcol, trow);
        sym = std::equal(tcol.begin(), tcol.end(), col) &&
              (m == 0 || std::equal(trow.begin(), trow.end(), row));
    }
    g->symmetric = sym;
    if (sym) {
        g->rev = g->fwd;
        g->rev.owns = false;
    } else {
        rc = upload_adj(g->rev, tcol.data(), trow.data(), n, m, &g->bytes, &g->max_deg);
        if (rc) {
            axbc_graph_destroy(g);
            return rc;
        }
    }
    rc = axbc_dalloc((void **)&g->reach, n * 4, &g->bytes);
    if (rc) {
        axbc_graph_destroy(g);
        return rc;
    }
    if (reach) CU(cudaMemcpy(g->reach, reach, n * 4, cudaMemcpyHostToDevice));
    else CU(cudaMemset(g->reach, 0, n * 4));
    rc = build_view(g, col, sym ? col : tcol.data());
    if (rc) {
        axbc_graph_destroy(g);
        return rc;
    }
    *out = g;
    return AXBC_OK;
}

extern "C" int axbc_graph_create(const uint32_t *col, const uint32_t *row, uint64_t n, uint64_t m,
                                 const uint32_t *reach, axbc_graph **g)
{
    CHECK_ARG(g && col && (row || m == 0), "axbc_graph_create: null argument");
    CHECK_ARG(n > 0 && n < 0xffffffffull, "axbc_graph_create: n must be in [1, 2^32-1)");
    CHECK_ARG(col[0] == 0 && col[n] == m, "axbc_graph_create: col[0] must be 0 and col[n] == m");
    for (uint64_t v = 0; v < n; v++)
        CHECK_ARG(col[v] <= col[v + 1], "axbc_graph_create: col is not non-decreasing");
    for (uint64_t e = 0; e < m; e++)
        CHECK_ARG(row[e] < n, "axbc_graph_create: row id out of range");
    return graph_from_host(col, row, n, m, reach, 0, g);
}

extern "C" int axbc_graph_destroy(axbc_graph *g)
{
    if (!g) return AXBC_OK;
    free_adj(g->brev);
    free_adj(g->bfwd);
    if (g->renumbered) {
        axbc_dfree(g->breach);
        axbc_dfree(g->to_view);
        axbc_dfree(g->from_view);
    }
    free_adj(g->rev);
    free_adj(g->fwd);
    axbc_dfree(g->reach);
    axbc_dfree(g->deg2p);
    axbc_dfree(g->sdn);
    axbc_dfree(g->seg_end);
    axbc_dfree(g->lcc);
    axbc_dfree(g->lcc_local);
    axbc_dfree(g->lcc_csum);
    delete g;
    return AXBC_OK;
}

extern "C" int axbc_graph_info(const axbc_graph *g, uint64_t *n, uint64_t *m, uint64_t *bytes,
                               int *symmetric)
{
    CHECK_ARG(g, "axbc_graph_info: null graph");
    if (n) *n = g->n;
    if (m) *m = g->m;
    if (bytes) *bytes = g->bytes;
    if (symmetric) *symmetric = g->symmetric;
    return AXBC_OK;
}

__global__ void k_degrees(const uint32_t *__restrict__ col, uint32_t *__restrict__ deg, uint64_t n)
{
    for (uint64_t v = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; v < n;
         v += (uint64_t)gridDim.x * blockDim.x)
        deg[v] = col[v + 1] - col[v];
}

extern "C" int axbc_graph_get_deg(const axbc_graph *g, uint32_t *deg_host)
{
    CHECK_ARG(g && deg_host, "axbc_graph_get_deg: null argument");
    uint32_t *d = nullptr;
    TRY(axbc_dalloc((void **)&d, g->n * 4, nullptr));
    k_degrees<<<1024, 256>>>(g->fwd.col, d, g->n);
    cudaError_t e = cudaGetLastError();
    if (e == cudaSuccess) e = cudaMemcpy(deg_host, d, g->n * 4, cudaMemcpyDeviceToHost);
    axbc_dfree(d);
    if (e != cudaSuccess) return axbc_cuda_fail(e, "get_deg", __FILE__, __LINE__);
    return AXBC_OK;
}

extern "C" int axbc_graph_get_csc(const axbc_graph *g, uint32_t *col_host, uint32_t *row_host,
                                  uint32_t *reach_host)
{
    CHECK_ARG(g, "axbc_graph_get_csc: null graph");
    if (col_host) CU(cudaMemcpy(col_host, g->fwd.col, (g->n + 1) * 4, cudaMemcpyDeviceToHost));
    if (row_host && g->m) CU(cudaMemcpy(row_host, g->fwd.row, g->m * 4, cudaMemcpyDeviceToHost));
    if (reach_host) CU(cudaMemcpy(reach_host, g->reach, g->n * 4, cudaMemcpyDeviceToHost));
    return AXBC_OK;
}

// ------------------------------------------------------------ generators

// splitmix64 finaliser: the counter-based random source of the generators
__device__ __forceinline__ uint64_t mix64(uint64_t z)
{
    z += 0x9E3779B97F4A7C15ull;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

// bijective scramble of [0, 2^bits): odd multiplies and xor-shifts mod 2^bits
__device__ __forceinline__ uint32_t scramble(uint32_t x, int bits, uint64_t seed)
{
    const uint64_t mask = (bits >= 64) ? ~0ull : ((1ull << bits) - 1);
    uint64_t y = x;
    uint64_t a = (mix64(seed) | 1ull), b = mix64(seed + 1), c = (mix64(seed + 2) | 1ull);
    y = (y * a + b) & mask;
    y ^= y >> (bits / 2 + 1);
    y = (y * c) & mask;
    y ^= y >> (bits / 3 + 1);
    y = (y * a + c) & mask;
    return (uint32_t)y;
}

// key of a directed adjacency entry in CSC order: column (second vertex) in
// the high half, row (first vertex) in the low half
__host__ __device__ __forceinline__ uint64_t ckey(uint32_t u, uint32_t v) { return ((uint64_t)v << 32) | u; }

// R-MAT: edge e descends `scale` levels choosing quadrant a/b/c/d with
// probabilities .57/.19/.19/.05
__global__ void k_rmat(uint64_t nedges, int scale, uint64_t seed, int directed,
                       uint64_t *__restrict__ keys, unsigned long long *__restrict__ nkeys)
{
    const uint32_t TA = (uint32_t)(0.57 * 4294967296.0);
    const uint32_t TB = (uint32_t)(0.76 * 4294967296.0);
    const uint32_t TC = (uint32_t)(0.95 * 4294967296.0);
    for (uint64_t e = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; e < nedges;
         e += (uint64_t)gridDim.x * blockDim.x) {
        uint32_t u = 0, v = 0;
        uint64_t h = 0;
        for (int l = 0; l < scale; l++) {
            if ((l & 1) == 0) h = mix64(seed ^ (e * 0xD6E8FEB86659FD93ull + (uint64_t)l));
            uint32_t r = (l & 1) ? (uint32_t)(h >> 32) : (uint32_t)h;
            uint32_t bu = 0, bv = 0;
            if (r < TA) {
            } else if (r < TB) {
                bv = 1;
            } else if (r < TC) {
                bu = 1;
            } else {
                bu = 1;
                bv = 1;
            }
            u = (u << 1) | bu;
            v = (v << 1) | bv;
        }
        u = scramble(u, scale, seed * 31 + 7);
        v = scramble(v, scale, seed * 31 + 7);
        keys[2 * e] = ckey(u, v);
        keys[2 * e + 1] = (directed || u == v) ? ~0ull : ckey(v, u);
    }
    (void)nkeys;
}

// grid edges: index < nh horizontal (x,y)-(x+1,y), else vertical (x,y)-(x,y+1)
__global__ void k_grid(uint32_t side, uint64_t nh, uint64_t ntot, uint32_t keep_thr, uint64_t seed,
                       uint64_t *__restrict__ keys, unsigned long long *__restrict__ kept)
{
    unsigned long long local = 0;
    for (uint64_t e = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; e < ntot;
         e += (uint64_t)gridDim.x * blockDim.x) {
        uint32_t a, b;
        if (e < nh) {
            uint32_t y = (uint32_t)(e / (side - 1)), x = (uint32_t)(e % (side - 1));
            a = y * side + x;
            b = a + 1;
        } else {
            uint64_t f = e - nh;
            uint32_t y = (uint32_t)(f / side), x = (uint32_t)(f % side);
            a = y * side + x;
            b = a + side;
        }
        bool keep = (uint32_t)mix64(seed ^ (e * 0x9E3779B97F4A7C15ull)) >= keep_thr;
        keys[2 * e] = keep ? ckey(a, b) : ~0ull;
        keys[2 * e + 1] = keep ? ckey(b, a) : ~0ull;
        local += keep;
    }
    atomicAdd(kept, local);
}

__global__ void k_longrange(uint64_t count, uint64_t nverts, uint64_t seed, uint64_t *__restrict__ keys)
{
    for (uint64_t e = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; e < count;
         e += (uint64_t)gridDim.x * blockDim.x) {
        uint64_t h = mix64(seed ^ (0xA5A5A5A5ull + e * 0xD6E8FEB86659FD93ull));
        uint32_t a = (uint32_t)((h & 0xffffffffull) % nverts);
        uint32_t b = (uint32_t)((h >> 32) % nverts);
        keys[2 * e] = ckey(a, b);
        keys[2 * e + 1] = (a == b) ? ~0ull : ckey(b, a);
    }
}

// keep the first copy of every key, drop self-loops except `quirk` (the
// lexicographically first (u,v) edge, which norm_graph always keeps),
// src/axbc2d.c:818-841
__global__ void k_mark(const uint64_t *__restrict__ keys, uint64_t nk, uint64_t quirk,
                       uint8_t *__restrict__ flag)
{
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < nk;
         i += (uint64_t)gridDim.x * blockDim.x) {
        uint64_t k = keys[i];
        bool f = (k != ~0ull) && (i == 0 || keys[i - 1] != k);
        uint32_t u = (uint32_t)k, v = (uint32_t)(k >> 32);
        if (f && u == v && k != quirk) f = false;
        flag[i] = f;
    }
}

__global__ void k_split(const uint64_t *__restrict__ keys, uint64_t m, uint32_t *__restrict__ row,
                        uint32_t *__restrict__ cnt)
{
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < m;
         i += (uint64_t)gridDim.x * blockDim.x) {
        uint64_t k = keys[i];
        row[i] = (uint32_t)k;
        atomicAdd(&cnt[(uint32_t)(k >> 32)], 1u);
    }
}

// lexicographically smallest (u,v) = (row, column) among valid keys
__global__ void k_min_uv(const uint64_t *__restrict__ keys, uint64_t nk, unsigned long long *out)
{
    unsigned long long best = ~0ull;
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < nk;
         i += (uint64_t)gridDim.x * blockDim.x) {
        uint64_t k = keys[i];
        if (k == ~0ull) continue;
        unsigned long long uv = ((unsigned long long)(uint32_t)k << 32) | (k >> 32);
        best = best < uv ? best : uv;
    }
    atomicMin(out, best);
}

// One-degree reduction of a sorted, duplicate-free symmetric list on the device
// (degree_reduction, src/axbc2d.c:695-807).  Entry i is the pair (a, b) = (key
// >> 32, key & 0xffffffff); the list is ordered by (a, b), the order the
// reference sorts (u, v) pairs in, because the pair set is symmetric.
//   - entry i is a leaf entry when a != b and it is the only entry of a;
//   - entries that are neither leaf entries nor self-loops form the kept list;
//     a kept entry (x, y) is dropped when y is a leaf vertex: the reference's
//     merge of the removed pairs (y's neighbour, y) against the kept list
//     finds exactly these, since every such pair is in the kept list;
//   - reach[x] counts the removed pairs (x, leaf) that the merge consumed:
//     those with x <= the first vertex of the last kept entry (none when the
//     kept list is empty).
__global__ void k_leaf_entries(const uint64_t *__restrict__ keys, uint64_t m, uint8_t *__restrict__ leafv,
                               uint8_t *__restrict__ kind, unsigned long long *__restrict__ last_kept)
{
    unsigned long long best = 0;
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < m;
         i += (uint64_t)gridDim.x * blockDim.x) {
        const uint64_t k = keys[i];
        const uint32_t a = (uint32_t)(k >> 32), b = (uint32_t)k;
        const bool alone = (i == 0 || (uint32_t)(keys[i - 1] >> 32) != a) &&
                           (i + 1 == m || (uint32_t)(keys[i + 1] >> 32) != a);
        uint8_t t;
        if (a == b) {
            t = 0;  // self-loop: dropped
        } else if (alone) {
            t = 1;  // leaf entry
            leafv[a] = 1;
        } else {
            t = 2;  // kept entry
            best = best > i + 1 ? best : i + 1;
        }
        kind[i] = t;
    }
    atomicMax(last_kept, best);
}

__global__ void k_leaf_reduce(const uint64_t *__restrict__ keys, uint64_t m, const uint8_t *__restrict__ leafv,
                              uint8_t *__restrict__ kind, uint32_t *__restrict__ reach,
                              const unsigned long long *__restrict__ last_kept)
{
    const unsigned long long lk = *last_kept;  // 1 + index of the last kept entry, 0 if none
    const uint32_t amax = lk ? (uint32_t)(keys[lk - 1] >> 32) : 0;
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < m;
         i += (uint64_t)gridDim.x * blockDim.x) {
        const uint64_t k = keys[i];
        const uint32_t b = (uint32_t)k;
        if (kind[i] == 1) {
            if (lk && b <= amax) atomicAdd(&reach[b], 1u);
            kind[i] = 0;
        } else if (kind[i] == 2) {
            kind[i] = leafv[b] ? 0 : 1;
        }
    }
}

// Sort device keys, dedupe, reduce degree-1 vertices (H == 1), build the CSC
// and wrap it in a graph.

int axbc_keys_to_graph(uint64_t *d_keys, uint64_t nk, uint64_t n, int symmetric, int H,
                       axbc_graph **out)
{
    cudaStream_t s = 0;
    size_t tmp_bytes = 0;
    unsigned long long m = 0;
    {
        DBuf sorted, tmp, mn, flag, nsel;
        TRY(sorted.alloc(nk * 8));
        // all 64 bits: the all-ones padding keys must sort last
        cub::DeviceRadixSort::SortKeys(nullptr, tmp_bytes, d_keys, sorted.as<uint64_t>(), (int64_t)nk, 0, 64, s);
        TRY(tmp.alloc(tmp_bytes));
        cub::DeviceRadixSort::SortKeys(tmp.p, tmp_bytes, d_keys, sorted.as<uint64_t>(), (int64_t)nk, 0, 64, s);
        CU_LAUNCH("radix sort");
        tmp.release();

        TRY(mn.alloc(8));
        CU(cudaMemset(mn.p, 0xff, 8));
        k_min_uv<<<1024, 256>>>(sorted.as<uint64_t>(), nk, mn.as<unsigned long long>());
        unsigned long long minuv = ~0ull;
        CU(cudaMemcpy(&minuv, mn.p, 8, cudaMemcpyDeviceToHost));
        uint64_t quirk = ~0ull;
        if (minuv != ~0ull && (uint32_t)(minuv >> 32) == (uint32_t)minuv)
            quirk = ckey((uint32_t)minuv, (uint32_t)minuv);

        TRY(flag.alloc(nk));
        k_mark<<<2048, 256>>>(sorted.as<uint64_t>(), nk, quirk, flag.as<uint8_t>());
        CU_LAUNCH("k_mark");
        TRY(nsel.alloc(8));
        tmp_bytes = 0;
        cub::DeviceSelect::Flagged(nullptr, tmp_bytes, sorted.as<uint64_t>(), flag.as<uint8_t>(), d_keys,
                                   nsel.as<unsigned long long>(), (int64_t)nk, s);
        TRY(tmp.alloc(tmp_bytes));
        cub::DeviceSelect::Flagged(tmp.p, tmp_bytes, sorted.as<uint64_t>(), flag.as<uint8_t>(), d_keys,
                                   nsel.as<unsigned long long>(), (int64_t)nk, s);
        CU_LAUNCH("select");
        CU(cudaMemcpy(&m, nsel.p, 8, cudaMemcpyDeviceToHost));
    }
    if (m >= 0xffffffffull) {
        axbc_set_error("graph has %llu adjacency entries; 32-bit offsets hold < 2^32", m);
        return AXBC_ERR_RANGE;
    }

    std::vector<uint32_t> reach;
    if (H == 1 && m > 0) {
        if (!symmetric) {
            axbc_set_error("one-degree reduction of a generated graph needs a symmetric graph");
            return AXBC_ERR_INVALID;
        }
        DBuf leafv, kind, dreach, last, kept, nsel, tmp;
        TRY(leafv.alloc(n));
        TRY(kind.alloc(m));
        TRY(dreach.alloc(n * 4));
        TRY(last.alloc(8));
        CU(cudaMemset(leafv.p, 0, n));
        CU(cudaMemset(dreach.p, 0, n * 4));
        CU(cudaMemset(last.p, 0, 8));
        k_leaf_entries<<<2048, 256>>>(d_keys, m, leafv.as<uint8_t>(), kind.as<uint8_t>(),
                                      last.as<unsigned long long>());
        CU_LAUNCH("k_leaf_entries");
        k_leaf_reduce<<<2048, 256>>>(d_keys, m, leafv.as<uint8_t>(), kind.as<uint8_t>(), dreach.as<uint32_t>(),
                                     last.as<unsigned long long>());
        CU_LAUNCH("k_leaf_reduce");
        TRY(kept.alloc(m * 8));
        TRY(nsel.alloc(8));
        tmp_bytes = 0;
        cub::DeviceSelect::Flagged(nullptr, tmp_bytes, d_keys, kind.as<uint8_t>(), kept.as<uint64_t>(),
                                   nsel.as<unsigned long long>(), (int64_t)m, s);
        TRY(tmp.alloc(tmp_bytes));
        cub::DeviceSelect::Flagged(tmp.p, tmp_bytes, d_keys, kind.as<uint8_t>(), kept.as<uint64_t>(),
                                   nsel.as<unsigned long long>(), (int64_t)m, s);
        CU_LAUNCH("select kept entries");
        CU(cudaMemcpy(&m, nsel.p, 8, cudaMemcpyDeviceToHost));
        CU(cudaMemcpy(d_keys, kept.p, m * 8, cudaMemcpyDeviceToDevice));
        reach.resize(n);
        CU(cudaMemcpy(reach.data(), dreach.p, n * 4, cudaMemcpyDeviceToHost));
    }

    std::vector<uint32_t> col(n + 1), cnt(n + 1), row(m);
    {
        DBuf drow, dcnt;
        TRY(drow.alloc(m * 4));
        TRY(dcnt.alloc((n + 1) * 4));
        CU(cudaMemset(dcnt.p, 0, (n + 1) * 4));
        k_split<<<2048, 256>>>(d_keys, m, drow.as<uint32_t>(), dcnt.as<uint32_t>());
        CU_LAUNCH("k_split");
        CU(cudaMemcpy(cnt.data(), dcnt.p, (n + 1) * 4, cudaMemcpyDeviceToHost));
        CU(cudaMemcpy(row.data(), drow.p, m * 4, cudaMemcpyDeviceToHost));
    }
    col[0] = 0;
    for (uint64_t v = 0; v < n; v++) col[v + 1] = col[v] + cnt[v];
    return graph_from_host(col.data(), row.data(), n, m, reach.empty() ? nullptr : reach.data(), symmetric, out);
}

// adjacency keys of a host edge list: (u,v) and, when mirrored and u != v, (v,u)
__global__ void k_list_to_keys(const uint64_t *__restrict__ edges, uint64_t ne, uint64_t n, int mirror,
                               uint64_t *__restrict__ keys, int *__restrict__ bad)
{
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < ne;
         i += (uint64_t)gridDim.x * blockDim.x) {
        const uint64_t u = edges[2 * i], v = edges[2 * i + 1];
        if (u >= n || v >= n) {
            atomicExch(bad, 1);
            keys[(mirror ? 2 : 1) * i] = ~0ull;
            if (mirror) keys[2 * i + 1] = ~0ull;
            continue;
        }
        if (mirror) {
            keys[2 * i] = ckey((uint32_t)u, (uint32_t)v);
            keys[2 * i + 1] = u == v ? ~0ull : ckey((uint32_t)v, (uint32_t)u);
        } else {
            keys[i] = ckey((uint32_t)u, (uint32_t)v);
        }
    }
}

extern "C" int axbc_graph_from_edges(const uint64_t *edges, uint64_t nedges, uint64_t n, int undirected,
                                     int H, axbc_graph **g)
{
    CHECK_ARG(g && (edges || nedges == 0), "axbc_graph_from_edges: null argument");
    CHECK_ARG(n > 0 && n < 0xffffffffull, "axbc_graph_from_edges: n must be in [1, 2^32-1)");
    CHECK_ARG(H == 0 || H == 1, "axbc_graph_from_edges: H must be 0 or 1");
    CHECK_ARG(!(H == 1 && !undirected),
              "axbc_graph_from_edges: the one-degree reduction runs on undirected graphs here "
              "(axbc_edges_to_csc takes directed ones)");
    const uint64_t nk = undirected ? 2 * nedges : nedges;
    if (nk == 0) return graph_from_host(std::vector<uint32_t>(n + 1, 0).data(), nullptr, n, 0, nullptr, 1, g);
    DBuf bad, dedges, keys;
    TRY(bad.alloc(sizeof(int)));
    TRY(dedges.alloc(nedges * 16));
    TRY(keys.alloc(nk * 8));
    CU(cudaMemset(bad.p, 0, sizeof(int)));
    CU(cudaMemcpy(dedges.p, edges, nedges * 16, cudaMemcpyHostToDevice));
    k_list_to_keys<<<2048, 256>>>(dedges.as<uint64_t>(), nedges, n, undirected, keys.as<uint64_t>(),
                                  bad.as<int>());
    CU_LAUNCH("k_list_to_keys");
    int hbad = 0;
    CU(cudaMemcpy(&hbad, bad.p, sizeof(int), cudaMemcpyDeviceToHost));
    if (hbad) {
        axbc_set_error("axbc_graph_from_edges: an edge has a vertex >= n");
        return AXBC_ERR_INVALID;
    }
    dedges.release();
    return axbc_keys_to_graph(keys.as<uint64_t>(), nk, n, undirected, H, g);
}

extern "C" int axbc_graph_generate_rmat(int scale, int edgefactor, uint64_t seed, int directed,
                                        int H, axbc_graph **g)
{
    CHECK_ARG(g, "axbc_graph_generate_rmat: null output");
    CHECK_ARG(scale >= 1 && scale <= 30, "axbc_graph_generate_rmat: scale must be in [1,30]");
    CHECK_ARG(edgefactor >= 1 && edgefactor <= 1024, "axbc_graph_generate_rmat: bad edgefactor");
    CHECK_ARG(H == 0 || H == 1, "axbc_graph_generate_rmat: H must be 0 or 1");
    const uint64_t n = 1ull << scale;
    const uint64_t ne = n * (uint64_t)edgefactor;
    DBuf keys;
    TRY(keys.alloc(2 * ne * 8));
    k_rmat<<<4096, 256>>>(ne, scale, seed, directed, keys.as<uint64_t>(), nullptr);
    CU_LAUNCH("k_rmat");
    return axbc_keys_to_graph(keys.as<uint64_t>(), 2 * ne, n, !directed, H, g);
}

extern "C" int axbc_graph_generate_grid(uint32_t side, double drop_prob, double longrange_frac,
                                        uint64_t seed, axbc_graph **g)
{
    CHECK_ARG(g, "axbc_graph_generate_grid: null output");
    CHECK_ARG(side >= 2 && side <= 32768, "axbc_graph_generate_grid: side must be in [2,32768]");
    CHECK_ARG(drop_prob >= 0 && drop_prob < 1, "axbc_graph_generate_grid: bad drop probability");
    const uint64_t n = (uint64_t)side * side;
    const uint64_t nh = (uint64_t)(side - 1) * side, nv = nh, ntot = nh + nv;
    DBuf keys, dkept;
    TRY(dkept.alloc(8));
    CU(cudaMemset(dkept.p, 0, 8));
    // room for the long-range edges: at most longrange_frac * ntot of them
    const uint64_t lr_cap = (uint64_t)(longrange_frac * (double)ntot) + 1;
    TRY(keys.alloc((2 * ntot + 2 * lr_cap) * 8));
    const uint32_t thr = (uint32_t)(drop_prob * 4294967296.0);
    k_grid<<<2048, 256>>>(side, nh, ntot, thr, seed, keys.as<uint64_t>(), dkept.as<unsigned long long>());
    CU_LAUNCH("k_grid");
    unsigned long long kept = 0;
    CU(cudaMemcpy(&kept, dkept.p, 8, cudaMemcpyDeviceToHost));
    uint64_t lr = (uint64_t)(longrange_frac * (double)kept);
    if (lr > lr_cap) lr = lr_cap;
    if (lr) k_longrange<<<256, 256>>>(lr, n, seed, keys.as<uint64_t>() + 2 * ntot);
    CU_LAUNCH("k_longrange");
    return axbc_keys_to_graph(keys.as<uint64_t>(), 2 * ntot + 2 * lr, n, 1, 0, g);
}

// ------------------------------------------------- static distributions

// (uint32)deg^2, the low 32 bits of the square (src/axbc2d.c:2681-2685)
__global__ void k_deg2(const uint32_t *__restrict__ col, uint32_t *__restrict__ out, uint64_t n)
{
    for (uint64_t v = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; v < n;
         v += (uint64_t)gridDim.x * blockDim.x) {
        uint64_t d = col[v + 1] - col[v];
        out[v] = (uint32_t)(d * d);
    }
}

// neighbour-degree sums, uint32 (sum_deg_neigh_func, src/axbc2d.c:1758-1845)
__global__ void k_sdn(const uint32_t *__restrict__ col, const uint32_t *__restrict__ row,
                      uint32_t *__restrict__ out, uint64_t n)
{
    const unsigned lane = lane_id();
    const uint64_t nw = (uint64_t)gridDim.x * blockDim.x / 32;
    for (uint64_t v = (blockIdx.x * (uint64_t)blockDim.x + threadIdx.x) / 32; v < n; v += nw) {
        uint32_t s = 0;
        for (uint32_t e = col[v] + lane; e < col[v + 1]; e += 32) {
            uint32_t w = row[e];
            s += col[w + 1] - col[w];
        }
        s = __reduce_add_sync(FULL_MASK, s);
        if (lane == 0) out[v] = s;
    }
}

// ends of the non-decreasing runs of a wrapping uint32 prefix
__global__ void k_wraps(const uint32_t *__restrict__ p, uint64_t n, uint32_t *__restrict__ ends,
                        uint32_t *__restrict__ count, uint32_t cap)
{
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i + 1 < n;
         i += (uint64_t)gridDim.x * blockDim.x) {
        if (p[i + 1] < p[i]) {
            uint32_t k = atomicAdd(count, 1u);
            if (k < cap) ends[k] = (uint32_t)(i + 1);
        }
    }
}

int axbc_build_deg_dist(axbc_graph *g, cudaStream_t s)
{
    if (g->have_deg_dist) return AXBC_OK;
    const uint64_t n = g->n;
    DBuf d2, tmp, ends, cnt;
    TRY(d2.alloc(n * 4));
    ALLOC_MISSING(g->deg2p, n * 4, &g->bytes);
    ALLOC_MISSING(g->sdn, n * 4, &g->bytes);
    k_deg2<<<1024, 256, 0, s>>>(g->fwd.col, d2.as<uint32_t>(), n);
    k_sdn<<<2048, 256, 0, s>>>(g->fwd.col, g->fwd.row, g->sdn, n);
    CU_LAUNCH("deg2/sdn");
    size_t tb = 0;
    cub::DeviceScan::InclusiveSum(nullptr, tb, d2.as<uint32_t>(), g->deg2p, (int64_t)n, s);
    TRY(tmp.alloc(tb));
    cub::DeviceScan::InclusiveSum(tmp.p, tb, d2.as<uint32_t>(), g->deg2p, (int64_t)n, s);
    CU_LAUNCH("deg2 scan");
    // run ends: the prefix wraps at most (total / 2^32) + 1 times
    const uint32_t cap = 1u << 20;
    TRY(ends.alloc(cap * 4));
    TRY(cnt.alloc(4));
    CU(cudaMemsetAsync(cnt.p, 0, 4, s));
    k_wraps<<<1024, 256, 0, s>>>(g->deg2p, n, ends.as<uint32_t>(), cnt.as<uint32_t>(), cap);
    CU_LAUNCH("k_wraps");
    uint32_t nw = 0;
    CU(cudaMemcpyAsync(&nw, cnt.p, 4, cudaMemcpyDeviceToHost, s));
    CU(cudaStreamSynchronize(s));
    if (nw > cap) {
        axbc_set_error("degree^2 prefix wraps too often");
        return AXBC_ERR_RANGE;
    }
    std::vector<uint32_t> h(nw);
    if (nw) CU(cudaMemcpy(h.data(), ends.p, nw * 4, cudaMemcpyDeviceToHost));
    std::sort(h.begin(), h.end());
    h.push_back((uint32_t)n);
    axbc_dfree(g->seg_end);  // an earlier, failed call may have left one
    g->seg_end = nullptr;
    TRY(axbc_dalloc((void **)&g->seg_end, h.size() * 4, &g->bytes));
    g->n_seg = (uint32_t)h.size();
    CU(cudaMemcpy(g->seg_end, h.data(), h.size() * 4, cudaMemcpyHostToDevice));
    CU(cudaMemcpy(&g->sum_deg, g->deg2p + n - 1, 4, cudaMemcpyDeviceToHost));
    g->have_deg_dist = true;
    return AXBC_OK;
}

// |adj(w) ∩ adj(i)| without i, by binary search of the shorter list's entries
// in the longer one (adjacency lists are sorted and duplicate-free)
__device__ __forceinline__ uint32_t isect_count(const uint32_t *a, uint32_t da, const uint32_t *b,
                                                uint32_t db, uint32_t skip)
{
    if (da > db) {
        const uint32_t *t = a;
        a = b;
        b = t;
        uint32_t td = da;
        da = db;
        db = td;
    }
    uint32_t c = 0;
    for (uint32_t k = 0; k < da; k++) {
        uint32_t x = a[k];
        if (x == skip) continue;
        uint32_t lo = 0, hi = db;
        while (lo < hi) {
            uint32_t mid = (lo + hi) >> 1;
            if (b[mid] < x) lo = mid + 1;
            else hi = mid;
        }
        c += (lo < db && b[lo] == x);
    }
    return c;
}

// lcc_func (src/axbc2d.c:1847-1935): counter(i) = sum over neighbours w of
// |adj(w) \ {i} ∩ adj(i)|, uint32.  Lanes take neighbours; vertices with more
// than SPAN neighbours are split over their span items.
__global__ void k_lcc_count(Adj a, uint32_t *__restrict__ counter)
{
    const unsigned lane = lane_id();
    const uint64_t ntask = a.n + a.n_heavy_items;
    const uint64_t nw = (uint64_t)gridDim.x * blockDim.x / 32;
    for (uint64_t t = (blockIdx.x * (uint64_t)blockDim.x + threadIdx.x) / 32; t < ntask; t += nw) {
        uint32_t i, b0, b1;
        if (t < a.n) {
            i = (uint32_t)t;
            uint32_t d = a.col[i + 1] - a.col[i];
            if (d < 2 || d > AXBC_SPAN) continue;
            b0 = a.col[i];
            b1 = a.col[i + 1];
        } else {
            i = a.hitem_v[t - a.n];
            uint32_t k = a.hitem_k[t - a.n];
            b0 = a.col[i] + k * AXBC_SPAN;
            b1 = min(a.col[i + 1], b0 + AXBC_SPAN);
        }
        const uint32_t *ai = a.row + a.col[i];
        const uint32_t di = a.col[i + 1] - a.col[i];
        uint32_t c = 0;
        for (uint32_t e = b0 + lane; e < b1; e += 32) {
            uint32_t w = a.row[e];
            c += isect_count(a.row + a.col[w], a.col[w + 1] - a.col[w], ai, di, i);
        }
        c = __reduce_add_sync(FULL_MASK, c);
        if (lane == 0 && c) atomicAdd(&counter[i], c);
    }
}

__global__ void k_lcc_final(const uint32_t *__restrict__ col, const uint32_t *__restrict__ counter,
                            float *__restrict__ out, uint64_t n)
{
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n;
         i += (uint64_t)gridDim.x * blockDim.x) {
        uint32_t d = col[i + 1] - col[i];
        out[i] = (d < 2) ? 0.0f
                         : __fdiv_rn(__uint2float_rn(counter[i]), __uint2float_rn(d * (d - 1u)));
    }
}

int axbc_build_lcc(axbc_graph *g, cudaStream_t s)
{
    if (g->have_lcc) return AXBC_OK;
    const uint64_t n = g->n;
    DBuf cnt;
    TRY(cnt.alloc(n * 4));
    ALLOC_MISSING(g->lcc, n * 4, &g->bytes);
    ALLOC_MISSING(g->lcc_local, n * 8, &g->bytes);
    ALLOC_MISSING(g->lcc_csum, ((n + AXBC_SAMPLE_BLOCK - 1) / AXBC_SAMPLE_BLOCK) * 8, &g->bytes);
    CU(cudaMemsetAsync(cnt.p, 0, n * 4, s));
    k_lcc_count<<<4096, 256, 0, s>>>(g->fwd, cnt.as<uint32_t>());
    k_lcc_final<<<1024, 256, 0, s>>>(g->fwd.col, cnt.as<uint32_t>(), g->lcc, n);
    CU_LAUNCH("lcc");
    TRY(axbc_hprefix_launch(g->lcc, n, g->lcc_local, g->lcc_csum, s));
    const uint64_t nb = (n + AXBC_SAMPLE_BLOCK - 1) / AXBC_SAMPLE_BLOCK;
    CU(cudaMemcpyAsync(&g->S_lcc, g->lcc_csum + nb - 1, 8, cudaMemcpyDeviceToHost, s));
    CU(cudaStreamSynchronize(s));
    g->have_lcc = true;
    return AXBC_OK;
}

extern "C" int axbc_graph_degree2(axbc_graph *g, uint32_t *out_host)
{
    CHECK_ARG(g && out_host, "axbc_graph_degree2: null argument");
    uint32_t *d = nullptr;
    TRY(axbc_dalloc((void **)&d, g->n * 4, nullptr));
    k_deg2<<<1024, 256>>>(g->fwd.col, d, g->n);
    CU_LAUNCH("k_deg2");
    cudaError_t e = cudaMemcpy(out_host, d, g->n * 4, cudaMemcpyDeviceToHost);
    axbc_dfree(d);
    if (e != cudaSuccess) return axbc_cuda_fail(e, "degree2", __FILE__, __LINE__);
    return AXBC_OK;
}

extern "C" int axbc_graph_sum_deg_neigh(axbc_graph *g, uint32_t *out_host)
{
    CHECK_ARG(g && out_host, "axbc_graph_sum_deg_neigh: null argument");
    TRY(axbc_build_deg_dist(g, 0));
    CU(cudaMemcpy(out_host, g->sdn, g->n * 4, cudaMemcpyDeviceToHost));
    return AXBC_OK;
}

extern "C" int axbc_graph_lcc(axbc_graph *g, float *out_host)
{
    CHECK_ARG(g && out_host, "axbc_graph_lcc: null argument");
    TRY(axbc_build_lcc(g, 0));
    CU(cudaMemcpy(out_host, g->lcc, g->n * 4, cudaMemcpyDeviceToHost));
    return AXBC_OK;
}
