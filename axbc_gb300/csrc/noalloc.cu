// One Brandes pass (the plain form of axbc_run_pivot) that allocates nothing.
//
// For callers that cannot allocate device memory themselves or through the
// library: a host application whose device memory is owned by another
// allocator or budget (a framework that reserved the GPU's memory up front),
// a real-time loop that must not call cudaMalloc/cudaFree because they can
// synchronise the device, or a plug-in that may only use the buffers its host
// hands it.  The caller passes the graph and the bc output as device
// pointers; every scratch array of the pass lives in one file-scope
// __device__ array of fixed size, which each GPU that loads the library holds
// until the process exits.
//
// Limits: at most AXBC_STATIC_MAX_N vertices and AXBC_STATIC_MAX_ITEMS span
// items of vertices with more than 1024 neighbours; larger graphs are rejected
// with AXBC_ERR_RANGE before anything runs.  The forward levels always push
// from the frontier, so no transpose is needed and directed graphs work.
//
// The first call on a device looks up the array's device address with
// cudaGetSymbolAddress (once per device, with that device current, and again
// only if the device's context changed, e.g. after cudaDeviceReset); make that
// first call before any stream capture.  All calls share the array and it
// keeps the last call's contents: every call clears what must start at zero.
// Calls that overlap on the GPU (two host threads, or two streams) race on the
// array: serialise them.
#include <cuda.h>

#include <mutex>

#include "common.cuh"

#define AXBC_STATIC_MAX_N (1u << 18)
#define AXBC_STATIC_MAX_ITEMS (1u << 14)
#define AXBC_STATIC_MAX_DEVICES 64

namespace {
// scratch layout, in 4-byte words
constexpr size_t W_LVL = 0;
constexpr size_t W_SIGMA = W_LVL + AXBC_STATIC_MAX_N;
constexpr size_t W_DELTA = W_SIGMA + AXBC_STATIC_MAX_N;
constexpr size_t W_QUEUE = W_DELTA + AXBC_STATIC_MAX_N;
constexpr size_t W_ZERO = W_QUEUE + AXBC_STATIC_MAX_N + 1;
constexpr size_t W_PART = W_ZERO + AXBC_STATIC_MAX_N;
constexpr size_t W_HV = W_PART + AXBC_STATIC_MAX_ITEMS;
constexpr size_t W_HFIRST = W_HV + AXBC_STATIC_MAX_ITEMS;
constexpr size_t W_IV = W_HFIRST + AXBC_STATIC_MAX_ITEMS + 1;
constexpr size_t W_IK = W_IV + AXBC_STATIC_MAX_ITEMS;
constexpr size_t W_CNT = W_IK + AXBC_STATIC_MAX_ITEMS;  // 2 words: heavy vertices, items
constexpr size_t W_PC = (W_CNT + 2 + 63) & ~size_t(63);  // PivotCounters, 256-byte aligned
constexpr size_t W_TOTAL = W_PC + 64;
}  // namespace

static __device__ __align__(256) uint32_t g_static_scratch[W_TOTAL];

// the plain-form kernels (single.cu), launched here unchanged
__global__ void k_reset1(int32_t *lvl, uint32_t *sigma, float *delta, const uint32_t *reach, uint64_t n);
__global__ void k_set_root1(uint32_t v0, int level, uint32_t sig, int32_t *lvl, uint32_t *sigma,
                            uint32_t *queue, PivotCounters *pc, const uint32_t *col,
                            const uint32_t *rcol);
__global__ void k_fwd_push1(Adj a, const uint32_t *rcol, uint32_t qs, uint32_t nf, int32_t *lvl,
                            uint32_t *sigma, uint32_t *queue, PivotCounters *pc, int L);
__global__ void k_bwd1(Adj a, const uint32_t *queue, uint32_t ls, uint32_t nseg, const int32_t *lvl,
                       const uint32_t *sigma, float *delta, const uint32_t *reach, float *partial,
                       int d);
__global__ void k_bwd_combine1(Adj a, const int32_t *lvl, float *delta, const uint32_t *reach,
                               const float *partial, int d);
__global__ void k_reach_sum1(const int32_t *lvl, const uint32_t *reach, uint64_t n, PivotCounters *pc);
__global__ void k_update1(float *bc, const float *delta, uint64_t n, uint32_t v0, double p,
                          const uint32_t *reach_v0_ptr, unsigned long long nvt_base,
                          const PivotCounters *pc, int add_all, int add_sum);

// Span items of the vertices with more than one span of neighbours, in vertex
// order, written into the scratch (one block; counts beyond the limits are
// reported, not written).
__global__ void k_static_heavy(const uint32_t *__restrict__ col, uint32_t n, uint32_t *heavy_v,
                               uint32_t *heavy_first, uint32_t *item_v, uint32_t *item_k,
                               uint32_t *counts)
{
    __shared__ uint32_t sh[1024], ss[1024];
    const uint32_t t = threadIdx.x, nt = blockDim.x;
    const uint32_t per = (n + nt - 1) / nt;
    const uint32_t lo = min(n, t * per), hi = min(n, lo + per);
    uint32_t h = 0, sp = 0;
    for (uint32_t v = lo; v < hi; v++) {
        const uint32_t d = col[v + 1] - col[v];
        if (d > AXBC_SPAN) {
            h++;
            sp += (d + AXBC_SPAN - 1) / AXBC_SPAN;
        }
    }
    sh[t] = h;
    ss[t] = sp;
    __syncthreads();
    if (t == 0) {  // exclusive scan of the per-thread counts
        uint32_t a = 0, b = 0;
        for (uint32_t i = 0; i < nt; i++) {
            const uint32_t x = sh[i], y = ss[i];
            sh[i] = a;
            ss[i] = b;
            a += x;
            b += y;
        }
        counts[0] = a;
        counts[1] = b;
        if (a <= AXBC_STATIC_MAX_ITEMS && b <= AXBC_STATIC_MAX_ITEMS) heavy_first[a] = b;
    }
    __syncthreads();
    uint32_t hi_idx = sh[t], it = ss[t];
    for (uint32_t v = lo; v < hi; v++) {
        const uint32_t d = col[v + 1] - col[v];
        if (d <= AXBC_SPAN) continue;
        const uint32_t spans = (d + AXBC_SPAN - 1) / AXBC_SPAN;
        if (hi_idx < AXBC_STATIC_MAX_ITEMS && it + spans <= AXBC_STATIC_MAX_ITEMS) {
            heavy_v[hi_idx] = v;
            heavy_first[hi_idx] = it;
            for (uint32_t k = 0; k < spans; k++) {
                item_v[it + k] = v;
                item_k[it + k] = k;
            }
        }
        hi_idx++;
        it += spans;
    }
}

static std::mutex g_static_mu;
static uint32_t *g_static_addr[AXBC_STATIC_MAX_DEVICES];
// the context each cached address belongs to (driver context id, never
// reused): after cudaDeviceReset, or when the caller makes another context
// current, the array lives at another address and is looked up again
static unsigned long long g_static_ctx[AXBC_STATIC_MAX_DEVICES];
static uint64_t g_static_levstart[AXBC_STATIC_MAX_N + 2];

// id of the context current on this thread (0: none yet), through the
// driver's entry points as the runtime hands them out (no link to libcuda)
static int current_ctx_id(unsigned long long *id)
{
    typedef CUresult (*get_current_t)(CUcontext *);
    typedef CUresult (*get_id_t)(CUcontext, unsigned long long *);
    static get_current_t get_current = nullptr;
    static get_id_t get_id = nullptr;
    if (!get_current || !get_id) {
        cudaDriverEntryPointQueryResult q1, q2;
        void *f1 = nullptr, *f2 = nullptr;
        CU(cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &f1, 12000, cudaEnableDefault, &q1));
        CU(cudaGetDriverEntryPointByVersion("cuCtxGetId", &f2, 12000, cudaEnableDefault, &q2));
        if (q1 != cudaDriverEntryPointSuccess || q2 != cudaDriverEntryPointSuccess || !f1 || !f2) {
            axbc_set_error("axbc_bc_pivot_static: the driver offers no cuCtxGetCurrent/cuCtxGetId");
            return AXBC_ERR_CUDA;
        }
        get_current = (get_current_t)f1;
        get_id = (get_id_t)f2;
    }
    CUcontext ctx = nullptr;
    *id = 0;
    if (get_current(&ctx) != CUDA_SUCCESS || !ctx) return AXBC_OK;
    if (get_id(ctx, id) != CUDA_SUCCESS) {
        axbc_set_error("axbc_bc_pivot_static: cuCtxGetId failed");
        return AXBC_ERR_CUDA;
    }
    return AXBC_OK;
}

static int static_scratch(uint32_t **out)
{
    int dev = 0;
    CU(cudaGetDevice(&dev));
    if (dev < 0 || dev >= AXBC_STATIC_MAX_DEVICES) {
        axbc_set_error("device ordinal %d beyond %d", dev, AXBC_STATIC_MAX_DEVICES);
        return AXBC_ERR_RANGE;
    }
    unsigned long long ctx = 0;
    TRY(current_ctx_id(&ctx));
    if (!g_static_addr[dev] || ctx == 0 || ctx != g_static_ctx[dev]) {
        void *p = nullptr;
        // the array's name is a host-side stand-in; the kernels need its
        // device address, looked up once per device (and context) with the
        // device current
        CU(cudaGetSymbolAddress(&p, g_static_scratch));
        g_static_addr[dev] = (uint32_t *)p;
        if (ctx == 0) TRY(current_ctx_id(&ctx));  // the lookup made the context current
        g_static_ctx[dev] = ctx;
    }
    *out = g_static_addr[dev];
    return AXBC_OK;
}

extern "C" int axbc_bc_pivot_static(const uint32_t *col, const uint32_t *row, const uint32_t *reach,
                                    uint64_t n, uint64_t m, uint32_t v0, double p, int H,
                                    float *bc, void *stream, axbc_pivot_stats *stats)
{
    CHECK_ARG(col && (row || m == 0) && bc, "axbc_bc_pivot_static: null device pointer");
    CHECK_ARG(H == 0 || H == 1, "axbc_bc_pivot_static: H must be 0 or 1");
    if (n == 0 || n > AXBC_STATIC_MAX_N) {
        axbc_set_error("axbc_bc_pivot_static: n = %llu; this entry point holds at most %u vertices",
                       (unsigned long long)n, AXBC_STATIC_MAX_N);
        return AXBC_ERR_RANGE;
    }
    CHECK_ARG(m < 0xffffffffull, "axbc_bc_pivot_static: m must be < 2^32");
    CHECK_ARG(v0 < n, "axbc_bc_pivot_static: v0 >= n");
    std::lock_guard<std::mutex> lock(g_static_mu);
    uint32_t *S = nullptr;
    TRY(static_scratch(&S));
    cudaStream_t s = (cudaStream_t)stream;
    int32_t *lvl = (int32_t *)(S + W_LVL);
    uint32_t *sigma = S + W_SIGMA, *queue = S + W_QUEUE, *cnt = S + W_CNT;
    float *delta = (float *)(S + W_DELTA), *partial = (float *)(S + W_PART);
    PivotCounters *pc = (PivotCounters *)(S + W_PC);
    if (!reach) {
        CU(cudaMemsetAsync(S + W_ZERO, 0, n * 4, s));
        reach = S + W_ZERO;
    }

    // heavy-vertex span items for this graph
    Adj a;
    a.n = n;
    a.m = m;
    a.col = (uint32_t *)col;
    a.row = (uint32_t *)row;
    a.heavy_v = S + W_HV;
    a.heavy_first = S + W_HFIRST;
    a.hitem_v = S + W_IV;
    a.hitem_k = S + W_IK;
    a.owns = false;
    k_static_heavy<<<1, 1024, 0, s>>>(col, (uint32_t)n, a.heavy_v, a.heavy_first, a.hitem_v,
                                      a.hitem_k, cnt);
    CU_LAUNCH("k_static_heavy");
    uint32_t counts[2] = {0, 0};
    CU(cudaMemcpyAsync(counts, cnt, 8, cudaMemcpyDeviceToHost, s));
    CU(cudaStreamSynchronize(s));
    if (counts[0] > AXBC_STATIC_MAX_ITEMS || counts[1] > AXBC_STATIC_MAX_ITEMS) {
        axbc_set_error("axbc_bc_pivot_static: %u span items of high-degree vertices; the limit "
                       "is %u", counts[1], AXBC_STATIC_MAX_ITEMS);
        return AXBC_ERR_RANGE;
    }
    a.n_heavy = counts[0];
    a.n_heavy_items = counts[1];

    int sms = 0, dev = 0;
    CU(cudaGetDevice(&dev));
    CU(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    const int grid = 8 * (sms > 0 ? sms : 152);
    k_reset1<<<grid, 256, 0, s>>>(lvl, sigma, delta, reach, n);
    k_set_root1<<<1, 1, 0, s>>>(v0, 0, 1, lvl, sigma, queue, pc, col, col);
    CU_LAUNCH("reset/root");

    uint64_t *ls = g_static_levstart;
    ls[0] = 0;
    ls[1] = 1;
    uint64_t nvisited = 1;
    int level = 0;
    PivotCounters hc;
    for (;;) {
        level++;
        const uint32_t qs = (uint32_t)ls[level - 1], nf = (uint32_t)(ls[level] - ls[level - 1]);
        const uint32_t tail = qs + nf;
        CU(cudaMemcpyAsync(&pc->qtail, &tail, 4, cudaMemcpyHostToDevice, s));
        k_fwd_push1<<<grid, 256, 0, s>>>(a, col, qs, nf, lvl, sigma, queue, pc, level);
        CU_LAUNCH("forward level");
        CU(cudaMemcpyAsync(&hc, pc, sizeof hc, cudaMemcpyDeviceToHost, s));
        CU(cudaStreamSynchronize(s));
        const uint64_t nfrt = hc.qtail - tail;
        ls[level + 1] = ls[level] + nfrt;
        if (!nfrt) break;
        nvisited += nfrt;
    }
    int depth = level - 2;
    if (depth >= 0) {
        do {
            const uint32_t l0 = (uint32_t)ls[depth], nseg = (uint32_t)(ls[depth + 1] - ls[depth]);
            k_bwd1<<<grid, 256, 0, s>>>(a, queue, l0, nseg, lvl, sigma, delta, reach, partial, depth);
            if (a.n_heavy)
                k_bwd_combine1<<<(a.n_heavy + 255) / 256, 256, 0, s>>>(a, lvl, delta, reach, partial,
                                                                       depth);
            CU_LAUNCH("backward level");
            depth--;
        } while (depth > 0);
    }
    CU(cudaMemsetAsync(&pc->reach_sum, 0, 8, s));
    if (H == 1) k_reach_sum1<<<grid, 256, 0, s>>>(lvl, reach, n, pc);
    k_update1<<<grid, 256, 0, s>>>(bc, delta, n, v0, p, reach + v0, nvisited, pc, 1, H == 1);
    CU_LAUNCH("update");
    if (stats) {
        uint32_t reach_v0 = 0;
        CU(cudaMemcpyAsync(&hc, pc, sizeof hc, cudaMemcpyDeviceToHost, s));
        CU(cudaMemcpyAsync(&reach_v0, reach + v0, 4, cudaMemcpyDeviceToHost, s));
        CU(cudaStreamSynchronize(s));
        stats->nvisited = nvisited;
        stats->all = (H == 1 ? (uint32_t)hc.reach_sum : 0u) + reach_v0;
        stats->te = 2 * hc.newdeg;
        stats->levels = level;
        stats->pad = 0;
    } else {
        CU(cudaStreamSynchronize(s));
    }
    return AXBC_OK;
}
