// The reference's host/CUDA boundary (src/bc2d.h:136-190) implemented on top
// of the plain-form kernels: same names, signatures and call protocol, one
// implicit graph per process, print-and-exit on failure.
#include <cstdio>
#include <cstdlib>
#include <cstring>

#include "../../include/axbc_compat.h"
#include "common.cuh"

// The host program's vertex count (src/axbc2d.c:29), when it defines one.
extern "C" __attribute__((weak)) uint64_t N;

namespace {
uint64_t g_n_override = 0;
axbc_graph *g_graph = nullptr;
axbc_ctx *g_ctx = nullptr;
uint32_t g_frt = 0;  // queue offset of the current frontier
uint32_t *g_reach_v0 = nullptr;  // device scalar set by setcuda
uint32_t g_last_all = 0;

uint64_t compat_n()
{
    if (g_n_override) return g_n_override;
    if (&N != nullptr) return N;
    return 0;
}

[[noreturn]] void die(const char *what)
{
    fprintf(stderr, "axbc_gb300 error in %s: %s\n", what, axbc_last_error());
    exit(EXIT_FAILURE);
}

void need(int rc, const char *what)
{
    if (rc != AXBC_OK) die(what);
}

void need_ctx(const char *what)
{
    if (!g_ctx) {
        axbc_set_error("initcuda has not been called");
        die(what);
    }
}

void cu(cudaError_t e, const char *what)
{
    if (e != cudaSuccess) {
        axbc_set_error("%s", cudaGetErrorString(e));
        die(what);
    }
}
}  // namespace

extern "C" void axbc_compat_set_n(uint64_t n) { g_n_override = n; }

extern "C" size_t initcuda(uint64_t ned, uint32_t *col, uint32_t *row)
{
    const uint64_t n = compat_n();
    if (n == 0) {
        axbc_set_error("vertex count unknown: define uint64_t N or call axbc_compat_set_n");
        die("initcuda");
    }
    if (g_ctx) fincuda();
    need(axbc_graph_create(col, row, n, ned, nullptr, &g_graph), "initcuda");
    need(axbc_ctx_create(g_graph, nullptr, &g_ctx), "initcuda");
    need(axbc_ensure_single(g_ctx), "initcuda");
    need(axbc_dalloc((void **)&g_reach_v0, 4, &g_ctx->bytes), "initcuda");
    cu(cudaMemset(g_reach_v0, 0, 4), "initcuda");
    return (size_t)(g_graph->bytes + g_ctx->bytes);
}

extern "C" void fincuda(void)
{
    axbc_dfree(g_reach_v0);
    g_reach_v0 = nullptr;
    axbc_ctx_destroy(g_ctx);
    axbc_graph_destroy(g_graph);
    g_ctx = nullptr;
    g_graph = nullptr;
}

extern "C" void init_bc_1degree_device(uint32_t *reach)
{
    need_ctx("init_bc_1degree_device");
    cu(cudaMemcpy(g_graph->reach, reach, g_graph->n * 4, cudaMemcpyHostToDevice),
       "init_bc_1degree_device");
}

extern "C" void setcuda(uint64_t ned, uint32_t *col, uint32_t *row, uint32_t reach_v0)
{
    (void)ned;
    (void)col;
    (void)row;
    need_ctx("setcuda");
    need(axbc_single_reset(g_ctx), "setcuda");
    cu(cudaMemcpyAsync(g_reach_v0, &reach_v0, 4, cudaMemcpyHostToDevice, g_ctx->stream), "setcuda");
    cu(cudaStreamSynchronize(g_ctx->stream), "setcuda");
    g_frt = 0;
}

extern "C" void set_mlp_cuda(uint32_t row, int level, int sigma)
{
    need_ctx("set_mlp_cuda");
    if (row >= g_graph->n) {
        axbc_set_error("vertex %u >= N", row);
        die("set_mlp_cuda");
    }
    need(axbc_single_set_root(g_ctx, row, level, (uint32_t)sigma), "set_mlp_cuda");
    g_frt = 0;
}

extern "C" uint32_t scan_col_csc_cuda_mono(int ncol, int level)
{
    need_ctx("scan_col_csc_cuda_mono");
    uint64_t nfrt = 0;
    need(axbc_single_forward_level(g_ctx, g_frt, (uint32_t)ncol, level, &nfrt),
         "scan_col_csc_cuda_mono");
    g_frt += (uint32_t)ncol;
    return (uint32_t)nfrt;
}

extern "C" uint32_t scan_frt_csc_cuda_mono(int offset, int ncol, int depth)
{
    need_ctx("scan_frt_csc_cuda_mono");
    if (ncol > 0)
        need(axbc_single_backward_level(g_ctx, (uint32_t)offset, (uint32_t)ncol, depth),
             "scan_frt_csc_cuda_mono");
    cu(cudaStreamSynchronize(g_ctx->stream), "scan_frt_csc_cuda_mono");
    return (uint32_t)ncol;
}

extern "C" void pre_update_bc_cuda(uint32_t *reach, uint32_t v0, uint32_t *all)
{
    (void)reach;
    (void)v0;
    need_ctx("pre_update_bc_cuda");
    need(axbc_single_reach_sum(g_ctx), "pre_update_bc_cuda");
    unsigned long long s = 0;
    cu(cudaMemcpyAsync(&s, &g_ctx->pc->reach_sum, 8, cudaMemcpyDeviceToHost, g_ctx->stream),
       "pre_update_bc_cuda");
    cu(cudaStreamSynchronize(g_ctx->stream), "pre_update_bc_cuda");
    g_last_all = (uint32_t)s;
    *all = (uint32_t)s;
}

extern "C" void update_bc_cuda(uint32_t v0, double p, int ncol, const uint64_t nvisited)
{
    (void)ncol;
    need_ctx("update_bc_cuda");
    need(axbc_single_update(g_ctx, v0, p, g_reach_v0, nvisited, 0, 0), "update_bc_cuda");
    cu(cudaStreamSynchronize(g_ctx->stream), "update_bc_cuda");
}

extern "C" void get_bc(float *bc)
{
    need_ctx("get_bc");
    need(axbc_get_bc(g_ctx, bc), "get_bc");
}

extern "C" void get_delta(float *delta)
{
    need_ctx("get_delta");
    need(axbc_get_delta(g_ctx, delta), "get_delta");
}

extern "C" void get_deg(uint32_t *deg)
{
    need_ctx("get_deg");
    need(axbc_graph_get_deg(g_graph, deg), "get_deg");
}

extern "C" void get_sigma(uint32_t *sigma)
{
    need_ctx("get_sigma");
    need(axbc_get_sigma(g_ctx, sigma), "get_sigma");
}

extern "C" void get_lvl(int *lvl)
{
    need_ctx("get_lvl");
    need(axbc_get_levels(g_ctx, lvl), "get_lvl");
}

extern "C" void get_frt(uint32_t *frt)
{
    need_ctx("get_frt");
    cu(cudaMemcpy(frt, g_ctx->queue, g_graph->n * 4, cudaMemcpyDeviceToHost), "get_frt");
}

// visited bitmask, one bit per vertex (MSKGET, src/bc2d.h:102-104)
__global__ void k_msk(const int32_t *__restrict__ lvl, uint64_t n, uint32_t *msk)
{
    const uint64_t words = (n + 31) / 32;
    for (uint64_t w = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; w < words;
         w += (uint64_t)gridDim.x * blockDim.x) {
        uint32_t m = 0;
        for (int b = 0; b < 32; b++) {
            const uint64_t v = w * 32 + b;
            if (v < n && lvl[v] >= 0) m |= 1u << b;
        }
        msk[w] = m;
    }
}

extern "C" void get_msk(uint32_t *msk)
{
    need_ctx("get_msk");
    const uint64_t words = (g_graph->n + 31) / 32;
    uint32_t *d = nullptr;
    need(axbc_dalloc((void **)&d, words * 4, nullptr), "get_msk");
    k_msk<<<256, 256, 0, g_ctx->stream>>>(g_ctx->lvl, g_graph->n, d);
    cu(cudaGetLastError(), "get_msk");
    cu(cudaMemcpyAsync(msk, d, words * 4, cudaMemcpyDeviceToHost, g_ctx->stream), "get_msk");
    cu(cudaStreamSynchronize(g_ctx->stream), "get_msk");
    axbc_dfree(d);
}

extern "C" void get_all(uint32_t *all)
{
    *all = g_last_all;
    g_last_all = 0;
}

extern "C" void *CudaMallocHostSet(size_t size, int val)
{
    void *p = nullptr;
    cu(cudaMallocHost(&p, size), "CudaMallocHostSet");
    memset(p, val, size);
    return p;
}

extern "C" void CudaFreeHost(void *ptr)
{
    if (ptr) cu(cudaFreeHost(ptr), "CudaFreeHost");
}
