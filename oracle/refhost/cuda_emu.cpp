/* Test infrastructure: the reference's host<->CUDA boundary (src/bc2d.h:
 * 136-190) implemented on the host, so that the reference's own driver
 * (src/axbc2d.c, compiled unchanged) runs its single-GPU path on a machine
 * without a GPU.
 *
 * - The kernels are the reference's own source text (src/cuda_kernels.cu:
 *   read_edge_count, scan_col_mono2, scan_frt_mono, update_bc, init_delta,
 *   set_degree and the bmaxlt helper), copied unedited into
 *   oracle/_ref/mono_kernels.inc by extract_kernels.py and run one thread
 *   after another by emu_launch (cuda_shim.h).
 * - The host wrappers below restate src/cuda_kernels.cu's wrappers (line
 *   numbers cited on each); cudaMemset/cudaMemcpy become memset/memcpy, the
 *   Thrust exclusive scan a loop, and the reach reduction of
 *   deviceReduceKernel (whose warp shuffles a serial run cannot execute) a
 *   loop with the same uint32 arithmetic.
 * - Arithmetic: compiled without contraction or fast-math, so the float
 *   division (delta + 1) / sigma is IEEE-rounded; the reference's own build
 *   uses --use_fast_math (an approximate division within 2 ulp).
 *
 * With AXBC_REF_DUMP=path set, the run writes a record file: the CSC, reach,
 * one record per applied pivot (root, p, nvisited, and the final levels,
 * path counts and dependencies) and the final bc (before the driver's
 * division by 2 * nrounds).  tests/golden/make_ref_golden.py turns it into
 * fixtures.  Only oracle/Makefile builds this file, into oracle/_ref. */
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "mpi.h"
#include "bc2d.h"
#include "cuda_shim.h"

emu_dim3 threadIdx, blockIdx, blockDim, gridDim;

// __device__ LOCINT d_reach_v0 (src/cuda_kernels.cu:37)
static LOCINT d_reach_v0;

#include "mono_kernels.inc"

// device arrays of src/cuda_kernels.cu:41-81 (the mono path's subset)
static LOCINT *d_msk, *d_col, *d_row, *d_deg, *d_cbuf, *d_cbuf_start, *d_sbuf, *d_frt, *d_frt_start;
static LOCINT *d_sig, *d_reach;
static uint32_t *d_snum;
static int *d_lvl;
static float *d_delta, *d_bc;
static uint64_t d_ned;

// ------------------------------------------------------------------ dump
static FILE *dump_fp;
static uint32_t dump_v0;

static void dump_rec(uint32_t tag, const void *a, size_t na, const void *b = nullptr, size_t nb = 0)
{
    if (!dump_fp) return;
    const uint64_t len = na + nb;
    fwrite(&tag, 4, 1, dump_fp);
    fwrite(&len, 8, 1, dump_fp);
    if (na) fwrite(a, 1, na, dump_fp);
    if (nb) fwrite(b, 1, nb, dump_fp);
}

enum { REC_CSC = 1, REC_REACH = 2, REC_PIVOT = 3, REC_BC = 4, REC_END = 5 };

static void *emu_alloc(size_t bytes, int val)
{
    void *p = malloc(bytes ? bytes : 1);
    if (!p) {
        fprintf(stderr, "host emulation: cannot allocate %zu bytes\n", bytes);
        exit(EXIT_FAILURE);
    }
    memset(p, val, bytes);
    return p;
}

static void not_emulated(const char *f)
{
    fprintf(stderr, "host emulation: %s belongs to the 2-D multi-GPU path, which is not emulated "
                    "(run with -p 1x1 and without -m)\n", f);
    exit(EXIT_FAILURE);
}

// CudaMallocHostSet / CudaFreeHost (src/cuda_kernels.cu:837-850)
void *CudaMallocHostSet(size_t size, int val) { return emu_alloc(size, val); }
void CudaFreeHost(void *ptr) { free(ptr); }

int assignDeviceToProcess() { return 0; }

// initcuda (src/cuda_kernels.cu:1558-1646), mono path with ONEPREFIX
size_t initcuda(uint64_t ned, LOCINT *col, LOCINT *row)
{
    const char *path = getenv("AXBC_REF_DUMP");
    if (path && !dump_fp) {
        dump_fp = fopen(path, "wb");
        if (!dump_fp) {
            fprintf(stderr, "host emulation: cannot write %s\n", path);
            exit(EXIT_FAILURE);
        }
        const uint64_t hdr[2] = {N, ned};
        const uint32_t tag = REC_CSC;
        const uint64_t len = sizeof(hdr) + (col_bl + 1) * 4 + ned * 4;
        fwrite(&tag, 4, 1, dump_fp);
        fwrite(&len, 8, 1, dump_fp);
        fwrite(hdr, sizeof(hdr), 1, dump_fp);
        fwrite(col, 4, col_bl + 1, dump_fp);
        fwrite(row, 4, ned, dump_fp);
    }
    d_ned = ned;
    d_col = (LOCINT *)emu_alloc((col_bl + 1) * sizeof(*d_col), 0);
    d_row = (LOCINT *)emu_alloc(ned * sizeof(*d_row), 0);
    memcpy(d_col, col, (col_bl + 1) * sizeof(*col));
    memcpy(d_row, row, ned * sizeof(*row));
    d_deg = (LOCINT *)emu_alloc(col_bl * sizeof(*d_deg), 0);
    emu_launch(set_degree, (col_bl + THREADS - 1) / THREADS, THREADS, d_col, d_deg, (LOCINT)col_bl);
    d_cbuf_start = (LOCINT *)emu_alloc(MAX(row_bl, row_pp) * sizeof(*d_cbuf_start), 0);
    d_sbuf = (LOCINT *)emu_alloc(MAX(row_bl, row_pp) * sizeof(*d_sbuf), 0);
    d_snum = (uint32_t *)emu_alloc((C + 1) * sizeof(*d_snum), 0);
    d_msk = (LOCINT *)emu_alloc(((row_pp + BITS(d_msk) - 1) / BITS(d_msk)) * sizeof(*d_msk), 0);
    d_lvl = (int *)emu_alloc(row_pp * sizeof(*d_lvl), -1);
    d_frt = d_sbuf;
    d_frt_start = d_sbuf;
    d_cbuf = d_cbuf_start;
    d_sig = (LOCINT *)emu_alloc(row_pp * sizeof(*d_sig), 0);
    d_delta = (float *)emu_alloc(row_pp * sizeof(*d_delta), 0);
    d_bc = (float *)emu_alloc(row_pp * sizeof(*d_bc), 0);
    d_reach = (LOCINT *)emu_alloc(row_pp * sizeof(*d_reach), 0);
    return 0;
}

// fincuda (src/cuda_kernels.cu:1649-1693); the dump ends with the final bc
void fincuda()
{
    if (dump_fp) {
        dump_rec(REC_BC, d_bc, row_pp * sizeof(float));
        dump_rec(REC_END, nullptr, 0);
        fclose(dump_fp);
        dump_fp = nullptr;
    }
    free(d_col);
    free(d_row);
    free(d_deg);
    free(d_cbuf_start);
    free(d_sbuf);
    free(d_snum);
    free(d_msk);
    free(d_lvl);
    free(d_sig);
    free(d_delta);
    free(d_bc);
    free(d_reach);
}

// init_bc_1degree_device (src/cuda_kernels.cu:1515-1519)
void init_bc_1degree_device(LOCINT *reach)
{
    memcpy(d_reach, reach, row_pp * sizeof(*reach));
    dump_rec(REC_REACH, reach, row_pp * sizeof(*reach));
}

// setcuda (src/cuda_kernels.cu:1532-1554), mono path
void setcuda(uint64_t ned, LOCINT *col, LOCINT *row, LOCINT reach_v0)
{
    (void)ned;
    (void)col;
    (void)row;
    memset(d_lvl, -1, row_pp * sizeof(*d_lvl));
    memset(d_sig, 0, row_pp * sizeof(*d_sig));
    emu_launch(init_delta, (row_pp + THREADS - 1) / THREADS, THREADS, d_reach, d_delta, (int)row_pp);
    memset(d_msk, 0, ((row_pp + BITS(d_msk) - 1) / BITS(d_msk)) * sizeof(*d_msk));
    d_reach_v0 = reach_v0;
    memset(tlvl, 0, sizeof(*tlvl) * MAX_LVL);
    d_cbuf = d_cbuf_start;
    d_frt = d_frt_start;
}

// set_mlp_cuda (src/cuda_kernels.cu:862-876)
void set_mlp_cuda(LOCINT row, int level, int sigma)
{
    d_msk[row / BITS(d_msk)] |= (1ULL << (row % BITS(d_msk)));
    d_lvl[row] = level;
    d_sig[row] = (LOCINT)sigma;
    d_frt[0] = row;
    dump_v0 = row;
}

// scan_col_csc_cuda_mono (src/cuda_kernels.cu:1088-1177) with ONEPREFIX and
// THRUST: frontier degrees, exclusive scan, edge-parallel expansion
LOCINT scan_col_csc_cuda_mono(int ncol, int level)
{
    LOCINT i, nfrt = 0, nrow = 0;
    int blocks;
    d_snum[0] = 0;
    emu_launch(read_edge_count, (ncol + THREADS - 1) / THREADS, THREADS, (const LOCINT *)d_deg,
               (const LOCINT *)d_frt, (LOCINT)ncol, d_cbuf);
    i = d_cbuf[ncol - 1];
    nrow = i;
    {  // thrust::exclusive_scan over d_cbuf[0, ncol)
        LOCINT run = 0;
        for (int k = 0; k < ncol; k++) {
            const LOCINT x = d_cbuf[k];
            d_cbuf[k] = run;
            run += x;
        }
    }
    i = d_cbuf[ncol - 1];
    nrow += i;
    tlvl[level] = nrow;
    if (nrow) {
        blocks = (((nrow + ROWXTH - 1) / ROWXTH) + THREADS - 1) / THREADS;
        emu_launch(scan_col_mono2, blocks, THREADS, (const LOCINT *)d_row, (const LOCINT *)d_col, nrow,
                   (const LOCINT *)d_frt, (const LOCINT *)d_cbuf, (LOCINT)ncol, d_msk, d_lvl, d_sig, level,
                   d_frt + ncol, d_snum);
    }
    nfrt = d_snum[0];
    d_frt = d_frt + ncol;
    d_cbuf = d_cbuf + ncol;
    return nfrt;
}

// scan_frt_csc_cuda_mono (src/cuda_kernels.cu:1013-1080) with ONEPREFIX
LOCINT scan_frt_csc_cuda_mono(int offset, int ncol, int depth)
{
    if (!ncol) return ncol;
    const int nrow = tlvl[depth + 1];
    LOCINT *d_ncbuf = d_cbuf_start + offset;
    if (!nrow) return ncol;
    const int blocks = (((nrow + ROWXTHD - 1) / ROWXTHD) + THREADS - 1) / THREADS;
    emu_launch(scan_frt_mono, blocks, THREADS, (const LOCINT *)d_row, (const LOCINT *)d_col, (LOCINT)nrow,
               (const LOCINT *)(d_frt_start + offset), (const LOCINT *)d_ncbuf, (LOCINT)ncol,
               (const LOCINT *)d_sig, d_delta, (const int *)d_lvl, depth);
    return ncol;
}

// pre_update_bc_cuda (src/cuda_kernels.cu:358-373): all = sum of reach[v]
// over the vertices with lvl[v] > 0, in uint32 arithmetic (deviceReduceKernel,
// :339-354)
void pre_update_bc_cuda(LOCINT *reach, LOCINT v0, LOCINT *all)
{
    (void)reach;
    (void)v0;
    LOCINT sum = 0;
    for (LOCINT i = 0; i < row_pp; i++) sum += d_reach[i] * (d_lvl[i] > 0);
    all[0] = sum;
}

// update_bc_cuda (src/cuda_kernels.cu:289-302)
void update_bc_cuda(LOCINT v0, double p, int ncol, const uint64_t nvisited)
{
    int r0 = -1;
    if (GI2PI(v0) == (LOCINT)myrow) r0 = GI2LOCI(v0);
    if (dump_fp) {
        struct {
            uint32_t v0, r0;
            double p;
            uint64_t nvisited;
        } h = {dump_v0, (uint32_t)r0, p, nvisited};
        const size_t a = row_pp * 4;
        const uint64_t len = sizeof(h) + 3 * a;
        const uint32_t tag = REC_PIVOT;
        fwrite(&tag, 4, 1, dump_fp);
        fwrite(&len, 8, 1, dump_fp);
        fwrite(&h, sizeof(h), 1, dump_fp);
        fwrite(d_lvl, 1, a, dump_fp);
        fwrite(d_sig, 1, a, dump_fp);
        fwrite(d_delta, 1, a, dump_fp);
    }
    emu_launch(update_bc, (ncol + THREADS - 1) / THREADS, THREADS, (const float *)d_delta, r0, p,
               (LOCINT)ncol, d_bc, d_reach, nvisited);
}

// getters (src/cuda_kernels.cu:1431-1477), one rank
void get_bc(float *bc) { memcpy(bc, d_bc, row_pp * sizeof(*d_bc)); }
void get_delta(float *delta) { memcpy(delta, d_delta, row_pp * sizeof(*d_delta)); }
void get_deg(LOCINT *deg) { memcpy(deg, d_deg, col_bl * sizeof(*d_deg)); }
void get_sigma(LOCINT *sigma) { memcpy(sigma + (mycol * row_bl), d_sig + (mycol * row_bl), row_bl * sizeof(*d_sig)); }
void get_lvl(int *lvl) { memcpy(lvl + (mycol * row_bl), d_lvl + (mycol * row_bl), row_bl * sizeof(*d_lvl)); }

// the 2-D multi-GPU path's entry points: linked, never called with -p 1x1
LOCINT scan_col_csc_cuda(LOCINT *, LOCINT, int *, int, LOCINT *, int *, LOCINT *, LOCINT *, int)
{
    not_emulated("scan_col_csc_cuda");
    return 0;
}
LOCINT scan_frt_csc_cuda(const LOCINT *, int, int, float *)
{
    not_emulated("scan_frt_csc_cuda");
    return 0;
}
LOCINT write_delta_cuda(LOCINT, float *, float *)
{
    not_emulated("write_delta_cuda");
    return 0;
}
LOCINT append_rows_cuda(LOCINT *, LOCINT, int *, int, LOCINT *, LOCINT *, LOCINT, int)
{
    not_emulated("append_rows_cuda");
    return 0;
}
int set_delta_cuda(float *, int)
{
    not_emulated("set_delta_cuda");
    return 0;
}
void set_get_overlap(LOCINT *, int *) { not_emulated("set_get_overlap"); }
void get_frt(LOCINT *) { not_emulated("get_frt"); }
void get_cbuf(LOCINT *) { not_emulated("get_cbuf"); }
void get_msk(LOCINT *) { not_emulated("get_msk"); }
void get_all(LOCINT *) { not_emulated("get_all"); }
void set_lvl(int *) { not_emulated("set_lvl"); }
void set_sigma(LOCINT *) { not_emulated("set_sigma"); }
