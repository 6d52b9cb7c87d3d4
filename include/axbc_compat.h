/*
 * axbc_gb300 -- the reference's own host/CUDA boundary, re-implemented.
 *
 * fvella/axbc's host driver (src/axbc2d.c) drives the single-GPU Brandes pass
 * through the extern "C" functions declared in src/bc2d.h:136-190 and defined
 * in src/cuda_kernels.cu.  libaxbc_gb300.so exports the ones that path uses
 * under the same names and signatures, so that driver can link against this
 * library instead of cuda_kernels.o.  LOCINT is uint32_t (the reference's
 * default build, src/bc2d.h:18).
 *
 * Conventions kept from the reference: one implicit graph per process; every
 * call returns synchronised; a CUDA failure prints a message and exits the
 * process (MY_CUDA_CHECK, src/cudamacro.h:1-16).  The vertex count comes from
 * the host program's global `uint64_t N` (src/axbc2d.c:29) when it defines
 * one, else from axbc_compat_set_n().  The 2-D multi-GPU entry points of
 * src/bc2d.h (scan_col_csc_cuda, append_rows_cuda, ...) are not provided.
 */
#ifndef AXBC_COMPAT_H
#define AXBC_COMPAT_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Vertex count for callers that do not define the global N. */
void axbc_compat_set_n(uint64_t n);

/* initcuda, src/cuda_kernels.cu:1558-1662: upload the CSC (col has N+1
 * entries, row ned), compute degrees; returns device bytes allocated. */
size_t initcuda(uint64_t ned, uint32_t *col, uint32_t *row);
/* fincuda, :1666-1693 */
void fincuda(void);
/* init_bc_1degree_device, :1515-1519: upload reach[N] */
void init_bc_1degree_device(uint32_t *reach);
/* setcuda, :1532-1554: lvl = -1, sigma = 0, delta = reach, remember reach_v0 */
void setcuda(uint64_t ned, uint32_t *col, uint32_t *row, uint32_t reach_v0);
/* set_mlp_cuda, :862-876: seed `row` with level and sigma; frontier = {row} */
void set_mlp_cuda(uint32_t row, int level, int sigma);
/* scan_col_csc_cuda_mono, :1088-1177: expand the ncol-vertex frontier to
 * `level`; returns the size of the new frontier, which becomes current. */
uint32_t scan_col_csc_cuda_mono(int ncol, int level);
/* scan_frt_csc_cuda_mono, :1013-1080: dependencies of the ncol vertices at
 * frontier offset `offset` (depth `depth`); returns ncol. */
uint32_t scan_frt_csc_cuda_mono(int offset, int ncol, int depth);
/* pre_update_bc_cuda, :358-373: *all = sum of reach over vertices at level > 0 */
void pre_update_bc_cuda(uint32_t *reach, uint32_t v0, uint32_t *all);
/* update_bc_cuda, :289-302 */
void update_bc_cuda(uint32_t v0, double p, int ncol, const uint64_t nvisited);
/* getters, :1431-1477 (N entries each) */
void get_bc(float *bc);
void get_delta(float *delta);
void get_deg(uint32_t *deg);
void get_sigma(uint32_t *sigma);
void get_lvl(int *lvl);
void get_frt(uint32_t *frt);
void get_msk(uint32_t *msk);
void get_all(uint32_t *all);
/* pinned host buffers, :837-849 */
void *CudaMallocHostSet(size_t size, int val);
void CudaFreeHost(void *ptr);

#ifdef __cplusplus
}
#endif
#endif /* AXBC_COMPAT_H */
