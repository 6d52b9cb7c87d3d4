/* Test infrastructure: the CUDA built-ins that the reference's mono kernels
 * use, for running those kernels' own source text on the host (cuda_emu.cpp).
 *
 * A launch runs every (block, thread) of its grid one after the other.  For
 * kernels without barriers, warp shuffles or shared memory -- the mono
 * kernels read_edge_count, scan_col_mono2, scan_frt_mono, update_bc,
 * init_delta, set_degree -- that is one of the interleavings the GPU may
 * produce: each atomic below is applied whole, in thread order.  Integer
 * results (levels, uint32 path counts) do not depend on the interleaving;
 * float dependency sums do, in their last bits, as on the GPU. */
#ifndef AXBC_REFHOST_CUDA_SHIM_H
#define AXBC_REFHOST_CUDA_SHIM_H

#include <stdint.h>

#define __global__
#define __device__

struct emu_dim3 {
    unsigned x, y, z;
};
extern emu_dim3 threadIdx, blockIdx, blockDim, gridDim;

template <class T> static inline T __ldg(const T *p) { return *p; }

static inline unsigned atomicOr(unsigned *a, unsigned v)
{
    const unsigned o = *a;
    *a = o | v;
    return o;
}

/* ((old >= limit) ? 0 : old + 1), returning old */
static inline unsigned atomicInc(unsigned *a, unsigned limit)
{
    const unsigned o = *a;
    *a = o >= limit ? 0u : o + 1u;
    return o;
}

static inline unsigned atomicAdd(unsigned *a, unsigned v)
{
    const unsigned o = *a;
    *a = o + v;
    return o;
}

static inline float atomicAdd(float *a, float v)
{
    const float o = *a;
    *a = o + v;
    return o;
}

/* kernel<<<grid, block>>>(args...) */
template <class K, class... A> static void emu_launch(K kernel, unsigned grid, unsigned block, A... args)
{
    gridDim = {grid, 1, 1};
    blockDim = {block, 1, 1};
    for (unsigned b = 0; b < grid; b++)
        for (unsigned t = 0; t < block; t++) {
            blockIdx = {b, 0, 0};
            threadIdx = {t, 0, 0};
            kernel(args...);
        }
}

#endif
