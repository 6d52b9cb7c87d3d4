/* Test host (test infrastructure): the reference's single-GPU driver order,
 * bc_func_mono (src/axbc2d.c:1514-1659), restated in C against the
 * reference-named entry points of include/axbc_compat.h and linked against
 * libaxbc_gb300.so the way the reference's host links its CUDA file.  The
 * vertex count reaches the library through the host's global N, as in the
 * reference (src/axbc2d.c:29).
 *
 * Usage: compat_host GRAPH PIVOTS OUT H
 *   GRAPH   uint64 n, uint64 m, uint32 col[n+1], uint32 row[m], uint32 reach[n]
 *   PIVOTS  uint64 k, uint32 v[k]   (each pivot with p = 1/n)
 *   OUT     receives float bc[n], then uint32 deg[n]
 */
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>

#include "axbc_compat.h"

uint64_t N; /* the reference host's global vertex count */

static void *read_all(FILE *f, size_t bytes)
{
    void *p = malloc(bytes ? bytes : 1);
    if (!p || (bytes && fread(p, 1, bytes, f) != bytes)) {
        fprintf(stderr, "compat_host: short read\n");
        exit(2);
    }
    return p;
}

int main(int argc, char **argv)
{
    if (argc != 5) {
        fprintf(stderr, "usage: compat_host GRAPH PIVOTS OUT H\n");
        return 2;
    }
    const int H = atoi(argv[4]);
    FILE *fg = fopen(argv[1], "rb"), *fp = fopen(argv[2], "rb");
    if (!fg || !fp) return 2;
    uint64_t hdr[2], k = 0;
    if (fread(hdr, 8, 2, fg) != 2 || fread(&k, 8, 1, fp) != 1) return 2;
    const uint64_t n = hdr[0], m = hdr[1];
    uint32_t *col = (uint32_t *)read_all(fg, (n + 1) * 4);
    uint32_t *row = (uint32_t *)read_all(fg, m * 4);
    uint32_t *reach = (uint32_t *)read_all(fg, n * 4);
    uint32_t *piv = (uint32_t *)read_all(fp, k * 4);
    fclose(fg);
    fclose(fp);

    N = n;
    if (initcuda(m, col, row) == 0) return 3;
    init_bc_1degree_device(reach);
    /* frontier offsets per level (the reference's hFnum) */
    uint64_t *hF = (uint64_t *)calloc(n + 3, sizeof(uint64_t));
    for (uint64_t i = 0; i < k; i++) {
        const uint32_t v0 = piv[i];
        setcuda(m, col, row, reach[v0]);
        set_mlp_cuda(v0, 0, 1);
        uint64_t nfrt = 1, nvisited = 1;
        int level = 0;
        hF[0] = 0;
        for (;;) {
            level++;
            hF[level] = hF[level - 1] + nfrt;
            nfrt = scan_col_csc_cuda_mono((int)nfrt, level);
            if (!nfrt) break;
            nvisited += nfrt;
        }
        /* depths level-2 .. 1, at least one pass (the reference's do-while);
         * a degree-0 root has no depth to process */
        int depth = level - 2;
        if (depth >= 0) do {
                scan_frt_csc_cuda_mono((int)hF[depth], (int)(hF[depth + 1] - hF[depth]), depth);
                depth--;
            } while (depth > 0);
        uint32_t all = 0;
        if (H == 1) pre_update_bc_cuda(reach, v0, &all);
        update_bc_cuda(v0, 1.0 / (double)n, (int)n, nvisited + all + reach[v0]);
    }
    float *bc = (float *)malloc(n * sizeof(float));
    uint32_t *deg = (uint32_t *)malloc(n * sizeof(uint32_t));
    get_bc(bc);
    get_deg(deg);
    fincuda();
    FILE *fo = fopen(argv[3], "wb");
    if (!fo || fwrite(bc, 4, n, fo) != n || fwrite(deg, 4, n, fo) != n) return 4;
    fclose(fo);
    free(hF);
    free(bc);
    free(deg);
    free(col);
    free(row);
    free(reach);
    free(piv);
    return 0;
}
