/* Test infrastructure: exposes the reference's Graph500 generator (compiled
 * from its own sources by oracle/Makefile) through one C call, with the
 * arguments gen_graph passes (src/axbc2d.c:518-527): initiator
 * .57/.19/.19/.05, seeds 23 and 24, (2^scale)*edgefactor edges. */
#include <stdint.h>
#include <stdlib.h>
/* make_graph.h's sequential prototype ends in a stray comma and does not
 * compile, so the signature of the sequential make_graph is declared here. */
void make_graph(int log_numverts, int64_t desired_nedges, uint64_t userseed1,
                uint64_t userseed2, const double initiator[4], int64_t *nedges,
                int64_t **result);

int64_t ref_kron_edges(int scale, int edgef, uint64_t seed1, uint64_t seed2, int64_t **out)
{
    double initiator[4] = {.57, .19, .19, .05};
    int64_t ned = 0;
    make_graph(scale, (((int64_t)1) << scale) * edgef, seed1, seed2, initiator, &ned, out);
    return ned;
}

/* the same with another initiator */
int64_t ref_kron_edges_ini(int scale, int edgef, uint64_t seed1, uint64_t seed2, const double ini[4],
                           int64_t **out)
{
    double initiator[4] = {ini[0], ini[1], ini[2], ini[3]};
    int64_t ned = 0;
    make_graph(scale, (((int64_t)1) << scale) * edgef, seed1, seed2, initiator, &ned, out);
    return ned;
}

void ref_kron_free(void *p) { free(p); }
