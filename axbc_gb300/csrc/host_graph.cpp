// Host-side graph ingest with the reference's semantics: edge-file reader,
// mirror, norm_graph, one-degree reduction and CSC build
// (src/axbc2d.c:333-445, 695-907, 2551-2622).
#include <algorithm>
#include <cinttypes>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <vector>

#include "../../include/axbc.h"

void axbc_set_error(const char *fmt, ...);

namespace {

struct Edge {
    uint64_t u, v;
    bool operator<(const Edge &o) const { return u != o.u ? u < o.u : v < o.v; }
    bool operator==(const Edge &o) const { return u == o.u && v == o.v; }
};

// norm_graph: sort, drop repeats and self-loops -- except that the first edge
// of the sorted list is always kept (src/axbc2d.c:818-841)
void norm(std::vector<Edge> &e)
{
    if (e.empty()) return;
    std::sort(e.begin(), e.end());
    size_t l = 1;
    for (size_t i = 1; i < e.size(); i++) {
        if (!(e[i] == e[i - 1]) && e[i].u != e[i].v) e[l++] = e[i];
    }
    e.resize(l);
}

// One-degree reduction on a sorted list (src/axbc2d.c:695-807).  A vertex u
// whose only entry is (u,v) is removed: (v,u) goes to the removed list.  The
// removed pairs are then matched in order against the kept list and every
// match dropped; reach counts the removed pairs the matching consumed.
void degree_reduce(std::vector<Edge> &e, std::vector<uint32_t> &reach)
{
    const size_t ne_in = e.size();
    if (ne_in == 0) return;
    std::vector<Edge> keep, gone;
    keep.reserve(ne_in);
    const uint64_t NONE = ~0ull;
    uint64_t prev_u = NONE;
    for (size_t i = 0; i + 1 < ne_in; i++) {
        const Edge cur = e[i], nxt = e[i + 1];
        if (cur.u == cur.v || cur == nxt) {
            prev_u = cur.u;
            continue;
        }
        if (cur.u != nxt.u && cur.u != prev_u) gone.push_back({cur.v, cur.u});
        else keep.push_back(cur);
        prev_u = cur.u;
    }
    const Edge last = e[ne_in - 1];
    if (last.u == prev_u) keep.push_back(last);
    else if (last.u != last.v) gone.push_back({last.v, last.u});

    std::sort(gone.begin(), gone.end());
    size_t p = 0;
    if (!gone.empty()) {
        std::vector<Edge> out;
        out.reserve(keep.size());
        for (const Edge &k : keep) {
            while (p < gone.size() && k.u > gone[p].u) p++;
            if (p < gone.size() && k == gone[p]) {
                p++;
                continue;
            }
            out.push_back(k);
        }
        keep.swap(out);
    }
    for (size_t i = 0; i < p; i++) reach[gone[i].u]++;
    e.swap(keep);
}

// build_csc (src/axbc2d.c:883-907): column = second vertex, rows in list order
void csc(const std::vector<Edge> &e, uint64_t n, std::vector<uint32_t> &col,
         std::vector<uint32_t> &row)
{
    col.assign(n + 1, 0);
    row.resize(e.size());
    for (const Edge &x : e) col[x.v + 1]++;
    for (uint64_t i = 0; i < n; i++) col[i + 1] += col[i];
    std::vector<uint32_t> pos(col.begin(), col.end() - 1);
    for (const Edge &x : e) row[pos[x.v]++] = (uint32_t)x.u;
}

template <class T>
T *copy_out(const std::vector<T> &v)
{
    T *p = (T *)malloc(v.size() ? v.size() * sizeof(T) : sizeof(T));
    if (p && !v.empty()) memcpy(p, v.data(), v.size() * sizeof(T));
    return p;
}

}  // namespace

extern "C" int axbc_edges_to_csc(const uint64_t *edges, uint64_t nedges, uint64_t n,
                                 int undirected, int H, uint32_t **col, uint32_t **row,
                                 uint64_t *m, uint32_t **reach, uint64_t *removed_leaves)
{
    if (!col || !row || !m || !reach || (!edges && nedges)) {
        axbc_set_error("axbc_edges_to_csc: null argument");
        return AXBC_ERR_INVALID;
    }
    if (n == 0 || n >= 0xffffffffull) {
        axbc_set_error("axbc_edges_to_csc: n must be in [1, 2^32-1)");
        return AXBC_ERR_INVALID;
    }
    if (H != 0 && H != 1) {
        axbc_set_error("axbc_edges_to_csc: H must be 0 or 1 (the reference rejects H >= 2)");
        return AXBC_ERR_INVALID;
    }
    std::vector<Edge> e;
    e.reserve(undirected ? 2 * nedges : nedges);
    for (uint64_t i = 0; i < nedges; i++) {
        if (edges[2 * i] >= n || edges[2 * i + 1] >= n) {
            axbc_set_error("edge %" PRIu64 " (%" PRIu64 ", %" PRIu64 ") has a vertex >= n", i,
                           edges[2 * i], edges[2 * i + 1]);
            return AXBC_ERR_INVALID;
        }
        e.push_back({edges[2 * i], edges[2 * i + 1]});
    }
    if (undirected) {  // mirror (src/axbc2d.c:333-351)
        for (uint64_t i = 0; i < nedges; i++)
            if (edges[2 * i] != edges[2 * i + 1]) e.push_back({edges[2 * i + 1], edges[2 * i]});
    }
    std::vector<uint32_t> rch(n, 0);
    if (H != 0) {
        norm(e);
        degree_reduce(e, rch);
    }
    norm(e);
    if (e.size() >= 0xffffffffull) {
        axbc_set_error("too many adjacency entries for 32-bit offsets");
        return AXBC_ERR_RANGE;
    }
    std::vector<uint32_t> c, r;
    csc(e, n, c, r);
    uint64_t removed = 0;
    for (uint32_t x : rch) removed += x;
    *col = copy_out(c);
    *row = copy_out(r);
    *reach = copy_out(rch);
    *m = r.size();
    if (removed_leaves) *removed_leaves = removed;
    if (!*col || !*row || !*reach) {
        axbc_set_error("host allocation failed");
        return AXBC_ERR_NOMEM;
    }
    return AXBC_OK;
}

extern "C" void axbc_host_free(void *p) { free(p); }

// read_graph (src/axbc2d.c:356-445) for one rank: '#' lines are comments,
// "# Nodes: N Edges: M" headers are informational, other lines hold "u v".
// Lines that do not parse are skipped (the reference would repeat the
// previous edge, which norm_graph removes again).
extern "C" int axbc_read_edge_file(const char *path, uint64_t n, uint64_t **edges,
                                   uint64_t *nedges)
{
    if (!path || !edges || !nedges) {
        axbc_set_error("axbc_read_edge_file: null argument");
        return AXBC_ERR_INVALID;
    }
    FILE *fp = fopen(path, "r");
    if (!fp) {
        axbc_set_error("cannot open %s", path);
        return AXBC_ERR_INVALID;
    }
    std::vector<uint64_t> out;
    char line[1024];
    uint64_t lineno = 0;
    while (fgets(line, sizeof line, fp)) {
        lineno++;
        if (strchr(line, '#')) continue;
        uint64_t i, j;
        if (sscanf(line, "%" SCNu64 " %" SCNu64, &i, &j) != 2) continue;
        if (i >= n || j >= n) {
            fclose(fp);
            axbc_set_error("%s line %" PRIu64 ": invalid edge (%" PRIu64 ", %" PRIu64
                           ") for N=%" PRIu64,
                           path, lineno, i, j, n);
            return AXBC_ERR_INVALID;
        }
        out.push_back(i);
        out.push_back(j);
    }
    fclose(fp);
    *nedges = out.size() / 2;
    *edges = copy_out(out);
    return *edges ? AXBC_OK : AXBC_ERR_NOMEM;
}
