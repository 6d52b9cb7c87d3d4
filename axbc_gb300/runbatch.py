"""Run multi-source batches on a generated graph and print per-batch statistics.

    python -m axbc_gb300.runbatch --graph grid:1024 [--batches 1] [--width 32] [--seed 7]
    python -m axbc_gb300.runbatch --graph kron:21 [--edgefactor 16] ...

Graphs: `grid:SIDE` (SIDE x SIDE four-neighbour grid, 2% of edges dropped,
0.01% long-range edges, seed 7), `kron:SCALE` (the Graph500 generator with
the reference's seeds 23/24, undirected) or `rmat:SCALE` (the library's R-MAT
generator, undirected).  Pivots
are drawn uniformly among vertices of nonzero degree with p = 1/n.  One JSON
line per batch: wall time, levels, traversed edges, per-kind kernel times and
how many levels overflowed their vertex list.  Meant for profiling one kernel
on one workload (e.g. under ncu with -k/-s/-c).
"""
from __future__ import annotations

import argparse
import json
import time

import numpy as np


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--graph", default="grid:1024")
    ap.add_argument("--edgefactor", type=int, default=16)
    ap.add_argument("--batches", type=int, default=1)
    ap.add_argument("--width", type=int, default=32)
    ap.add_argument("--seed", type=int, default=7)
    ap.add_argument("--profile", action="store_true", help="time every kernel with CUDA events")
    ap.add_argument("--push-factor", type=float, default=None,
                    help="batched push/pull factor (default: the library's)")
    ap.add_argument("--levels", action="store_true",
                    help="with --profile: per forward level / backward depth times (ms, > 0.005)")
    a = ap.parse_args()
    import axbc_gb300 as ax
    kind, size = a.graph.split(":")
    if kind == "grid":
        G = ax.Graph.grid(int(size), 0.02, 1e-4, seed=7)
    elif kind == "kron":
        G = ax.Graph.kronecker(int(size), a.edgefactor, 23, 24)
    elif kind == "rmat":
        G = ax.Graph.rmat(int(size), a.edgefactor, seed=23)
    else:
        raise SystemExit(f"unknown graph kind {kind!r}")
    ctx = ax.Context(G)
    if a.push_factor is not None:
        ctx.set_tuning(32.0, a.push_factor)
    deg = G.deg()
    rng = np.random.default_rng(a.seed)
    cand = np.flatnonzero(deg > 0)
    for b in range(a.batches):
        piv = rng.choice(cand, a.width, replace=False).astype(np.uint32)
        ctx.profile(a.profile)
        t0 = time.perf_counter()
        st = ctx.run_batch(piv, np.full(a.width, 1.0 / G.n))
        ctx.sync()
        dt = time.perf_counter() - t0
        per_level = {}
        if a.profile and a.levels:
            for kind, tag, ms, _ in ctx.profile_records():
                if tag >= 0 and ms > 0.005:
                    key = f"{kind}@{tag}"
                    per_level[key] = round(per_level.get(key, 0.0) + ms, 3)
        pr = ctx.profile_read() if a.profile else {}
        ls = ctx.level_stats()
        print(json.dumps({
            "batch": b, "graph": a.graph, "n": G.n, "s": round(dt, 5),
            "levels": int(max(s["levels"] for s in st)), "te": int(sum(s["te"] for s in st)),
            "overflow_levels": int(np.sum(ls["list_count"] > ls["list_cap"])),
            "kernel_ms": {k: round(v[0], 3) for k, v in pr.items() if v[1]},
            **({"level_ms": per_level} if per_level else {})}), flush=True)


if __name__ == "__main__":
    main()
