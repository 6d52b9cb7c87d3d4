"""Regenerate the golden fixtures from the reference's own code.

Runs the reference's Graph500 generator (compiled from its sources into
oracle/_ref by `make -C oracle ref`) with the arguments of gen_graph
(src/axbc2d.c:518-527: initiator .57/.19/.19/.05, seeds 23 and 24,
edgefactor 16) and stores:
  kron_s10_ef16.npz   the scale-10 edge list (uint16 pairs, generator order)
  kron_summary.json   sha256 of the scale-10..20 edge lists and, per scale and
                      -H 0/1, the CSC size, isolated / degree-1 counts, maximum
                      degree, removed leaves, and sha256 of col/row/reach as
                      built by the reference pipeline (mirror, norm_graph,
                      degree_reduction, build_csc) restated in oracle/.
Scale 23 (the headline graph, about 3 minutes of CPU) is added with --s23.
Usage: python tests/golden/make_golden.py [--s23]
"""
import hashlib
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))
import oracle  # noqa: E402


def sha(a):
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def main():
    oracle.build(ref=True)
    if not oracle.ref_kron_available():
        raise SystemExit("reference generator not built (needs the reference sources)")
    scales = [10, 12, 14, 16, 18, 20] + ([23] if "--s23" in sys.argv else [])
    path = os.path.join(HERE, "kron_summary.json")
    out = json.load(open(path)) if os.path.exists(path) else {}
    for scale in scales:
        e = oracle.ref_kron_edges(scale, 16)
        n = 1 << scale
        ent = {"n": n, "edges": int(len(e)), "edges_sha256": sha(e.astype(np.int64))}
        for H in (0, 1):
            g = oracle.pipeline(e, n, True, H)
            d = g.deg
            ent[f"H{H}"] = {
                "m": int(g.m), "isolated": int((d == 0).sum()), "deg1": int((d == 1).sum()),
                "maxdeg": int(d.max()), "removed": int(g.rem_ed),
                "reach_sum": int(g.reach.sum()),
                "col_sha256": sha(g.col), "row_sha256": sha(g.row), "reach_sha256": sha(g.reach),
            }
        out[str(scale)] = ent
        if scale == 10 and not os.path.exists(os.path.join(HERE, "kron_s10_ef16.npz")):
            np.savez_compressed(os.path.join(HERE, "kron_s10_ef16.npz"),
                                edges=e.astype(np.uint16))
    with open(path, "w") as f:
        json.dump(out, f, indent=1, sort_keys=True)
    print(json.dumps({k: v["H0"]["m"] for k, v in out.items()}))


if __name__ == "__main__":
    main()
