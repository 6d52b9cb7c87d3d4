"""Accuracy report: an approximate bc output file against an exact one.

The output files are the reference's `-o` format, one `"%d\\t%.2f\\n"` line per
vertex (id, bc / 2 / rounds; src/axbc2d.c:3170-3176), as written by the CLI.
The report restates the reference's offline accuracy scripts:

- value error (scripts/old/bcstat.pl): mean and standard deviation of
  |exact - approx| over all vertices, the smallest nonzero and the largest
  difference with their vertices;
- rank score (scripts/old/diffrank.sh + diffrank.pl): both files sorted by
  printed value, descending, ties by vertex id; the top n kept, n = the number
  of exact values that do not print as 0.00; a position scores 1 when both
  lists hold the same vertex there, and a vertex misplaced in both lists scores
  1 - |position difference| / n; score = total / n;

plus Spearman's rank correlation and top-k overlaps.

    python -m axbc_gb300.report exact.log approx.log [--json]
"""
from __future__ import annotations

import argparse
import json
import math

import numpy as np


def read_bc_file(path):
    """(ids, values as printed) of a bc output file; lines that do not parse
    as `id<TAB>value` (headers of older formats) are skipped."""
    ids, vals, texts = [], [], []
    with open(path) as f:
        for line in f:
            parts = line.rstrip("\n").split("\t")
            if len(parts) != 2:
                continue
            try:
                i, v = int(parts[0]), float(parts[1])
            except ValueError:
                continue
            ids.append(i)
            vals.append(v)
            texts.append(parts[1])
    return np.array(ids, np.int64), np.array(vals, np.float64), texts


def value_error(exact, approx):
    """bcstat.pl: mean |d|, its standard deviation, min nonzero |d| and max |d|."""
    exact = np.asarray(exact, np.float64)
    approx = np.asarray(approx, np.float64)
    if exact.shape != approx.shape:
        raise ValueError("number of lines not equal")
    d = np.abs(exact - approx)
    n = len(d)
    ave = float(d.sum() / n) if n else 0.0
    var = float((d * d).sum() / n - ave * ave) if n else 0.0
    nz = np.flatnonzero(d > 0)
    imin = int(nz[np.argmin(d[nz])]) if len(nz) else -1
    imax = int(np.argmax(d)) if n and d.max() > 0 else -1
    return {"mean_abs_diff": ave, "std_abs_diff": math.sqrt(max(var, 0.0)),
            "min_nonzero_diff": float(d[imin]) if imin >= 0 else None, "min_node": imin,
            "max_diff": float(d[imax]) if imax >= 0 else 0.0, "max_node": imax}


def _order(ids, vals):
    """Vertex ids sorted by value descending, ties by id ascending (sort -k2nr -k1n)."""
    return ids[np.lexsort((ids, -vals))]


def rank_score(ids, exact, approx, exact_text=None):
    """diffrank.sh + diffrank.pl on two bc vectors over the same vertex ids."""
    ids = np.asarray(ids, np.int64)
    exact = np.asarray(exact, np.float64)
    approx = np.asarray(approx, np.float64)
    # n: entries before the first exact value printed as 0.00 in descending order
    printed = np.round(exact, 2) if exact_text is None else np.array([float(t) for t in exact_text])
    n = int(np.count_nonzero(printed != 0.0))
    fe = _order(ids, printed)[:n]
    fa = _order(ids, np.round(approx, 2))[:n]
    ok = int(np.count_nonzero(fe == fa))
    pos_e = {int(v): i for i, v in enumerate(fe) if fe[i] != fa[i]}
    pos_a = {int(v): i for i, v in enumerate(fa) if fe[i] != fa[i]}
    cnt = max(n, 1)
    hs = sum(1.0 - abs(pos_a[v] - pe) / cnt for v, pe in pos_e.items() if v in pos_a)
    return {"score": (ok + hs) / cnt, "ranked": n, "same_position": ok}


def spearman(exact, approx):
    """Spearman's rank correlation (average ranks for ties)."""
    def ranks(x):
        order = np.argsort(x, kind="mergesort")
        r = np.empty(len(x), np.float64)
        xs = x[order]
        i = 0
        while i < len(x):
            j = i
            while j + 1 < len(x) and xs[j + 1] == xs[i]:
                j += 1
            r[order[i:j + 1]] = (i + j) / 2.0
            i = j + 1
        return r
    a, b = ranks(np.asarray(exact, np.float64)), ranks(np.asarray(approx, np.float64))
    a -= a.mean()
    b -= b.mean()
    den = math.sqrt(float((a * a).sum() * (b * b).sum()))
    return float((a * b).sum() / den) if den > 0 else 1.0


def top_k_overlap(ids, exact, approx, k):
    te = set(_order(ids, np.asarray(exact, np.float64))[:k].tolist())
    ta = set(_order(ids, np.asarray(approx, np.float64))[:k].tolist())
    return len(te & ta) / max(k, 1)


def report(ids, exact, approx, exact_text=None):
    out = {"vertices": int(len(ids))}
    out.update(value_error(exact, approx))
    out.update(rank_score(ids, exact, approx, exact_text))
    out["spearman"] = spearman(exact, approx)
    for k in (10, 100, max(1, len(ids) // 100)):
        out[f"top{k}_overlap"] = top_k_overlap(ids, exact, approx, k)
    return out


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("exact")
    ap.add_argument("approx")
    ap.add_argument("--json", action="store_true")
    a = ap.parse_args()
    ie, ve, te = read_bc_file(a.exact)
    ia, va, _ = read_bc_file(a.approx)
    if not np.array_equal(ie, ia):
        raise SystemExit("the two files list different vertices")
    r = report(ie, ve, va, te)
    if a.json:
        print(json.dumps(r))
        return
    print(f"Average diff={r['mean_abs_diff']}; Dev. Standard={r['std_abs_diff']}; "
          f"Min diff={r['min_nonzero_diff']} (node={r['min_node']}), "
          f"Max diff={r['max_diff']} (node={r['max_node']})")
    print(f"Score={r['score']}")
    print(f"Spearman={r['spearman']:.6f}  " + "  ".join(
        f"{k}={v:.3f}" for k, v in r.items() if k.endswith("_overlap")))


if __name__ == "__main__":
    main()
