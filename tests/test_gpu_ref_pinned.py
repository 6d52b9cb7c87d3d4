"""The CUDA path against the reference program's own output.

Fixtures: tests/golden/ref_*.npz, written by the reference's single-GPU
program (see tests/test_ref_pinned.py and tests/golden/make_ref_golden.py).
Through the C ABI, for each recorded run:

  - the graph built on the device (the Graph500 generator and ingest on the
    GPU for -S, device ingest of the edge file for the grids) has the
    reference's CSC, bit for bit;
  - a sampled run at width 1 (the reference's sequence) draws the reference's
    pivots and stops where it stopped; probabilities exact for -z 0/1, within
    1e-4 relative for the float-weighted heuristics; bc within 1e-4 relative;
  - the plain per-pivot pass gives each pivot's levels and uint32 path counts
    bit for bit;
  - the batched pass over the reference's pivot list and probabilities gives
    the reference's bc within 1e-4 relative;
  - the command-line driver writes the reference's -o file (values within
    the %.2f rounding).
"""
import hashlib
import os
import subprocess

import numpy as np
import pytest

from test_ref_pinned import FIXTURES, GOLDEN, PROB_RTOL, RTOL, digest, load, sha

pytestmark = pytest.mark.gpu
ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CLI = os.path.join(ROOT, "axbc_gb300", "axbc")


def device_graph(ax, d):
    kind, size = str(d["graph"][0]), int(d["graph"][1])
    n = int(d["n"])
    if kind == "kron" and d["undirected"]:
        return ax.Graph.kronecker(size, 16, 23, 24, H=d["H"])
    if kind == "kron":
        e = ax.kron_edges(size, 16, 23, 24).astype(np.uint64)
        return ax.Graph.from_edges(e, n, undirected=False, H=d["H"])
    return ax.Graph.from_edges(d["edges"].astype(np.uint64), n, undirected=True, H=d["H"])


def close(got, want, what):
    got = np.asarray(got, np.float64)
    want = np.asarray(want, np.float64)
    bad = ~np.isclose(got, want, rtol=RTOL, atol=1e-3)
    assert not bad.any(), f"{what}: {bad.sum()} values beyond 1e-4 relative, e.g. {got[bad][:3]} vs {want[bad][:3]}"


@pytest.mark.parametrize("path", FIXTURES, ids=lambda p: os.path.basename(p)[4:-4])
def test_cuda_path_matches_reference_program(axbc, path):
    d = load(path)
    G = device_graph(axbc, d)
    col, row, reach = G.csc()
    assert sha(col) == str(d["col_sha"]) and sha(row) == str(d["row_sha"]) and sha(reach) == str(d["reach_sha"])
    ctx = axbc.Context(G)
    r = ctx.run_sampled(z=d["z"], nbfs=d["N"], bader_c=d["c"], nchecks=d["x"], H=d["H"], seed=4343543, W=1)
    assert np.array_equal(r["pivots"], d["pivots"]), "pivot sequence differs from the reference's"
    assert r["nrounds"] == int(d["rounds"]) and r["skipped"] == int(d["skipped"])
    assert r["stopped"] == bool(d["stopped"])
    if d["c"] > 0:
        assert np.array_equal(r["checks"], d["checks"])
    if d["z"] in (0, 1):
        assert np.array_equal(r["probs"], d["probs"])
    else:
        np.testing.assert_allclose(r["probs"], d["probs"], rtol=PROB_RTOL, atol=0)
    close(ctx.bc(), d["bc"], "bc of the sampled run")
    # plain passes: levels and path counts of the reference's pivots
    for i, (v0, p) in enumerate(zip(d["pivots"][:16], d["probs"][:16])):
        ctx.reset()
        st = ctx.run_pivot(int(v0), float(p), d["H"])
        assert np.array_equal(digest(ctx.levels(), ctx.sigma()), d["pivot_digest"][i]), f"pivot {i} ({v0})"
        assert st["nvisited"] + st["all"] == int(d["nvisited_all"][i])
        if i == 0:
            close(ctx.delta(), d["delta_first"], "dependencies of the first pivot")
    # batched passes over the reference's pivot list and probabilities
    ctx.reset()
    piv, pr = d["pivots"], d["probs"]
    for b in range(0, len(piv), 32):
        ctx.run_batch(piv[b:b + 32], pr[b:b + 32], d["H"], stats=False)
    close(ctx.bc(), d["bc"], "bc of the batched passes")
    ctx.close()
    G.close()


def test_cli_writes_the_reference_output_file(axbc, tmp_path):
    d = load(os.path.join(GOLDEN, "ref_s10_z0.npz"))
    out = tmp_path / "cli"
    argv = [str(a) for a in d["argv"]]
    r = subprocess.run([CLI, *argv, "-o", str(out)], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    got = open(f"{out}_1X1_0.log").read().splitlines()
    want = str(d["output_file"]).splitlines()
    assert len(got) == len(want)
    for a, b in zip(got, want):
        va, xa = a.split("\t")
        vb, xb = b.split("\t")
        assert va == vb
        assert abs(float(xa) - float(xb)) <= 0.0100001 + 1e-4 * abs(float(xb))
