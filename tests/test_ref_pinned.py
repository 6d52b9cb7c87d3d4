"""The oracle against the reference program's own output (CPU).

The fixtures tests/golden/ref_*.npz were written by the reference's
single-GPU program itself (src/axbc2d.c and its generator compiled unchanged
against a one-rank MPI stand-in, its mono kernels run from their own source
text on the host; recipe: oracle/Makefile `refbc`, generator:
tests/golden/make_ref_golden.py).  For each recorded run the oracle must
reproduce:

  - the CSC the reference built (SHA-256 of col, row, reach),
  - the pivot sequence, rounds, skipped rounds and the Bader stop, exactly,
  - the pivot probabilities: exactly for the uniform and degree-based
    heuristics; within 1e-4 relative for the float-weighted ones (LCC, bc,
    dependency, inverse bc, mixture), whose normalising sums the reference
    accumulates left to right in float (relative error up to (n-1) 2^-24) and
    this build in double,
  - every pivot's levels and uint32 path counts, bit for bit,
  - dependencies and bc within 1e-4 relative (the reference adds dependency
    terms with float atomics in thread order; the oracle in its canonical
    order).
"""
import glob
import hashlib
import os

import numpy as np
import pytest

GOLDEN = os.path.join(os.path.dirname(__file__), "golden")
FIXTURES = sorted(glob.glob(os.path.join(GOLDEN, "ref_*.npz")))
RTOL = 1e-4
PROB_RTOL = 1e-4


def load(path):
    d = dict(np.load(path))
    argv = [str(a) for a in d["argv"]]

    def opt(flag, default):
        return int(argv[argv.index(flag) + 1]) if flag in argv else default

    d["z"] = opt("-z", 0)
    d["N"] = opt("-N", 1)
    d["c"] = opt("-c", 1)
    d["x"] = opt("-x", 1)
    d["H"] = opt("-H", 0)
    d["undirected"] = "-U" not in argv
    return d


def sha(a):
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def digest(lvl, sig):
    return np.frombuffer(hashlib.sha256(lvl.astype(np.int32).tobytes() +
                                        sig.astype(np.uint32).tobytes()).digest(), np.uint8)


def graph_of(orc, d):
    kind, size = str(d["graph"][0]), int(d["graph"][1])
    n = int(d["n"])
    if kind == "kron":
        e = orc.kron_edges(size, 16, 23, 24).astype(np.uint64)
    else:
        e = d["edges"].astype(np.uint64)
    return orc.pipeline(e, n, d["undirected"], d["H"])


def assert_close(got, want, what):
    got = np.asarray(got, np.float64)
    want = np.asarray(want, np.float64)
    bad = ~np.isclose(got, want, rtol=RTOL, atol=1e-3)
    assert not bad.any(), f"{what}: {bad.sum()} values beyond 1e-4 relative, e.g. {got[bad][:3]} vs {want[bad][:3]}"


def test_fixtures_present():
    names = {os.path.basename(p)[4:-4] for p in FIXTURES}
    for need in ("s10_z0", "s10_H1_z1", "s10_z3", "s14_z0_N256", "grid64_z4_bader"):
        assert need in names


@pytest.mark.parametrize("path", FIXTURES, ids=lambda p: os.path.basename(p)[4:-4])
def test_oracle_matches_reference_program(orc, path):
    d = load(path)
    g = graph_of(orc, d)
    assert g.n == int(d["n"]) and g.m == int(d["m"])
    assert sha(g.col) == str(d["col_sha"]) and sha(g.row) == str(d["row_sha"])
    assert sha(g.reach) == str(d["reach_sha"])
    r = orc.run(g, z=d["z"], nbfs=d["N"], bader_c=d["c"], nchecks=d["x"], H=d["H"], seed=4343543, W=1)
    assert np.array_equal(r["pivots"], d["pivots"]), "pivot sequence differs from the reference's"
    assert r["nrounds"] == int(d["rounds"]) and r["skipped"] == int(d["skipped"])
    assert r["stopped"] == bool(d["stopped"])
    if d["c"] > 0:
        assert np.array_equal(r["checks"], d["checks"])
    if d["z"] in (0, 1):
        assert np.array_equal(r["probs"], d["probs"])
    else:
        np.testing.assert_allclose(r["probs"], d["probs"], rtol=PROB_RTOL, atol=0)
    assert_close(r["bc"], d["bc"], "bc")
    # every pivot of the reference's list: levels and path counts bit for bit
    for i, (v0, p) in enumerate(zip(d["pivots"], d["probs"])):
        _, lvl, sig, dl, st = orc.bc_pivot(g, int(v0), float(p), d["H"])
        assert np.array_equal(digest(lvl, sig), d["pivot_digest"][i]), f"pivot {i} ({v0}): levels/sigma differ"
        assert st["nvisited"] + st["all"] == int(d["nvisited_all"][i])
        if i == 0:
            assert_close(dl, d["delta_first"], "dependencies of the first pivot")
        if i == len(d["pivots"]) - 1:
            assert_close(dl, d["delta_last"], "dependencies of the last pivot")


def test_reference_output_file_format(orc):
    """The -o file: one line per vertex, "%d\\t%.2f" of bc / 2 / nrounds."""
    d = load(os.path.join(GOLDEN, "ref_s10_z0.npz"))
    lines = str(d["output_file"]).splitlines()
    assert len(lines) == int(d["n"])
    want = d["bc"].astype(np.float32) / np.float32(2.0) / np.float32(int(d["rounds"]))
    for k, line in enumerate(lines):
        v, val = line.split("\t")
        assert int(v) == k
        assert abs(float(val) - float(want[k])) <= 0.005 + 1e-6 * abs(float(want[k]))
