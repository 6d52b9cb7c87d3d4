"""The command-line driver on a GPU: the reference's option surface and output
file, and the accuracy report of a sampled run against the full enumeration."""
import os
import subprocess

import numpy as np
import pytest

from axbc_gb300 import report

pytestmark = pytest.mark.gpu
ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CLI = os.path.join(ROOT, "axbc_gb300", "axbc")


def run_cli(axbc, tmp_path, name, *opts):
    out = tmp_path / name
    r = subprocess.run([CLI, "-p", "1x1", "-S", "10", "-E", "16", "-o", str(out), *opts],
                       capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    path = f"{out}_1X1_0.log"
    assert os.path.exists(path), r.stdout
    return path, r.stdout


def test_cli_output_and_accuracy_report(axbc, tmp_path):
    # 1024 uniform rounds without repeated pivots: (almost) every vertex once
    exact, log = run_cli(axbc, tmp_path, "exact", "-N", "1024", "-z", "0", "-c", "0", "-W", "32")
    assert "Result written to file" in log
    ids, ve, te = report.read_bc_file(exact)
    assert np.array_equal(ids, np.arange(1024)) and (ve >= 0).all() and ve.max() > 0
    with open(exact) as f:
        first = f.readline()
    assert first.count("\t") == 1 and first.rstrip("\n").split("\t")[1].count(".") == 1
    approx, _ = run_cli(axbc, tmp_path, "approx", "-N", "128", "-z", "3", "-c", "0", "-W", "32")
    ia, va, _ = report.read_bc_file(approx)
    assert np.array_equal(ids, ia)
    r = report.report(ids, ve, va, te)
    assert 0.0 < r["score"] <= 1.0 and r["ranked"] > 0
    assert r["spearman"] > 0.5  # 128 bc-guided pivots already order the hubs
    same = report.report(ids, ve, ve, te)
    assert same["score"] == 1.0 and same["max_diff"] == 0.0
    # width 1 and width 32 give the same enumeration (static heuristic)
    exact1, _ = run_cli(axbc, tmp_path, "exact1", "-N", "1024", "-z", "0", "-c", "0", "-W", "1")
    _, v1, _ = report.read_bc_file(exact1)
    assert np.array_equal(v1, ve)


@pytest.mark.parametrize("opts,H,z,nbfs,W,undirected", [
    (("-N", "96", "-z", "1", "-c", "0", "-H", "1", "-W", "64"), 1, 1, 96, 64, True),
    (("-N", "200", "-z", "5", "-c", "0"), 0, 5, 200, 1, True),
    (("-N", "64", "-z", "0", "-c", "0", "-U", "-W", "32"), 0, 0, 64, 32, False),
])
def test_cli_output_file_equals_the_reference_definition(axbc, orc, tmp_path, opts, H, z, nbfs, W,
                                                         undirected):
    """The reference's command line on its own generated input (-S 10 -E 16:
    the Graph500 generator, seeds 23/24; -U keeps its pairs directed): the
    output file is the oracle's run on the reference pipeline's graph, printed
    as bc/2/nrounds with "%d\\t%.2f"."""
    path, _ = run_cli(axbc, tmp_path, f"ref{z}{int(undirected)}", *opts)
    e = orc.kron_edges(10, 16).astype(np.uint64)
    g = orc.pipeline(e, 1024, undirected, H)
    want = orc.run(g, z=z, nbfs=nbfs, bader_c=0, nchecks=1, H=H, seed=4343543, W=W)
    bc = want["bc"].astype(np.float32)
    lines = [f"{k}\t{float(bc[k]) / 2.0 / want['nrounds']:.2f}\n" for k in range(1024)]
    with open(path) as f:
        got = f.readlines()
    assert got == lines
