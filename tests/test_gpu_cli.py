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
