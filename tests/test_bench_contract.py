"""bench.py's command line (CPU): the defaults the round-end runs rely on and
the workloads it offers."""
import os
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _parse(monkeypatch, *argv):
    sys.path.insert(0, ROOT)
    import bench
    monkeypatch.setattr(sys, "argv", ["bench.py", *argv])
    return bench, bench.parse()


def test_defaults(monkeypatch):
    bench, a = _parse(monkeypatch)
    assert a.gpus == 1 and a.warmup >= 3 and a.steps >= 1
    assert a.impl == "gb300" and a.workload == "headline"
    assert a.scale == 23 and a.edgefactor == 16 and a.pivots == 1024 and a.width == 32 and a.z == 3


def test_reference_arm_and_workloads(monkeypatch):
    bench, a = _parse(monkeypatch, "--impl", "reference", "--gpus", "2", "--steps", "5", "--warmup", "4")
    assert a.impl == "reference" and a.gpus == 2 and a.steps == 5 and a.warmup == 4
    for w in ("serving", "config1", "config2", "config3"):
        _, b = _parse(monkeypatch, "--workload", w)
        assert b.workload == w
    assert set(bench.CONFIGS) == {"config1", "config2", "config3"}
    assert bench.CONFIGS["config2"]["W"] == 64 and bench.CONFIGS["config2"]["H"] == 1
