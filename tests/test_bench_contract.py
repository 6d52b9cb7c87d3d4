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


def test_traffic_is_the_committed_ratio_times_must_move_bytes(monkeypatch, tmp_path):
    """roofline.traffic: the ncu capture's DRAM bytes per must-move byte of the
    kernel build the run uses, times the run's own must-move bytes; nothing
    when the capture is of other kernel source, of another graph family, or
    when the run counted nothing."""
    import json
    bench, _ = _parse(monkeypatch)
    t = {"kronecker": {"graph": "kronecker-s22-ef16", "commit": "abc", "kernel_source_sha256": "S",
                       "kernels": {"k_bwd_step<1>": {"dram_per_must_move_byte": 2.0},
                                   "k_bwd_step<2>": {"dram_per_must_move_byte": 3.0}}}}
    (tmp_path / "profiles").mkdir()
    (tmp_path / "profiles" / "traffic.json").write_text(json.dumps(t))
    monkeypatch.setattr(bench, "ROOT", str(tmp_path))
    monkeypatch.setattr(bench, "kernel_source_digest", lambda: "S")
    assert bench.traffic_for("k_bwd_step", "kronecker-s23-ef16", 1e9, 1)[0] == 2e9
    assert bench.traffic_for("k_bwd_step", "kronecker-s23-ef16", 1e9, 2)[0] == 3e9
    assert bench.traffic_for("k_bwd_step", "grid-1024", 1e9, 1)[0] is None
    assert bench.traffic_for("k_fwd_pull_step", "kronecker-s23-ef16", 1e9, 1)[0] is None
    assert bench.traffic_for("k_bwd_step", "kronecker-s23-ef16", None, 1)[0] is None
    monkeypatch.setattr(bench, "kernel_source_digest", lambda: "other")
    val, note = bench.traffic_for("k_bwd_step", "kronecker-s23-ef16", 1e9, 1)
    assert val is None and "stale" in note


def test_committed_traffic_capture_is_of_the_committed_kernels():
    """profiles/traffic.json names the SHA-256 of the batched kernels' source
    it was captured from; bench.py reports DRAM traffic only while they match."""
    import json
    sys.path.insert(0, ROOT)
    import bench
    with open(os.path.join(ROOT, "profiles", "traffic.json")) as f:
        t = json.load(f)
    ent = t["kronecker"]
    assert ent["kernel_source_sha256"] == bench.kernel_source_digest()
    for k in ("k_bwd_step<1>", "k_bwd_step<2>", "k_fwd_pull_step<1>", "k_fwd_pull_step<2>"):
        assert ent["kernels"][k]["dram_per_must_move_byte"] > 0
