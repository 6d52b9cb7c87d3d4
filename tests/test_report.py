"""The accuracy report (restating the reference's scripts/old/ bcstat.pl and
diffrank.pl) on hand-made cases, and through the CLI's output format."""
import numpy as np

from axbc_gb300 import report


def test_value_error_matches_bcstat_definition():
    e = np.array([1.0, 2.0, 3.0, 0.0])
    a = np.array([1.0, 2.5, 1.0, 0.25])
    r = report.value_error(e, a)
    d = np.abs(e - a)
    assert r["mean_abs_diff"] == d.mean()
    assert np.isclose(r["std_abs_diff"], np.sqrt((d * d).mean() - d.mean() ** 2))
    assert r["min_node"] == 3 and r["min_nonzero_diff"] == 0.25
    assert r["max_node"] == 2 and r["max_diff"] == 2.0


def test_rank_score_identical_and_swapped():
    ids = np.arange(6)
    e = np.array([5.0, 4.0, 3.0, 2.0, 0.0, 0.0])
    assert report.rank_score(ids, e, e)["score"] == 1.0
    # swap the top two: both misplaced by one position out of n = 4
    a = np.array([4.0, 5.0, 3.0, 2.0, 0.0, 0.0])
    r = report.rank_score(ids, e, a)
    assert r["ranked"] == 4 and r["same_position"] == 2
    assert np.isclose(r["score"], (2 + 2 * (1 - 1 / 4)) / 4)
    # a vertex that leaves the top n scores nothing for its slot
    a2 = np.array([5.0, 4.0, 3.0, 0.0, 2.0, 0.0])
    r2 = report.rank_score(ids, e, a2)
    assert r2["same_position"] == 3 and np.isclose(r2["score"], 3 / 4)


def test_ties_break_by_vertex_id():
    ids = np.arange(4)
    e = np.array([1.0, 1.0, 1.0, 0.0])
    a = np.array([1.0, 1.0, 1.0, 0.0])
    assert report.rank_score(ids, e, a)["score"] == 1.0
    assert report.top_k_overlap(ids, e, a, 2) == 1.0


def test_spearman():
    x = np.arange(10, dtype=float)
    assert np.isclose(report.spearman(x, x), 1.0)
    assert np.isclose(report.spearman(x, -x), -1.0)


def test_files_in_the_cli_format(tmp_path):
    e = np.array([3.25, 0.0, 1.5, 7.0])
    a = np.array([3.0, 0.0, 1.75, 7.0])
    for name, v in (("e.log", e), ("a.log", a)):
        with open(tmp_path / name, "w") as f:
            for i, x in enumerate(v):
                f.write("%d\t%.2f\n" % (i, x))
    ie, ve, te = report.read_bc_file(tmp_path / "e.log")
    ia, va, _ = report.read_bc_file(tmp_path / "a.log")
    assert np.array_equal(ie, ia) and np.array_equal(ve, e)
    r = report.report(ie, ve, va, te)
    assert r["ranked"] == 3 and r["score"] == 1.0 and r["max_diff"] == 0.25
