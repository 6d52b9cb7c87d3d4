"""The product's host graph pipeline (libaxbc_gb300: axbc_edges_to_csc,
axbc_read_edge_file) against the oracle's restatement of the reference."""
import os

import numpy as np
import pytest

GOLDEN = os.path.join(os.path.dirname(__file__), "golden")


def _same(axbc, orc, edges, n, undirected, H):
    col, row, reach, rem = axbc.edges_to_csc(edges, n, undirected, H)
    g = orc.pipeline(edges, n, undirected, H)
    assert np.array_equal(col, g.col)
    assert np.array_equal(row, g.row)
    assert np.array_equal(reach, g.reach)
    assert rem == int(g.reach.sum())


@pytest.mark.parametrize("H", [0, 1])
@pytest.mark.parametrize("undirected", [True, False])
def test_golden_kronecker(axbc, orc, H, undirected):
    e = np.load(os.path.join(GOLDEN, "kron_s10_ef16.npz"))["edges"].astype(np.uint64)
    _same(axbc, orc, e, 1024, undirected, H)


@pytest.mark.parametrize("seed", range(12))
@pytest.mark.parametrize("H", [0, 1])
def test_random_multigraphs(axbc, orc, seed, H):
    rng = np.random.default_rng(seed)
    n = int(rng.integers(2, 200))
    m = int(rng.integers(0, 4 * n))
    e = rng.integers(0, n, size=(m, 2)).astype(np.uint64)
    # duplicates and self-loops on purpose
    if m:
        e = np.concatenate([e, e[: m // 5], np.repeat(e[:3, :1], 2, axis=1)])
    _same(axbc, orc, e, n, bool(seed % 2), H)


def test_empty_and_edge_cases(axbc, orc):
    _same(axbc, orc, np.zeros((0, 2), np.uint64), 5, True, 0)
    _same(axbc, orc, np.zeros((0, 2), np.uint64), 5, True, 1)
    _same(axbc, orc, np.array([[3, 3]], np.uint64), 5, True, 1)
    _same(axbc, orc, np.array([[0, 0], [0, 1]], np.uint64), 2, True, 0)
    _same(axbc, orc, np.array([[1, 0]], np.uint64), 2, True, 1)


def test_rejects_bad_input(axbc):
    with pytest.raises(axbc.AxbcError):
        axbc.edges_to_csc(np.array([[0, 5]], np.uint64), 5, True, 0)
    with pytest.raises(axbc.AxbcError):
        axbc.edges_to_csc(np.array([[0, 1]], np.uint64), 5, True, 2)


def test_read_edge_file(axbc, tmp_path):
    p = tmp_path / "g.txt"
    p.write_text("# Directed graph\n# Nodes: 6 Edges: 4\n0 1\n1\t2\n\n3 4\n5 0\n")
    e = axbc.read_edge_file(str(p), 6)
    assert e.tolist() == [[0, 1], [1, 2], [3, 4], [5, 0]]
    bad = tmp_path / "bad.txt"
    bad.write_text("0 1\n7 2\n")
    with pytest.raises(axbc.AxbcError):
        axbc.read_edge_file(str(bad), 6)


def _adversarial(rng):
    """Random multigraph with the structures the one-degree reduction treats
    specially: isolated edges, stars, self-loops (one on vertex 0, which sorts
    first), repeated edges, a leaf on the largest id."""
    n = int(rng.integers(2, 400))
    parts = [rng.integers(0, n, size=(int(rng.integers(0, 3 * n)), 2))]
    for _ in range(int(rng.integers(0, 6))):
        parts.append(rng.integers(0, n, size=(1, 2)))
    for _ in range(int(rng.integers(0, 4))):
        hub = rng.integers(0, n)
        leaves = rng.integers(0, n, size=int(rng.integers(1, 20)))
        parts.append(np.stack([np.full(len(leaves), hub), leaves], 1))
    if rng.random() < 0.5:
        loops = rng.integers(0, n, size=int(rng.integers(1, 5)))
        parts.append(np.stack([loops, loops], 1))
        parts.append(np.array([[0, 0]]))
    if rng.random() < 0.5:
        parts.append(np.array([[n - 1, int(rng.integers(0, n))]]))
    e = np.concatenate(parts).astype(np.uint64)
    e = e[rng.permutation(len(e))]
    if rng.random() < 0.3:
        e = np.concatenate([e, e[: len(e) // 3]])
    return e, n


@pytest.mark.parametrize("seed", range(40))
def test_adversarial_multigraphs(axbc, orc, seed):
    rng = np.random.default_rng(9000 + seed)
    e, n = _adversarial(rng)
    undirected = bool(rng.random() < 0.8)
    H = int(rng.random() < 0.6)
    _same(axbc, orc, e, n, undirected, H)
