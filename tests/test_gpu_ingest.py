"""Device graph ingest (axbc_graph_from_edges: mirror, norm_graph, one-degree
reduction, build_csc on the GPU) against the oracle's restatement of the
reference pipeline, on random multigraphs with the structures the one-degree
reduction treats specially: isolated edges, stars, self-loops (one sorting
first), repeated edges, vertices of degree 1 next to the largest ids."""
import gc

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def random_edges(rng):
    n = int(rng.integers(2, 500))
    parts = [rng.integers(0, n, size=(int(rng.integers(0, 4 * n)), 2))]
    for _ in range(int(rng.integers(0, 6))):  # isolated edges
        a, b = rng.integers(0, n, size=2)
        parts.append(np.array([[a, b]]))
    for _ in range(int(rng.integers(0, 4))):  # stars
        hub = rng.integers(0, n)
        leaves = rng.integers(0, n, size=int(rng.integers(1, 20)))
        parts.append(np.stack([np.full(len(leaves), hub), leaves], 1))
    if rng.random() < 0.5:  # self-loops, one of them on vertex 0 (sorts first)
        loops = rng.integers(0, n, size=int(rng.integers(1, 5)))
        parts.append(np.stack([loops, loops], 1))
        parts.append(np.array([[0, 0]]))
    if rng.random() < 0.5:  # a leaf on the largest id
        parts.append(np.array([[n - 1, int(rng.integers(0, n))]]))
    e = np.concatenate(parts).astype(np.uint64)
    e = e[rng.permutation(len(e))]
    if rng.random() < 0.3:
        e = np.concatenate([e, e[: len(e) // 3]])  # repeats
    return e, n


@pytest.mark.parametrize("case", range(60))
def test_device_ingest_matches_reference_pipeline(axbc, orc, case):
    rng = np.random.default_rng(7000 + case)
    e, n = random_edges(rng)
    undirected = bool(rng.random() < 0.8)
    H = int(rng.random() < 0.6) if undirected else 0
    g = orc.pipeline(e, n, undirected, H)
    G = axbc.Graph.from_edges(e, n, undirected, H)
    col, row, reach = G.csc()
    what = f"case {case}: n={n} edges={len(e)} undirected={undirected} H={H}"
    assert G.m == g.m, what
    assert np.array_equal(col, g.col), what
    assert np.array_equal(row[: g.m], g.row[: g.m]), what
    assert np.array_equal(reach, g.reach), what
    # and equal to the host pipeline of the library
    hc, hr, hrch, _ = axbc.edges_to_csc(e, n, undirected, H)
    assert np.array_equal(hc, col) and np.array_equal(hr[: g.m], row[: g.m]) and np.array_equal(hrch, reach)


def test_device_ingest_edge_cases(axbc, orc):
    for e, n, H in (
        (np.zeros((0, 2)), 5, 0),
        (np.zeros((0, 2)), 5, 1),
        (np.array([[3, 3]]), 5, 0),         # one self-loop: kept (sorts first)
        (np.array([[3, 3]]), 5, 1),
        (np.array([[1, 2]]), 4, 1),         # one isolated edge
        (np.array([[0, 1], [2, 3]]), 4, 1),
        (np.array([[0, 1], [0, 2], [0, 3]]), 4, 1),   # a star: all leaves go
        (np.array([[2, 2], [2, 3]]), 4, 1),  # a self-loop keeps its vertex
    ):
        e = np.asarray(e, np.uint64)
        g = orc.pipeline(e, n, True, H)
        G = axbc.Graph.from_edges(e, n, True, H)
        col, row, reach = G.csc()
        assert np.array_equal(col, g.col), (e.tolist(), H)
        assert np.array_equal(row[: g.m], g.row[: g.m]), (e.tolist(), H)
        assert np.array_equal(reach, g.reach), (e.tolist(), H)
    with pytest.raises(axbc.AxbcError):
        axbc.Graph.from_edges(np.array([[0, 9]], np.uint64), 5)
    with pytest.raises(axbc.AxbcError):
        axbc.Graph.from_edges(np.array([[0, 1]], np.uint64), 5, undirected=False, H=1)


def test_device_ingest_and_generator_free_everything_on_failure(axbc, orc):
    """Every device allocation of the ingest and generator paths made to fail
    in turn: the call reports AXBC_ERR_NOMEM, holds no device bytes afterwards,
    and the next call succeeds."""
    L = axbc.lib()
    rng = np.random.default_rng(5)
    e = rng.integers(0, 300, size=(1200, 2)).astype(np.uint64)
    gc.collect()  # objects of earlier tests freed by the collector would move the counter
    gc.disable()
    try:
        _ingest_failures(axbc, L, e)
    finally:
        gc.enable()


def _ingest_failures(axbc, L, e):
    calls = [lambda: axbc.Graph.from_edges(e, 300, True, 1),
             lambda: axbc.Graph.kronecker(8, 16, H=1),
             lambda: axbc.Graph.rmat(8, 8, H=0),
             lambda: axbc.Graph.grid(20, 0.02, 1e-2)]
    for call in calls:
        base = L.axbc_device_bytes_live()
        failures = 0
        # ingest, the adjacency with its task tables, and (on graphs with a
        # vertex of more than 64 neighbours) the renumbered view of the batched passes
        for k in range(80):
            L.axbc_inject_alloc_failure_after(k)
            try:
                G = call()
            except axbc.AxbcError as ex:
                assert ex.status == 3, ex
                failures += 1
                assert L.axbc_device_bytes_live() == base, f"leak after failing allocation {k}"
                continue
            finally:
                L.axbc_inject_alloc_failure_after(-1)
            G.close()
            assert L.axbc_device_bytes_live() == base
            break
        else:
            raise AssertionError("call still failing after 80 allocations")
        assert failures >= 3
