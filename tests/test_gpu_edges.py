"""Edge cases through the CUDA path, against the oracle: graphs without edges,
graphs smaller than a batch, degree-0 roots, repeated roots in one pass, stars
folded by the one-degree reduction, and the level limit of the batched
traversal."""
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu
GOLDEN = os.path.join(os.path.dirname(__file__), "golden")


def same_bits(got, want, what):
    same = (got == want) | (np.isnan(got) & np.isnan(want))
    assert same.all(), f"{what}: {np.count_nonzero(~same)} values differ"


def make(axbc, orc, edges, n, undirected=True, H=0):
    g = orc.pipeline(np.asarray(edges, np.uint64).reshape(-1, 2), n, undirected, H)
    return g, axbc.Graph.from_csc(g.col, g.row, g.reach)


@pytest.mark.parametrize("z", [0, 1, 2, 3, 4, 5, 6])
def test_graph_without_edges(axbc, orc, z):
    g, G = make(axbc, orc, np.zeros((0, 2)), 16)
    assert g.m == 0
    ctx = axbc.Context(G)
    got = ctx.run_sampled(z=z, nbfs=16, bader_c=0, nchecks=2, seed=3, W=8)
    want = orc.run(g, z=z, nbfs=16, bader_c=0, nchecks=2, seed=3, W=8)
    assert got["nrounds"] == want["nrounds"] == 0
    for k in ("skipped", "dropped", "ui_end", "stopped"):
        assert got[k] == want[k], k
    same_bits(ctx.bc(), want["bc"], "bc")
    assert not ctx.bc().any()


@pytest.mark.parametrize("W", [1, 32, 64])
def test_graph_smaller_than_a_batch(axbc, orc, W):
    # a path of 3 and a triangle, 7 vertices (one isolated): fewer vertices than lanes
    e = [(0, 1), (1, 2), (3, 4), (4, 5), (5, 3)]
    g, G = make(axbc, orc, e, 7)
    ctx = axbc.Context(G)
    for z in (0, 3, 4):
        got = ctx.run_sampled(z=z, nbfs=7, bader_c=0, nchecks=1, seed=5, W=W)
        want = orc.run(g, z=z, nbfs=7, bader_c=0, nchecks=1, seed=5, W=W)
        assert np.array_equal(got["pivots"], want["pivots"])
        for k in ("nrounds", "skipped", "dropped", "ui_end", "te"):
            assert got[k] == want[k], (z, k)
        same_bits(ctx.bc(), want["bc"], f"z={z}")


def test_degree_zero_roots_in_a_batch(axbc, orc):
    e = [(0, 1), (1, 2), (2, 3)]
    g, G = make(axbc, orc, e, 8)  # vertices 4..7 isolated
    ctx = axbc.Context(G)
    piv = np.array([4, 0, 5, 2], np.uint32)
    p = np.array([0.25, 0.5, 0.125, 1.0])
    st = ctx.run_batch(piv, p)
    want, dl, te = orc.bc_pivots(g, piv, p)
    assert sum(s["te"] for s in st) == te
    same_bits(ctx.bc(), want, "bc")
    same_bits(ctx.delta(), dl, "last delta")
    for v, pp in zip(piv, p):
        ctx.reset()
        ctx.run_pivot(v, pp, 0)
        want1, _, _ = orc.bc_pivots(g, np.array([v], np.uint32), np.array([pp]))
        same_bits(ctx.bc(), want1, f"plain pivot {v}")


@pytest.mark.parametrize("H", [0, 1])
def test_star_and_one_degree_reduction(axbc, orc, H):
    # hub 0 with 40 leaves, plus a second hub 41 sharing two leaves with it
    e = [(0, i) for i in range(1, 41)] + [(41, 1), (41, 2), (41, 42)]
    g, G = make(axbc, orc, e, 43, True, H)
    ctx = axbc.Context(G)
    for z in (0, 1):
        got = ctx.run_sampled(z=z, nbfs=43, bader_c=0, nchecks=1, H=H, seed=9, W=32)
        want = orc.run(g, z=z, nbfs=43, bader_c=0, nchecks=1, H=H, seed=9, W=32)
        assert np.array_equal(got["pivots"], want["pivots"])
        same_bits(ctx.bc(), want["bc"], f"H={H} z={z}")


def test_level_limit_is_an_error_and_the_context_recovers(axbc, orc):
    # a path of 70 000 vertices: from an end, deeper than the batched traversal's
    # 65 534 levels
    n = 70000
    e = np.stack([np.arange(n - 1), np.arange(1, n)], 1)
    g, G = make(axbc, orc, e, n)
    ctx = axbc.Context(G)
    with pytest.raises(axbc.AxbcError) as ex:
        ctx.run_batch(np.array([0], np.uint32), np.array([1.0 / n]))
    assert ex.value.status == 5  # AXBC_ERR_RANGE
    # the plain form has no level table and completes; the batched form still
    # works from a middle vertex (35 000 levels)
    ctx.reset()
    ctx.run_pivot(0, 1.0 / n, 0)
    want, _, _ = orc.bc_pivots(g, np.array([0], np.uint32), np.array([1.0 / n]))
    same_bits(ctx.bc(), want, "plain pass over 70 000 levels")
    ctx.reset()
    mid = np.array([n // 2, n // 2 + 1], np.uint32)
    ctx.run_batch(mid, np.array([1.0 / n, 1.0 / n]))
    want2, _, _ = orc.bc_pivots(g, mid, np.array([1.0 / n, 1.0 / n]))
    same_bits(ctx.bc(), want2, "batched pass after the error")


def test_repeated_pivots_in_one_batch(axbc, orc):
    """Lanes of different server requests can share a root: the level-0 list
    holds each root once, every lane still counts its own paths."""
    e = np.load(os.path.join(GOLDEN, "kron_s10_ef16.npz"))["edges"]
    g, G = make(axbc, orc, e, 1024)
    deg = g.deg
    hub = int(np.argmax(deg))
    other = int(np.flatnonzero(deg > 0)[3])
    piv = np.array([hub, other, hub, hub, other, 5], np.uint32)
    p = np.array([0.5, 0.25, 0.125, 0.5, 0.75, 1.0])
    ctx = axbc.Context(G)
    ctx.run_batch(piv, p)
    want, dl, _ = orc.bc_pivots(g, piv, p)
    same_bits(ctx.bc(), want, "bc with repeated roots")
    same_bits(ctx.delta(), dl, "last delta")
