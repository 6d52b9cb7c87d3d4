"""The benchmark configurations as parity cases at full size.

Config 1: the reference's scale-14 graph, -z 0 -N 256, seed 1.
Config 2: the reference's scale-20 graph, one-degree reduction (-H 1), heuristic 1, width 64.
Config 3: 2048x2048 grid, 2% of edges dropped (seed 7), 0.01% long-range edges,
heuristic 4 with Bader's stop (-c 1 -x 8).  On this graph uint32 path counts
wrap and floats overflow (hundreds of BFS levels): comparisons are type for
type, and inf/NaN positions must match.
The oracle runs a bounded number of pivots on the full graphs."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def same_floats(got, want, what, rtol=1e-4):
    assert got.shape == want.shape
    nan_g, nan_w = np.isnan(got), np.isnan(want)
    assert np.array_equal(nan_g, nan_w), f"{what}: NaN positions differ"
    ok = ~nan_g
    np.testing.assert_allclose(got[ok], want[ok], rtol=rtol, atol=1e-6, err_msg=what)
    assert np.array_equal(got[ok], want[ok]), f"{what}: last-bit differences"


def csc_of(orc, G):
    col, row, reach = G.csc()
    return orc.CSC(col, row, reach)


@pytest.fixture(scope="module")
def kron20(axbc, orc):
    # the reference's scale-20 input (Graph500 generator, seeds 23/24), -H 1
    G = axbc.Graph.kronecker(20, 16, H=1)
    return G, csc_of(orc, G)


def test_config2_scale20_H1_z1_sampled(axbc, orc, kron20):
    G, g = kron20
    assert int(g.reach.sum()) > 0  # leaves were folded into reach
    ctx = axbc.Context(G)
    got = ctx.run_sampled(z=1, nbfs=80, bader_c=0, nchecks=1, H=1, seed=1, W=64)
    want = orc.run(g, z=1, nbfs=80, bader_c=0, nchecks=1, H=1, seed=1, W=64)
    assert np.array_equal(got["pivots"], want["pivots"])
    assert np.array_equal(got["probs"], want["probs"])
    assert got["te"] == want["te"] and got["skipped"] == want["skipped"]
    same_floats(ctx.bc(), want["bc"], "bc, scale 20")


def test_config2_full_budget_runs_and_is_deterministic(axbc, kron20):
    G, _ = kron20
    ctx = axbc.Context(G)
    a = ctx.run_sampled(z=1, nbfs=4096, bader_c=0, nchecks=1, H=1, seed=1, W=64)
    bc_a = ctx.bc()
    b = ctx.run_sampled(z=1, nbfs=4096, bader_c=0, nchecks=1, H=1, seed=1, W=64)
    assert a["nrounds"] == b["nrounds"] and a["te"] == b["te"] and a["nrounds"] > 1000
    assert np.array_equal(bc_a, ctx.bc())
    assert np.all(bc_a >= 0)


@pytest.fixture(scope="module")
def grid2048(axbc, orc):
    G = axbc.Graph.grid(2048, 0.02, 1e-4, seed=7)
    return G, csc_of(orc, G)


def test_config3_grid_batch_matches_oracle(axbc, orc, grid2048):
    G, g = grid2048
    ctx = axbc.Context(G)
    deg = g.deg
    rng = np.random.default_rng(7)
    piv = rng.choice(np.flatnonzero(deg > 0), 16, replace=False).astype(np.uint32)
    p = np.full(16, 1.0 / G.n)
    stats = ctx.run_batch(piv, p)
    want, dl, te = orc.bc_pivots(g, piv, p)
    assert sum(s["te"] for s in stats) == te
    assert max(s["levels"] for s in stats) > 200  # high diameter
    same_floats(ctx.bc(), want, "grid bc")
    same_floats(ctx.delta(), dl, "grid last delta")
    sig, lvl, _ = ctx.batch_source(0)
    _, olvl, osig, _, _ = orc.bc_pivot(g, int(piv[0]), p[0])
    assert np.array_equal(lvl, olvl) and np.array_equal(sig, osig)
    assert np.any(osig == 0) or osig.max() > 2**31  # counts wrap mod 2^32 on this graph


def test_config3_grid_sampled_adaptive_matches_oracle(axbc, orc, grid2048):
    G, g = grid2048
    ctx = axbc.Context(G)
    got = ctx.run_sampled(z=4, nbfs=48, bader_c=1, nchecks=8, seed=7, W=16)
    want = orc.run(g, z=4, nbfs=48, bader_c=1, nchecks=8, seed=7, W=16)
    assert np.array_equal(got["checks"], want["checks"])
    assert np.array_equal(got["pivots"], want["pivots"])
    assert got["nrounds"] == want["nrounds"] and got["stopped"] == want["stopped"]
    same_floats(ctx.bc(), want["bc"], "grid sampled bc")


@pytest.mark.parametrize("W", [1, 32, 64])
def test_config1_scale14_z0_sampled(axbc, orc, W):
    """Config 1: the reference's scale-14 graph (Graph500 generator, seeds
    23/24, built on the device), -H 0 -z 0 -N 256 -c 0, seed 1: the whole run
    bit for bit against the oracle on the reference pipeline's CSC of the
    restated generator's edges."""
    G = axbc.Graph.kronecker(14, 16)
    g = orc.pipeline(orc.kron_edges(14, 16).astype(np.uint64), 1 << 14, True, 0)
    col, row, _ = G.csc()
    assert np.array_equal(col, g.col) and np.array_equal(row, g.row)
    assert g.m == 430200
    ctx = axbc.Context(G)
    got = ctx.run_sampled(z=0, nbfs=256, bader_c=0, nchecks=1, H=0, seed=1, W=W)
    want = orc.run(g, z=0, nbfs=256, bader_c=0, nchecks=1, H=0, seed=1, W=W)
    assert np.array_equal(got["pivots"], want["pivots"])
    for k in ("nrounds", "skipped", "dropped", "te"):
        assert got[k] == want[k], k
    same_floats(ctx.bc(), want["bc"], "bc, config 1")
