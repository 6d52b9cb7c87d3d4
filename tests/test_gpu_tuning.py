"""The autotuner and the counting builds of the traversal kernels, through the
C ABI: neither may change a result.

- axbc_autotune times trial passes; afterwards the context's bc is what it
  was, the chosen factors and width are ones a sampled run accepts, and a run
  with them equals the oracle (and a run with fixed factors) bit for bit.
- axbc_ctx_count runs the counting builds of the forward push, forward pull
  and backward kernels; a counted run gives the same bits as an uncounted one,
  and its counts are consistent (every gather comes from a scanned entry)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

FACTORS = {0.03125, 0.125, 0.5, 1.0, 2.0, 4.0, 8.0, 16.0, 32.0}


@pytest.fixture(scope="module")
def kron12(axbc, orc):
    G = axbc.Graph.kronecker(12, 16)
    col, row, reach = G.csc()
    return G, orc.CSC(col, row, reach)


def test_autotune_keeps_bc_and_picks_usable_settings(axbc, orc, kron12):
    G, g = kron12
    ctx = axbc.Context(G)
    first = ctx.run_sampled(z=3, nbfs=64, bader_c=0, nchecks=1, H=0, seed=11, W=32)
    bc0, dl0 = ctx.bc(), ctx.delta()
    deg = G.deg()
    trial = np.random.default_rng(5).choice(np.flatnonzero(deg > 0), 64, replace=False).astype(np.uint32)
    t = ctx.autotune(trial)
    # the trial passes leave the context's results as they were
    assert np.array_equal(ctx.bc(), bc0)
    assert np.array_equal(ctx.delta(), dl0, equal_nan=True)
    assert t["push_factor_batch"] in FACTORS and t["push_factor_single"] in FACTORS
    assert t["batch_width"] in (8, 16, 32, 64)
    assert t["batch_te_per_s"] > 0 and t["plain_te_per_s"] > 0
    # a sampled run with the tuned width and factors equals the oracle
    ctx.reset()
    got = ctx.run_sampled(z=3, nbfs=96, bader_c=0, nchecks=1, H=0, seed=7, W=t["batch_width"])
    ref = orc.run(g, z=3, nbfs=96, bader_c=0, nchecks=1, H=0, seed=7, W=t["batch_width"])
    assert np.array_equal(got["pivots"], ref["pivots"])
    assert np.array_equal(ctx.bc(), ref["bc"], equal_nan=True)
    # and the factors only change directions, not bits
    tuned = ctx.bc()
    ctx.set_tuning(8.0, 8.0)
    ctx.reset()
    ctx.run_sampled(z=3, nbfs=96, bader_c=0, nchecks=1, H=0, seed=7, W=t["batch_width"])
    assert np.array_equal(ctx.bc(), tuned, equal_nan=True)
    assert first["nrounds"] > 0
    ctx.close()


@pytest.mark.parametrize("factor", [0.03125, 8.0, 1e30])
def test_counting_builds_change_no_bits(axbc, kron12, factor):
    G, _ = kron12
    ctx = axbc.Context(G)
    ctx.set_tuning(8.0, factor)
    ctx.run_sampled(z=3, nbfs=96, bader_c=0, nchecks=1, H=0, seed=3, W=32)
    want = ctx.bc()
    ctx.reset()
    ctx.count(True)
    ctx.run_sampled(z=3, nbfs=96, bader_c=0, nchecks=1, H=0, seed=3, W=32)
    counts = ctx.count_read()
    ctx.count(False)
    assert np.array_equal(ctx.bc(), want, equal_nan=True)
    bwd = counts["batch_bwd"]
    assert bwd["bytes"] > 0 and bwd["entries"] > 0 and bwd["pairs"] > 0
    # gathers are (entry, pivot) pairs: at most 32 per scanned entry
    assert bwd["gathers"] <= 32 * bwd["entries"]
    # every (vertex, pivot) dependency written is one reached pair: 96 pivots
    # reach at most n vertices each
    assert bwd["pairs"] <= 96 * G.n
    fwd = [counts.get(k) for k in ("batch_fwd_push", "batch_fwd_pull") if counts.get(k)]
    assert fwd, "no forward launch counted"
    for c in fwd:
        assert c["gathers"] <= 32 * c["entries"] and c["bytes"] >= 8 * c["entries"]
    if factor >= 1e30:
        assert "batch_fwd_pull" in counts
    # reading clears the counters
    assert ctx.count_read() == {}
    ctx.close()
