"""The persistent level loop: a batched pass as one cooperative launch with a
bounded grid barrier between its phases.

- The barrier itself: every round completes; with one block that never
  arrives, the first wait runs out of its (short) budget, every block
  returns, the failure site is reported and the device stays usable.
- Results: a pass run persistently equals the same pass run as step
  launches, bit for bit, and the oracle, on a grid, a graph with heavy
  vertices, a directed graph, with one-degree reduction, and on a graph deep
  enough that the loop must ask the host for more level masks mid-pass."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def same_bits(got, want, what):
    same = (got == want) | (np.isnan(got) & np.isnan(want))
    assert same.all(), f"{what}: {np.count_nonzero(~same)} values differ"


@pytest.mark.parametrize("bps", [1, 2, 4])
def test_grid_barrier_rounds(axbc, bps):
    site, leads, ms = axbc.selftest_grid_barrier(blocks_per_sm=bps, rounds=2000)
    assert site == 0 and leads == 2000
    assert ms / 2000 < 0.1  # well under 100 us per barrier


def test_grid_barrier_wait_runs_out_and_device_stays_usable(axbc):
    # block 0 never arrives: every other block gives up after ~2^22 cycles
    site, leads, _ = axbc.selftest_grid_barrier(blocks_per_sm=2, rounds=10, budget_cycles=1 << 22,
                                                absent_block=0)
    assert site == 1 and leads == 0
    site, leads, _ = axbc.selftest_grid_barrier(blocks_per_sm=2, rounds=10)
    assert site == 0 and leads == 10
    G = axbc.Graph.grid(64, 0.02, 1e-3, seed=3)
    ctx = axbc.Context(G)
    ctx.set_persistent(1)
    ctx.run_batch(np.arange(8, dtype=np.uint32), np.full(8, 1.0 / G.n), 0, stats=False)
    assert np.isfinite(ctx.bc()).all()


def graphs(axbc, orc):
    out = {"grid128": axbc.Graph.grid(128, 0.02, 1e-3, seed=5),
           "kron12": axbc.Graph.kronecker(12, 16),
           "kron11_H1": axbc.Graph.kronecker(11, 16, H=1)}
    e = axbc.kron_edges(10, 16).astype(np.uint64)
    out["kron10_directed"] = axbc.Graph.from_edges(e, 1024, undirected=False, H=0)
    # 1600 x 3 grid: about 1600 levels, more than the loop's first allocation
    side_edges = []
    W, Hh = 3, 1600
    for y in range(Hh):
        for x in range(W):
            v = y * W + x
            if x + 1 < W:
                side_edges.append((v, v + 1))
            if y + 1 < Hh:
                side_edges.append((v, v + W))
    out["strip"] = axbc.Graph.from_edges(np.array(side_edges, np.uint64), W * Hh, undirected=True, H=0)
    return out


@pytest.fixture(scope="module")
def gs(axbc, orc):
    return graphs(axbc, orc)


@pytest.mark.parametrize("k", [5, 32, 64])
@pytest.mark.parametrize("name", ["grid128", "kron12", "kron11_H1", "kron10_directed", "strip"])
def test_persistent_pass_equals_step_launches_and_oracle(axbc, orc, gs, name, k):
    G = gs[name]
    H = 1 if name.endswith("H1") else 0
    deg = G.deg()
    cand = np.flatnonzero(deg > 0)
    piv = np.random.default_rng(7 + k).choice(cand, size=min(k, len(cand)), replace=False).astype(np.uint32)
    p = np.full(len(piv), 1.0 / G.n)
    res = {}
    for mode in (-1, 1):
        ctx = axbc.Context(G)
        ctx.set_persistent(mode)
        st = ctx.run_batch(piv, p, H)
        res[mode] = (ctx.bc(), ctx.delta(), st)
        ctx.close()
    same_bits(res[1][0], res[-1][0], f"{name}: bc persistent vs step launches")
    same_bits(res[1][1], res[-1][1], f"{name}: last dependencies")
    assert [s["levels"] for s in res[1][2]] == [s["levels"] for s in res[-1][2]]
    assert [s["te"] for s in res[1][2]] == [s["te"] for s in res[-1][2]]
    col, row, reach = G.csc()
    g = orc.CSC(col, row, reach)
    want, _, _ = orc.bc_pivots(g, piv, p, H)
    same_bits(res[1][0], want, f"{name}: bc persistent vs oracle")


def test_persistent_sampled_run_with_bader_stop(axbc, orc, gs):
    G = gs["grid128"]
    ctx = axbc.Context(G)
    ctx.set_persistent(1)
    got = ctx.run_sampled(z=4, nbfs=256, bader_c=1, nchecks=4, H=0, seed=21, W=32)
    col, row, reach = G.csc()
    want = orc.run(orc.CSC(col, row, reach), z=4, nbfs=256, bader_c=1, nchecks=4, H=0, seed=21, W=32)
    assert np.array_equal(got["pivots"], want["pivots"]) and got["stopped"] == want["stopped"]
    same_bits(ctx.bc(), want["bc"], "sampled run, persistent")
    # profiling sees the pass as one launch per batch
    ctx.reset()
    ctx.profile(True)
    ctx.run_sampled(z=0, nbfs=64, bader_c=0, nchecks=1, H=0, seed=3, W=32)
    prof = ctx.profile_read()
    ctx.profile(False)
    assert prof["batch_persistent"][1] >= 2 and prof["batch_fwd_pull"][1] == 0
