"""Seeded random cases through the whole sampled run against the oracle: random
multigraphs (self-loops, duplicates, isolated vertices, hubs), directed or not,
with or without the one-degree reduction, every heuristic, widths 1..64, with and
without Bader's stop."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def same_bits(got, want, what):
    same = (got == want) | (np.isnan(got) & np.isnan(want))
    assert same.all(), f"{what}: {np.count_nonzero(~same)} values differ"


def random_graph(rng):
    n = int(rng.integers(2, 400))
    kind = rng.integers(3)
    if kind == 0:  # uniform
        m = int(rng.integers(0, 6 * n))
        e = rng.integers(0, n, size=(m, 2))
    elif kind == 1:  # hubs: a few vertices take most edges
        m = int(rng.integers(n, 8 * n))
        hubs = rng.integers(0, n, size=max(1, n // 50))
        src = np.where(rng.random(m) < 0.7, rng.choice(hubs, m), rng.integers(0, n, m))
        e = np.stack([src, rng.integers(0, n, m)], 1)
    else:  # chain-like, high diameter
        m = n - 1
        e = np.stack([np.arange(m), np.arange(1, m + 1)], 1)
        extra = rng.integers(0, n, size=(int(rng.integers(0, 5)), 2))
        e = np.concatenate([e, extra])
    return e.astype(np.uint64), n


@pytest.mark.parametrize("case", range(200))
def test_random_sampled_runs(axbc, orc, case):
    rng = np.random.default_rng(1000 + case)
    e, n = random_graph(rng)
    undirected = bool(rng.random() < 0.75)
    H = int(rng.random() < 0.4) if undirected else 0
    g = orc.pipeline(e, n, undirected, H)
    G = axbc.Graph.from_csc(g.col, g.row, g.reach)
    z = int(rng.integers(0, 7))
    W = int(rng.choice([1, 3, 8, 32, 33, 64]))
    nbfs = int(rng.integers(1, min(n, 120) + 1))
    c, x = (0, 1) if rng.random() < 0.6 else (int(rng.integers(1, 3)), int(rng.integers(1, 6)))
    seed = int(rng.integers(1, 1 << 30))
    ctx = axbc.Context(G)
    got = ctx.run_sampled(z=z, nbfs=nbfs, bader_c=c, nchecks=x, H=H, seed=seed, W=W)
    want = orc.run(g, z=z, nbfs=nbfs, bader_c=c, nchecks=x, H=H, seed=seed, W=W)
    what = f"case {case}: n={n} m={g.m} undirected={undirected} H={H} z={z} W={W} N={nbfs} c={c} x={x}"
    assert np.array_equal(got["checks"], want["checks"]), what
    assert np.array_equal(got["pivots"], want["pivots"]), what
    assert np.array_equal(got["probs"], want["probs"], equal_nan=True), what
    for k in ("nrounds", "skipped", "dropped", "ui_end", "te", "stopped"):
        assert got[k] == want[k], (what, k)
    same_bits(ctx.bc(), want["bc"], what)
    same_bits(ctx.delta(), want["delta_last"], what + " (last delta)")


@pytest.mark.parametrize("case", range(40))
def test_random_plain_and_batch_passes(axbc, orc, case):
    """The plain one-pivot pass and the batched pass on random multigraphs,
    with random direction-switch factors, against the oracle's pivot list."""
    rng = np.random.default_rng(5000 + case)
    e, n = random_graph(rng)
    undirected = bool(rng.random() < 0.7)
    H = int(rng.random() < 0.4) if undirected else 0
    g = orc.pipeline(e, n, undirected, H)
    G = axbc.Graph.from_csc(g.col, g.row, g.reach)
    ctx = axbc.Context(G)
    f_plain, f_batch = (float(x) for x in rng.choice([0.0, 0.125, 1.0, 8.0, 1e30], size=2))
    ctx.set_tuning(f_plain, f_batch)
    k = int(rng.integers(1, 65))
    piv = rng.integers(0, n, size=k).astype(np.uint32)
    p = rng.random(k) + 1e-3
    want, dl, te = orc.bc_pivots(g, piv, p, H)
    what = f"case {case}: n={n} m={g.m} undirected={undirected} H={H} k={k} f={f_plain},{f_batch}"
    for v, pp in zip(piv[:6], p[:6]):
        ctx.run_pivot(int(v), float(pp), H)
    want6, _, _ = orc.bc_pivots(g, piv[:6], p[:6], H)
    same_bits(ctx.bc(), want6, what + " (plain)")
    ctx.reset()
    st = ctx.run_batch(piv, p, H)
    assert sum(s["te"] for s in st) == te, what
    same_bits(ctx.bc(), want, what + " (batch)")
    same_bits(ctx.delta(), dl, what + " (batch, last delta)")
