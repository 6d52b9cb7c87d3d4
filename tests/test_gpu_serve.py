"""Request server: requests batched across one shared multi-source pass get
exactly the bits they get alone (axbc_run_sampled) and from the oracle;
admission by device bytes; release and error paths."""
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu
GOLDEN = os.path.join(os.path.dirname(__file__), "golden")


def golden_edges():
    return np.load(os.path.join(GOLDEN, "kron_s10_ef16.npz"))["edges"].astype(np.uint64)


def same_bits(got, want, what):
    same = (got == want) | (np.isnan(got) & np.isnan(want))
    assert same.all(), f"{what}: {np.count_nonzero(~same)} values differ"


# (z, W, seed, nbfs, bader_c, nchecks): widths add up to more than one pass
MIX = [(0, 8, 1, 60, 0, 1), (3, 16, 2, 50, 0, 2), (4, 4, 3, 40, 0, 1), (1, 8, 4, 48, 0, 1),
       (5, 8, 5, 40, 0, 1), (6, 8, 6, 40, 0, 2), (2, 1, 7, 12, 0, 1), (0, 32, 8, 200, 1, 8),
       (4, 64, 9, 256, 1, 4), (3, 48, 10, 150, 0, 1)]


@pytest.fixture(scope="module")
def golden_graphs(axbc, orc):
    out = {}
    for H in (0, 1):
        g = orc.pipeline(golden_edges(), 1024, True, H)
        out[H] = (g, axbc.Graph.from_csc(g.col, g.row, g.reach))
    return out


def run_alone(axbc, G, H, z, W, seed, nbfs, c, x):
    ctx = axbc.Context(G)
    r = ctx.run_sampled(z=z, nbfs=nbfs, bader_c=c, nchecks=x, H=H, seed=seed, W=W)
    return r, ctx.bc()


def test_mixed_requests_match_alone_and_oracle(axbc, orc, golden_graphs):
    g, G = golden_graphs[0]
    srv = axbc.Server()
    gid = srv.add_graph(G, H=0)
    ids = [srv.submit(gid, z=z, nbfs=nb, bader_c=c, nchecks=x, H=0, seed=sd, W=W)
           for (z, W, sd, nb, c, x) in MIX]
    for rid, (z, W, sd, nb, c, x) in zip(ids, MIX):
        info = srv.wait(rid, timeout_ms=120000)
        assert info["state"] == "done", info["error"]
        bc, piv, pr = srv.result(rid, G.n)
        alone, bc_alone = run_alone(axbc, G, 0, z, W, sd, nb, c, x)
        assert np.array_equal(piv, alone["pivots"]) and np.array_equal(pr, alone["probs"])
        for k in ("nrounds", "skipped", "dropped", "ui_end", "te", "stopped"):
            assert info[k] == alone[k], (z, W, k)
        same_bits(bc, bc_alone, f"z={z} W={W}: server vs alone")
        want = orc.run(g, z=z, nbfs=nb, bader_c=c, nchecks=x, H=0, seed=sd, W=W)
        assert np.array_equal(piv, want["pivots"])
        same_bits(bc, want["bc"], f"z={z} W={W}: server vs oracle")
        srv.release(rid)
    st = srv.stats()
    assert st["completed"] == len(MIX) and st["in_use"] == 0
    # the mix shared passes: fewer passes than the requests' batches alone
    assert st["lanes"] > st["passes"]
    srv.close()


def test_two_graphs_and_one_degree_reduction(axbc, orc, golden_graphs):
    srv = axbc.Server()
    gids = {H: srv.add_graph(golden_graphs[H][1], H=H) for H in (0, 1)}
    jobs = []
    for k in range(6):
        H = k % 2
        z = (1, 3, 0)[k % 3]
        jobs.append((H, z, 8, 100 + k, 40))
    ids = [srv.submit(gids[H], z=z, nbfs=nb, nchecks=1, H=H, seed=sd, W=W)
           for (H, z, W, sd, nb) in jobs]
    for rid, (H, z, W, sd, nb) in zip(ids, jobs):
        info = srv.wait(rid, timeout_ms=120000)
        assert info["state"] == "done", info["error"]
        g, G = golden_graphs[H]
        bc, piv, _ = srv.result(rid, G.n)
        want = orc.run(g, z=z, nbfs=nb, bader_c=0, nchecks=1, H=H, seed=sd, W=W)
        assert np.array_equal(piv, want["pivots"])
        same_bits(bc, want["bc"], f"H={H} z={z}")
    srv.close()


def test_admission_waits_for_budget(axbc, golden_graphs):
    g, G = golden_graphs[0]
    probe = axbc.Server()
    gid = probe.add_graph(G, H=0)
    rid = probe.submit(gid, z=3, nbfs=20, nchecks=1, seed=1, W=4)
    one = probe.wait(rid, timeout_ms=60000)["bytes"]
    probe.close()
    # room for one request at a time: the others queue and run one after another
    srv = axbc.Server(hbm_budget=one + one // 2)
    gid = srv.add_graph(G, H=0)
    ids = [srv.submit(gid, z=3, nbfs=20, nchecks=1, seed=s, W=4) for s in range(1, 5)]
    infos = [srv.wait(r, timeout_ms=120000) for r in ids]
    assert all(i["state"] == "done" for i in infos)
    spans = sorted((i["start_ns"], i["finish_ns"]) for i in infos)
    for (s0, f0), (s1, f1) in zip(spans, spans[1:]):
        assert s1 >= f0  # never two admitted at once
    assert srv.stats()["completed"] == 4
    srv.close()


def test_submit_errors_and_release(axbc, golden_graphs):
    g, G = golden_graphs[0]
    srv = axbc.Server(hbm_budget=1 << 12)  # smaller than any request
    gid = srv.add_graph(G, H=0)
    with pytest.raises(axbc.AxbcError) as e:
        srv.submit(gid, z=0, nbfs=10, seed=1, W=4)
    assert e.value.status == 7  # AXBC_ERR_BUSY
    with pytest.raises(axbc.AxbcError):
        srv.submit(gid, z=0, nbfs=10, seed=1, W=33)  # wider than one pass
    with pytest.raises(axbc.AxbcError):
        srv.submit(gid, z=0, nbfs=10, seed=1, W=4, H=1)  # H differs from the graph's
    with pytest.raises(axbc.AxbcError):
        srv.poll(12345)
    srv.close()
    srv = axbc.Server()
    gid = srv.add_graph(G, H=0)
    rid = srv.submit(gid, z=0, nbfs=30, seed=2, W=8)
    assert srv.wait(rid, timeout_ms=60000)["state"] == "done"
    srv.release(rid)
    with pytest.raises(axbc.AxbcError):
        srv.poll(rid)
    srv.close()


@pytest.mark.parametrize("seed", [1, 2, 3])
def test_random_request_mixes(axbc, orc, seed):
    """Random requests over three random graphs, submitted at once: each result
    equals the oracle's run with the same parameters."""
    rng = np.random.default_rng(seed)
    srv = axbc.Server()
    graphs = []
    for k in range(3):
        n = int(rng.integers(50, 600))
        e = rng.integers(0, n, size=(int(rng.integers(n, 6 * n)), 2)).astype(np.uint64)
        H = int(rng.random() < 0.5)
        g = orc.pipeline(e, n, True, H)
        G = axbc.Graph.from_csc(g.col, g.row, g.reach)
        graphs.append((g, G, H, srv.add_graph(G, H=H)))
    jobs = []
    for _ in range(12):
        gi = int(rng.integers(3))
        g, G, H, gid = graphs[gi]
        z = int(rng.integers(0, 7))
        W = int(rng.choice([1, 4, 8, 16, 32, 64]))
        nbfs = int(rng.integers(1, min(g.n, 150)))
        c, x = (0, 1) if rng.random() < 0.6 else (1, int(rng.integers(1, 5)))
        sd = int(rng.integers(1, 1 << 30))
        jobs.append((gi, z, W, nbfs, c, x, sd, srv.submit(gid, z=z, nbfs=nbfs, bader_c=c, nchecks=x,
                                                            H=H, seed=sd, W=W)))
    for gi, z, W, nbfs, c, x, sd, rid in jobs:
        g, G, H, gid = graphs[gi]
        info = srv.wait(rid, timeout_ms=120000)
        assert info["state"] == "done", info["error"]
        bc, piv, pr = srv.result(rid, G.n)
        want = orc.run(g, z=z, nbfs=nbfs, bader_c=c, nchecks=x, H=H, seed=sd, W=W)
        what = f"graph {gi} z={z} W={W} N={nbfs} c={c} x={x}"
        assert np.array_equal(piv, want["pivots"]), what
        assert np.array_equal(pr, want["probs"], equal_nan=True), what
        for k in ("nrounds", "skipped", "dropped", "ui_end", "te", "stopped"):
            assert info[k] == want[k], (what, k)
        same_bits(bc, want["bc"], what)
    srv.close()


def test_failed_request_releases_its_budget(axbc, golden_graphs):
    """A request whose device state cannot be allocated (failure injected on the
    host) fails with its status; the server goes on serving and its budget
    account returns to zero."""
    g, G = golden_graphs[0]
    srv = axbc.Server()
    gid = srv.add_graph(G, H=0)
    axbc.lib().axbc_inject_alloc_failures(1)
    bad = srv.submit(gid, z=3, nbfs=20, nchecks=1, seed=1, W=4)
    info = srv.wait(bad, timeout_ms=60000)
    axbc.lib().axbc_inject_alloc_failures(0)
    assert info["state"] == "failed" and info["status"] == 3, info
    assert "injected" in info["error"]
    good = srv.submit(gid, z=3, nbfs=20, nchecks=1, seed=1, W=4)
    assert srv.wait(good, timeout_ms=60000)["state"] == "done"
    st = srv.stats()
    assert st["in_use"] == 0 and st["completed"] == 1
    srv.close()
    # a context whose buffers cannot be allocated reports it; the next one works
    axbc.lib().axbc_inject_alloc_failures(1)
    with pytest.raises(axbc.AxbcError) as e:
        axbc.Context(G)
    axbc.lib().axbc_inject_alloc_failures(0)
    assert e.value.status == 3
    ctx = axbc.Context(G)
    ctx.run_batch(np.array([1, 2], np.uint32), np.array([0.5, 0.5]))
