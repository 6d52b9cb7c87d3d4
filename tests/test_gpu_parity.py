"""CUDA path against the oracle, through the C ABI.

Levels and uint32 path counts must match bit for bit.  Dependencies and bc
are compared bit for bit as well: the kernels accumulate every dependency sum
in the oracle's canonical order, and the reference's own tolerance (1e-4
relative) is checked on top as the contract."""
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu
GOLDEN = os.path.join(os.path.dirname(__file__), "golden")
RTOL = 1e-4  # the reference contract for float bc


def golden_edges():
    return np.load(os.path.join(GOLDEN, "kron_s10_ef16.npz"))["edges"].astype(np.uint64)


def assert_float_exact(got, want, what):
    assert got.shape == want.shape
    np.testing.assert_allclose(got, want, rtol=RTOL, atol=1e-6, err_msg=what)
    same = (got == want) | (np.isnan(got) & np.isnan(want))
    assert same.all(), f"{what}: {np.count_nonzero(~same)} values differ in the last bits"


def make(axbc, orc, edges, n, undirected=True, H=0):
    g = orc.pipeline(edges, n, undirected, H)
    G = axbc.Graph.from_csc(g.col, g.row, g.reach)
    return g, G


def pivots_of(g, k, seed=0):
    deg = g.deg
    cand = np.flatnonzero(deg > 0)
    rng = np.random.default_rng(seed)
    hub = int(np.argmax(deg))
    pick = rng.choice(cand, size=min(k, len(cand)), replace=False)
    pick = [hub] + [int(v) for v in pick if v != hub]
    return np.array(pick[:k], np.uint32)


@pytest.mark.parametrize("H", [0, 1])
def test_plain_pivot_bit_exact(axbc, orc, H):
    g, G = make(axbc, orc, golden_edges(), 1024, True, H)
    ctx = axbc.Context(G)
    for v in pivots_of(g, 24, seed=H):
        p = 1.0 / 1024
        ctx.reset()
        st = ctx.run_pivot(v, p, H)
        bc, lvl, sig, dl, ost = orc.bc_pivot(g, int(v), p, H)
        assert np.array_equal(ctx.levels(), lvl)
        assert np.array_equal(ctx.sigma(), sig)
        assert_float_exact(ctx.delta(), dl, f"delta pivot {v}")
        assert_float_exact(ctx.bc(), bc, f"bc pivot {v}")
        assert st["nvisited"] == ost["nvisited"] and st["te"] == ost["te"]
        assert st["levels"] == ost["levels"] and st["all"] == ost["all"]


@pytest.mark.parametrize("factor", [0.0, 1e30])
def test_plain_push_only_and_pull_only(axbc, orc, factor):
    g, G = make(axbc, orc, golden_edges(), 1024)
    ctx = axbc.Context(G)
    ctx.set_tuning(factor, factor)
    piv = pivots_of(g, 12, seed=5)
    p = np.full(len(piv), 1.0 / 1024)
    for v, pp in zip(piv, p):
        ctx.run_pivot(v, pp, 0)
    want, dl, _ = orc.bc_pivots(g, piv, p)
    assert_float_exact(ctx.bc(), want, "bc")
    ctx.reset()
    ctx.run_batch(piv, p, 0)
    assert_float_exact(ctx.bc(), want, "batch bc")


@pytest.mark.parametrize("H", [0, 1])
@pytest.mark.parametrize("k", [1, 7, 32, 33, 64])
def test_batch_bit_exact(axbc, orc, H, k):
    g, G = make(axbc, orc, golden_edges(), 1024, True, H)
    ctx = axbc.Context(G)
    piv = pivots_of(g, k, seed=k + H)
    rng = np.random.default_rng(k)
    p = rng.uniform(0.001, 0.01, size=k)
    stats = ctx.run_batch(piv, p, H)
    want, dlast, te = orc.bc_pivots(g, piv, p, H)
    assert_float_exact(ctx.bc(), want, "bc")
    assert_float_exact(ctx.delta(), dlast, "last delta")
    assert sum(s["te"] for s in stats) == te
    for s in range(k):
        sig, lvl, dl = ctx.batch_source(s)
        _, olvl, osig, odl, ost = orc.bc_pivot(g, int(piv[s]), p[s], H)
        assert np.array_equal(lvl, olvl), f"levels of source {s}"
        assert np.array_equal(sig, osig), f"sigma of source {s}"
        assert_float_exact(dl, odl, f"delta of source {s}")
        assert stats[s]["nvisited"] == ost["nvisited"] and stats[s]["levels"] == ost["levels"]
        assert stats[s]["all"] == ost["all"]


def test_batch_accumulates_across_calls(axbc, orc):
    g, G = make(axbc, orc, golden_edges(), 1024)
    ctx = axbc.Context(G)
    piv = pivots_of(g, 64, seed=9)
    p = np.full(64, 1.0 / 1024)
    ctx.run_batch(piv[:32], p[:32])
    ctx.run_batch(piv[32:], p[32:])
    want, _, _ = orc.bc_pivots(g, piv, p)
    assert_float_exact(ctx.bc(), want, "bc after two batches")
    # widths alternating on one context (64-bit, 32-bit, 64-bit masks): the
    # level masks left by each pass are cleared in the layout it used
    more = pivots_of(g, 110, seed=10)
    pm = np.full(110, 1.0 / 1024)
    ctx.reset()
    ctx.run_batch(more[:50], pm[:50])
    ctx.run_batch(more[50:60], pm[50:60])
    ctx.run_batch(more[60:110], pm[60:110])
    want, _, _ = orc.bc_pivots(g, more, pm)
    assert_float_exact(ctx.bc(), want, "bc after passes of 50, 10 and 50 pivots")


def heavy_graph(seed=1):
    """A hub of degree ~3000 (> one 1024-position span), a second hub, a path."""
    rng = np.random.default_rng(seed)
    n = 4000
    e = [(0, i) for i in range(1, 3000)]
    e += [(1, int(i)) for i in rng.integers(2, n, 2500)]
    e += [tuple(map(int, x)) for x in rng.integers(0, n, size=(6000, 2))]
    e += [(3500 + i, 3501 + i) for i in range(400)]
    return np.array(e, np.uint64), n


@pytest.mark.parametrize("undirected", [True, False])
def test_heavy_vertices_and_directed(axbc, orc, undirected):
    e, n = heavy_graph()
    g, G = make(axbc, orc, e, n, undirected, 0)
    assert G.symmetric == undirected
    ctx = axbc.Context(G)
    piv = pivots_of(g, 64, seed=2)
    piv[0] = 0
    piv[40] = 1
    p = np.full(64, 1.0 / n)
    for factor in (0.0, 1.0, 1e30):
        ctx.set_tuning(factor, factor)
        ctx.reset()
        ctx.run_batch(piv, p, 0)
        want, _, _ = orc.bc_pivots(g, piv, p)
        assert_float_exact(ctx.bc(), want, f"batch bc, push factor {factor}")
        ctx.reset()
        for v, pp in zip(piv[:6], p[:6]):
            ctx.run_pivot(v, pp, 0)
        want6, _, _ = orc.bc_pivots(g, piv[:6], p[:6])
        assert_float_exact(ctx.bc(), want6, f"plain bc, push factor {factor}")


@pytest.mark.parametrize("W", [1, 32, 64])
@pytest.mark.parametrize("z", [0, 1, 2, 3, 4, 5, 6])
def test_sampled_run_matches_oracle(axbc, orc, z, W):
    """W = 64 draws 64 pivots per snapshot and traverses them as two passes."""
    H = 1 if z in (1, 3) else 0
    g, G = make(axbc, orc, golden_edges(), 1024, True, H)
    ctx = axbc.Context(G)
    nbfs = 70 if W == 1 else 150
    got = ctx.run_sampled(z=z, nbfs=nbfs, bader_c=0, nchecks=2, H=H, seed=4343543, W=W)
    want = orc.run(g, z=z, nbfs=nbfs, bader_c=0, nchecks=2, H=H, seed=4343543, W=W)
    assert np.array_equal(got["checks"], want["checks"])
    assert np.array_equal(got["pivots"], want["pivots"])
    assert np.array_equal(got["probs"], want["probs"])
    for k in ("nrounds", "skipped", "dropped", "ui_end", "te", "stopped"):
        assert got[k] == want[k], k
    assert_float_exact(ctx.bc(), want["bc"], "bc")
    assert_float_exact(ctx.delta(), want["delta_last"], "last delta")


@pytest.mark.parametrize("W", [1, 8, 32, 40, 64])
def test_bader_stop_matches_oracle(axbc, orc, W):
    g, G = make(axbc, orc, golden_edges(), 1024)
    ctx = axbc.Context(G)
    for c, x in ((1, 8), (2, 3)):
        got = ctx.run_sampled(z=0, nbfs=1024, bader_c=c, nchecks=x, seed=11, W=W)
        want = orc.run(g, z=0, nbfs=1024, bader_c=c, nchecks=x, seed=11, W=W)
        assert got["stopped"] == want["stopped"]
        assert got["nrounds"] == want["nrounds"] and got["skipped"] == want["skipped"]
        assert np.array_equal(got["pivots"], want["pivots"])
        assert_float_exact(ctx.bc(), want["bc"], "bc")


@pytest.mark.parametrize("W", [16, 64])
def test_bader_first_round_in_growing_passes(axbc, orc, W):
    """A run with Bader's stop traverses its first drawn round in passes of 1,
    1, 2, 4, ... pivots, testing the stop between passes before traversing on:
    the same pivots, counters and bits as the oracle's run at that width, and
    when the stop comes inside the first round, only the passes up to it."""
    G = axbc.Graph.grid(128, 0.02, 1e-3, seed=5)
    col, row, reach = G.csc()
    g = orc.CSC(col, row, reach)
    for z, c, x, seed in ((4, 1, 4, 7), (0, 1, 2, 3), (3, 2, 8, 5)):
        ctx = axbc.Context(G)
        got = ctx.run_sampled(z=z, nbfs=64, bader_c=c, nchecks=x, seed=seed, W=W)
        want = orc.run(g, z=z, nbfs=64, bader_c=c, nchecks=x, seed=seed, W=W)
        what = f"z={z} c={c} x={x} W={W}"
        assert got["stopped"] == want["stopped"], what
        for k in ("nrounds", "skipped", "dropped", "ui_end", "te"):
            assert got[k] == want[k], (what, k)
        assert np.array_equal(got["pivots"], want["pivots"]), what
        assert np.array_equal(got["checks"], want["checks"]), what
        assert_float_exact(ctx.bc(), want["bc"], what)
        assert_float_exact(ctx.delta(), want["delta_last"], what)
        k = int(want["nrounds"])
        if want["stopped"] and k < W:
            # passes cover 1, 2, 4, ... pivots: the one holding pivot k + 1 is the last
            assert got["batches"] <= max(1, int(np.ceil(np.log2(k + 1)))) + 1, (what, k, got["batches"])
        ctx.close()


def test_static_distributions(axbc, orc):
    for H in (0, 1):
        g, G = make(axbc, orc, golden_edges(), 1024, True, H)
        assert np.array_equal(G.degree2(), orc.degree2(g))
        assert np.array_equal(G.sum_deg_neigh(), orc.sum_deg_neigh(g))
        assert np.array_equal(G.lcc(), orc.lcc(g))
    e, n = heavy_graph(4)
    g, G = make(axbc, orc, e, n, False, 0)
    assert np.array_equal(G.lcc(), orc.lcc(g))


def test_compat_entry_points_drive_like_bc_func_mono(axbc, orc):
    """Call the reference-named functions in bc_func_mono's order
    (src/axbc2d.c:1514-1659) and compare with the oracle."""
    import ctypes as C
    for H in (0, 1):
        g = orc.pipeline(golden_edges(), 1024, True, H)
        L = axbc.lib()
        L.axbc_compat_set_n(1024)
        L.initcuda.restype = C.c_size_t
        L.initcuda.argtypes = [C.c_uint64, C.c_void_p, C.c_void_p]
        assert L.initcuda(g.m, g.col.ctypes.data, g.row.ctypes.data) > 0
        L.init_bc_1degree_device(g.reach.ctypes.data_as(C.c_void_p))
        L.scan_col_csc_cuda_mono.restype = C.c_uint32
        L.update_bc_cuda.argtypes = [C.c_uint32, C.c_double, C.c_int, C.c_uint64]
        piv = pivots_of(g, 10, seed=3 + H)
        for v0 in piv:
            v0 = int(v0)
            L.setcuda(C.c_uint64(g.m), None, None, C.c_uint32(int(g.reach[v0])))
            L.set_mlp_cuda(C.c_uint32(v0), 0, 1)
            hF = [0, 0]
            nfrt, level, nvisited = 1, 0, 1
            while True:
                level += 1
                hF.append(0)
                hF[level] = hF[level - 1] + nfrt
                nfrt = L.scan_col_csc_cuda_mono(nfrt, level)
                if not nfrt:
                    break
                nvisited += nfrt
            depth = level - 2
            while True:
                L.scan_frt_csc_cuda_mono(hF[depth], hF[depth + 1] - hF[depth], depth)
                depth -= 1
                if depth <= 0:
                    break
            allv = C.c_uint32(0)
            if H == 1:
                L.pre_update_bc_cuda(None, C.c_uint32(v0), C.byref(allv))
            a = allv.value + int(g.reach[v0])
            L.update_bc_cuda(v0, 1.0 / 1024, 1024, nvisited + a)
        bc = np.empty(1024, np.float32)
        L.get_bc(bc.ctypes.data_as(C.c_void_p))
        want, _, _ = orc.bc_pivots(g, piv, np.full(len(piv), 1.0 / 1024), H)
        assert_float_exact(bc, want, "compat bc")
        deg = np.empty(1024, np.uint32)
        L.get_deg(deg.ctypes.data_as(C.c_void_p))
        assert np.array_equal(deg, g.deg)
        L.fincuda()


def test_generated_rmat_is_a_reference_csc(axbc, orc):
    G = axbc.Graph.rmat(12, 16, seed=23)
    col, row, reach = G.csc()
    n = G.n
    src = np.repeat(np.arange(n, dtype=np.uint64), np.diff(col.astype(np.int64)))
    edges = np.stack([row.astype(np.uint64), src], axis=1)
    g = orc.pipeline(edges, n, False, 0)
    assert np.array_equal(g.col, col) and np.array_equal(g.row, row)
    assert G.symmetric
    ctx = axbc.Context(G)
    piv = pivots_of(g, 32, seed=1)
    p = np.full(32, 1.0 / n)
    ctx.run_batch(piv, p)
    want, _, _ = orc.bc_pivots(g, piv, p)
    assert_float_exact(ctx.bc(), want, "rmat bc")


def test_generated_rmat_H1_matches_host_pipeline(axbc, orc):
    G0 = axbc.Graph.rmat(11, 8, seed=5, H=0)
    G1 = axbc.Graph.rmat(11, 8, seed=5, H=1)
    col, row, _ = G0.csc()
    n = G0.n
    src = np.repeat(np.arange(n, dtype=np.uint64), np.diff(col.astype(np.int64)))
    edges = np.stack([row.astype(np.uint64), src], axis=1)
    g1 = orc.pipeline(edges, n, True, 1)
    c1, r1, rr1 = G1.csc()
    assert np.array_equal(c1, g1.col) and np.array_equal(r1, g1.row)
    assert np.array_equal(rr1, g1.reach)


def test_grid_high_diameter(axbc, orc):
    G = axbc.Graph.grid(48, 0.02, 1e-3, seed=7)
    col, row, reach = G.csc()
    g = orc.CSC(col, row, reach)
    ctx = axbc.Context(G)
    piv = pivots_of(g, 32, seed=4)
    p = np.full(32, 1.0 / G.n)
    ctx.run_batch(piv, p)
    want, _, _ = orc.bc_pivots(g, piv, p)
    assert_float_exact(ctx.bc(), want, "grid bc")
    got = ctx.run_sampled(z=4, nbfs=64, bader_c=1, nchecks=8, seed=7, W=16)
    ref = orc.run(g, z=4, nbfs=64, bader_c=1, nchecks=8, seed=7, W=16)
    assert np.array_equal(got["pivots"], ref["pivots"])
    assert_float_exact(ctx.bc(), ref["bc"], "grid sampled bc")


def test_full_size_properties(axbc):
    """Scale-18 Kronecker: the batched pass equals the plain pass bit for bit,
    and each pivot's dependencies satisfy sum(delta) = sum(depth - 1)."""
    G = axbc.Graph.rmat(18, 16, seed=23)
    deg = G.deg()
    ctx = axbc.Context(G)
    rng = np.random.default_rng(0)
    piv = rng.choice(np.flatnonzero(deg > 0), 32, replace=False).astype(np.uint32)
    p = np.full(32, 1.0 / G.n)
    ctx.run_batch(piv, p)
    bc_batch = ctx.bc()
    for s in (0, 13, 31):
        sig, lvl, dl = ctx.batch_source(s)
        reached = lvl >= 0
        assert lvl[piv[s]] == 0 and sig[piv[s]] == 1
        nonroot = reached & (lvl > 0)
        lhs = float(np.sum(dl[nonroot], dtype=np.float64))
        rhs = float(np.sum(lvl[nonroot] - 1, dtype=np.float64))
        assert abs(lhs - rhs) <= 1e-4 * max(1.0, rhs)
    ctx.reset()
    for v, pp in zip(piv, p):
        ctx.run_pivot(v, pp, 0)
    assert_float_exact(ctx.bc(), bc_batch, "plain vs batched at scale 18")


def test_division_fast_path_is_exact(axbc):
    for seed in (1, 2, 3):
        bad, slow = axbc.selftest_division(1 << 25, seed)
        assert bad == 0
        assert slow < (1 << 25) // 4  # the exact divide is the exception


def _lrand48(x):
    x = (0x5DEECE66D * x + 0xB) & ((1 << 48) - 1)
    return x, x >> 17


@pytest.mark.parametrize("z", [0, 1, 2, 3, 5])
def test_sample_and_stop_primitives_rebuild_the_run(axbc, orc, z):
    """axbc_sample + axbc_run_pivot + axbc_bader_check, driven by the
    reference's round loop (src/axbc2d.c:2729-3156) written out here, give the
    sampled run's pivots, probabilities and bc."""
    H = 1 if z in (1, 3) else 0
    g, G = make(axbc, orc, golden_edges(), 1024, True, H)
    n, nbfs, seed, nchecks = 1024, 40, 77, 3
    ctx = axbc.Context(G)
    x = axbc.srand48(seed)
    checks = []
    for _ in range(nchecks):  # uniform_int(N, 0): lrand48 % (N + 1)
        x, r = _lrand48(x)
        checks.append(r % (n + 1))
    if z == 0:
        x, _ = _lrand48(x)
    used = np.zeros(n + 1, bool)
    deg = g.deg
    piv, probs = [], []
    for ui in range(nbfs):
        while True:
            v, p, x, _ = ctx.sample(z, x, 0, first=not piv)
            if not (v < n and used[v]):
                break
        if v >= n or deg[v] == 0:
            if v < n:
                used[v] = True
            continue
        used[v] = True
        ctx.run_pivot(v, p, H)
        piv.append(v)
        probs.append(p)
    want = orc.run(g, z=z, nbfs=nbfs, bader_c=0, nchecks=nchecks, H=H, seed=seed, W=1)
    assert np.array_equal(np.array(checks, np.uint32), want["checks"])
    assert np.array_equal(np.array(piv, np.uint32), want["pivots"])
    assert np.array_equal(np.array(probs), want["probs"])
    assert_float_exact(ctx.bc(), want["bc"], "bc from the primitives")
    # the stop test on that bc, against the oracle's arithmetic
    bc = want["bc"]
    for c in (0, 1, 2):
        sat = all(float(bc[v]) / 2.0 >= c * n if v < n else 0.0 >= c * n for v in checks)
        assert ctx.bader_check(checks, c) == sat


@pytest.mark.parametrize("z", [0, 1, 2])
def test_static_heuristics_do_not_depend_on_width(axbc, orc, z):
    """With a distribution no pivot changes, the width only groups the same pivot
    sequence into passes: bc bits, pivots and counters are the same at every width
    (the request server relies on this to run static requests 64 wide).  With
    Bader's stop the applied pivots and bc still agree; only the round counter
    depends on where the stopping round ends."""
    H = 1 if z == 1 else 0
    g, G = make(axbc, orc, golden_edges(), 1024, True, H)
    ctx = axbc.Context(G)
    # round limits below the number of vertices the heuristic can draw: past
    # that, every round runs the reference's full rejection loop (N*N draws)
    for c, x, nbfs, seed in ((0, 1, 200, 99), (1, 8, 300, 11)):
        runs = {}
        for W in (1, 8, 32, 64):
            r = ctx.run_sampled(z=z, nbfs=nbfs, bader_c=c, nchecks=x, H=H, seed=seed, W=W)
            runs[W] = (r, ctx.bc())
        r1, bc1 = runs[1]
        for W, (r, bc) in runs.items():
            assert np.array_equal(r["pivots"], r1["pivots"]) and np.array_equal(r["probs"], r1["probs"])
            keys = ("nrounds", "skipped", "dropped", "te", "stopped") + (("ui_end",) if c == 0 else ())
            for k in keys:
                assert r[k] == r1[k], (c, W, k)
            assert np.array_equal(bc.view(np.uint32), bc1.view(np.uint32)), (c, W)
