"""The CPU oracle, pinned: drand48 against libc, the graph pipeline against the
reference generator's golden fixtures, Brandes against textbook exact BC."""
import ctypes
import hashlib
import json
import os

import numpy as np
import pytest

GOLDEN = os.path.join(os.path.dirname(__file__), "golden")


def sha(a):
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def test_drand48_matches_libc(orc):
    libc = ctypes.CDLL("libc.so.6")
    libc.lrand48.restype = ctypes.c_long
    libc.srand48.argtypes = [ctypes.c_long]
    for seed in (4343543, 1, 0, 2**31 - 1, -5, 2**40 + 17):
        libc.srand48(seed)
        want = [libc.lrand48() for _ in range(200)]
        assert list(orc.lrand48_seq(seed, 200)) == want


def test_pipeline_matches_golden_summary(orc):
    summ = json.load(open(os.path.join(GOLDEN, "kron_summary.json")))
    e = np.load(os.path.join(GOLDEN, "kron_s10_ef16.npz"))["edges"].astype(np.uint64)
    ent = summ["10"]
    assert len(e) == ent["edges"]
    assert sha(e.astype(np.int64)) == ent["edges_sha256"]
    for H in (0, 1):
        g = orc.pipeline(e, 1024, True, H)
        want = ent[f"H{H}"]
        assert g.m == want["m"]
        assert sha(g.col) == want["col_sha256"]
        assert sha(g.row) == want["row_sha256"]
        assert sha(g.reach) == want["reach_sha256"]
        assert g.rem_ed == want["removed"]


@pytest.mark.parametrize("scale", [12, 14])
def test_reference_generator_pinned(orc, scale):
    """With the reference generator built here (oracle/_ref), regenerate and
    compare against the committed summary (scale 14 matches the published
    config sizes: m=430200, 3744 isolated, max degree 3823)."""
    if not orc.ref_kron_available():
        pytest.skip("reference generator not built on this machine")
    ent = json.load(open(os.path.join(GOLDEN, "kron_summary.json")))[str(scale)]
    e = orc.ref_kron_edges(scale, 16)
    assert sha(e.astype(np.int64)) == ent["edges_sha256"]
    for H in (0, 1):
        g = orc.pipeline(e, 1 << scale, True, H)
        assert sha(g.col) == ent[f"H{H}"]["col_sha256"]
        assert sha(g.row) == ent[f"H{H}"]["row_sha256"]
        assert sha(g.reach) == ent[f"H{H}"]["reach_sha256"]


def _exact_bc(edges, n):
    nx = pytest.importorskip("networkx")
    G = nx.Graph()
    G.add_nodes_from(range(n))
    G.add_edges_from([tuple(map(int, x)) for x in edges if x[0] != x[1]])
    d = nx.betweenness_centrality(G, normalized=False)
    return np.array([d[i] for i in range(n)])


def _full_enumeration(orc, edges, n, order=0):
    g = orc.pipeline(edges, n, True, 0)
    deg = g.deg
    piv = np.array([v for v in range(n) if deg[v] > 0], np.uint32)
    bc, _, _ = orc.bc_pivots(g, piv, np.full(len(piv), 1.0 / n), 0, order)
    # output file convention: bc / 2 / nrounds (src/axbc2d.c:3174)
    return bc.astype(np.float64) / 2.0 / len(piv) * (len(piv) / n)


KNOWN = {
    "path": ([(i, i + 1) for i in range(9)], 10),
    "star": ([(0, i) for i in range(1, 12)], 12),
    "cycle": ([(i, (i + 1) % 11) for i in range(11)], 11),
    "complete": ([(i, j) for i in range(7) for j in range(i + 1, 7)], 7),
    "grid": ([(r * 5 + c, r * 5 + c + 1) for r in range(5) for c in range(4)]
             + [(r * 5 + c, r * 5 + c + 5) for r in range(4) for c in range(5)], 25),
    "two_components": ([(0, 1), (1, 2), (3, 4), (4, 5), (5, 6)], 9),
}


@pytest.mark.parametrize("name", sorted(KNOWN))
@pytest.mark.parametrize("order", [0, 1])
def test_known_answer_graphs(orc, name, order):
    edges, n = KNOWN[name]
    got = _full_enumeration(orc, np.array(edges, np.uint64), n, order)
    want = _exact_bc(edges, n)
    np.testing.assert_allclose(got, want, rtol=1e-5, atol=1e-5)


def test_random_graph_exact_bc(orc):
    rng = np.random.default_rng(3)
    n = 60
    edges = rng.integers(0, n, size=(150, 2)).astype(np.uint64)
    got = _full_enumeration(orc, edges, n)
    want = _exact_bc(edges, n)
    np.testing.assert_allclose(got, want, rtol=1e-4, atol=1e-4)


def test_canonical_and_plain_order_agree(orc):
    e = np.load(os.path.join(GOLDEN, "kron_s10_ef16.npz"))["edges"].astype(np.uint64)
    g = orc.pipeline(e, 1024, True, 1)
    piv = np.flatnonzero(g.deg > 0)[:64].astype(np.uint32)
    p = np.full(len(piv), 1.0 / 1024)
    a, _, _ = orc.bc_pivots(g, piv, p, 1, 0)
    b, _, _ = orc.bc_pivots(g, piv, p, 1, 1)
    np.testing.assert_allclose(a, b, rtol=1e-5, atol=1e-3)


def test_sigma_counts_shortest_paths(orc):
    # 3x3 grid: paths from corner 0 to corner 8 = C(4,2) = 6
    edges = [(r * 3 + c, r * 3 + c + 1) for r in range(3) for c in range(2)] + \
            [(r * 3 + c, r * 3 + c + 3) for r in range(2) for c in range(3)]
    g = orc.pipeline(np.array(edges, np.uint64), 9, True, 0)
    bc, lvl, sigma, delta, st = orc.bc_pivot(g, 0, 1.0 / 9)
    assert sigma[8] == 6 and lvl[8] == 4 and st["nvisited"] == 9 and st["levels"] == 5
    # dependency identity: sum of delta over non-root vertices = sum (d(s,t)-1)
    assert abs(float(delta[1:].sum()) - float((lvl[1:] - 1).sum())) < 1e-4


def test_one_degree_reduction_semantics(orc):
    # hub 0 with leaves 1..3, path 0-4-5, isolated couple 6-7
    edges = np.array([(0, 1), (0, 2), (0, 3), (0, 4), (4, 5), (6, 7)], np.uint64)
    g = orc.pipeline(edges, 8, True, 1)
    assert g.deg[1] == g.deg[2] == g.deg[3] == 0
    assert g.reach[0] == 3 and g.reach[4] == 1
    # the couple: both edges dropped; their reach counts only what the merge consumed
    assert g.deg[6] == g.deg[7] == 0


def test_first_edge_self_loop_is_kept(orc):
    # norm_graph keeps the first sorted edge even when it is a self-loop
    edges = np.array([(0, 0), (0, 1), (1, 2), (2, 2)], np.uint64)
    g = orc.pipeline(edges, 3, True, 0)
    assert 0 in g.row[g.col[0]:g.col[1]]
    assert 2 not in g.row[g.col[2]:g.col[3]]


def test_run_reference_sequence_and_batched(orc):
    e = np.load(os.path.join(GOLDEN, "kron_s10_ef16.npz"))["edges"].astype(np.uint64)
    g = orc.pipeline(e, 1024, True, 0)
    r1 = orc.run(g, z=0, nbfs=100, bader_c=0, nchecks=1, seed=1, W=1)
    r32 = orc.run(g, z=0, nbfs=100, bader_c=0, nchecks=1, seed=1, W=32)
    # uniform sampling does not depend on bc: same pivots, same bc
    assert np.array_equal(r1["pivots"], r32["pivots"])
    assert np.array_equal(r1["bc"], r32["bc"])
    assert r1["nrounds"] + r1["skipped"] + r1["dropped"] == 100
    # the pivot sequence is the drand48 stream: check vertex, discarded draw, pivots
    seq = orc.lrand48_seq(1, 400) % 1025
    deg = g.deg
    draws = list(seq[2:])
    used, piv = set(), []
    for v in draws:
        if len(piv) == r1["nrounds"]:
            break
        if v in used:
            continue
        used.add(v)
        if v < 1024 and deg[v] > 0:
            piv.append(v)
    assert piv == list(r1["pivots"])


@pytest.mark.parametrize("z", [1, 2, 3, 4, 5, 6])
def test_run_heuristics_terminate(orc, z):
    e = np.load(os.path.join(GOLDEN, "kron_s10_ef16.npz"))["edges"].astype(np.uint64)
    g = orc.pipeline(e, 1024, True, 1)
    r = orc.run(g, z=z, nbfs=40, bader_c=1, nchecks=4, H=1, seed=4343543, W=1)
    assert r["nrounds"] > 0
    assert np.all(np.isfinite(r["probs"])) and np.all(r["probs"] > 0)
    assert len(set(r["pivots"].tolist())) == r["nrounds"]


def _bfs_counts(col, row, n, src):
    """Levels and exact (unbounded) shortest-path counts from src over the CSC
    adjacency (column c lists its neighbours), in plain Python integers."""
    lvl = [-1] * n
    sig = [0] * n
    lvl[src] = 0
    sig[src] = 1
    frontier = [src]
    while frontier:
        nxt = []
        for v in frontier:
            for e in range(col[v], col[v + 1]):
                u = int(row[e])
                if lvl[u] == -1:
                    lvl[u] = lvl[v] + 1
                    nxt.append(u)
                if lvl[u] == lvl[v] + 1:
                    sig[u] += sig[v]
        frontier = nxt
    return lvl, sig


@pytest.mark.parametrize("seed", range(6))
def test_oracle_sigma_against_unbounded_counts(orc, seed):
    """Self-consistency: the oracle's uint32 path counts equal exact counts
    reduced mod 2^32, on random graphs (no wrap) and on a grid whose counts
    exceed 2^32 (binomial coefficients)."""
    rng = np.random.default_rng(seed)
    if seed < 4:
        n = int(rng.integers(5, 300))
        e = rng.integers(0, n, size=(int(rng.integers(n, 5 * n)), 2)).astype(np.uint64)
    else:
        side = 40
        n = side * side
        e = np.array([(r * side + c, r * side + c + 1) for r in range(side) for c in range(side - 1)] +
                     [(r * side + c, (r + 1) * side + c) for r in range(side - 1) for c in range(side)],
                     np.uint64)
    g = orc.pipeline(e, n, True, 0)
    srcs = [0] if seed >= 4 else rng.integers(0, n, size=3).tolist()
    for s in srcs:
        lvl, sig = _bfs_counts(g.col, g.row, n, int(s))
        _, olvl, osig, _, _ = orc.bc_pivot(g, int(s), 1.0 / n)
        assert list(olvl) == lvl
        assert [int(x) for x in osig] == [c % (1 << 32) for c in sig]
        if seed >= 4:
            assert max(sig) > (1 << 32)  # the grid's counts wrap


@pytest.mark.parametrize("scale", [10, 12, 14])
def test_restated_generator_matches_golden(orc, scale):
    """oracle/kron.c (the Graph500 generator restated) reproduces the
    reference generator's edge list, order included, at the committed sizes."""
    ent = json.load(open(os.path.join(GOLDEN, "kron_summary.json")))[str(scale)]
    e = orc.kron_edges(scale, 16)
    assert len(e) == ent["edges"]
    assert sha(e) == ent["edges_sha256"]


@pytest.mark.parametrize("scale,edgef,seeds,ini", [
    (6, 16, (23, 24), (.57, .19, .19, .05)),
    (9, 4, (1, 2), (.57, .19, .19, .05)),
    (11, 16, (2**40 + 7, 99), (.45, .15, .15, .25)),
    (8, 32, (0, 0), (.25, .25, .25, .25)),
])
def test_restated_generator_against_reference_build(orc, scale, edgef, seeds, ini):
    """Other sizes, seeds (including high bits) and initiators: the restated
    generator against the reference generator compiled here, when it is."""
    if not orc.ref_kron_available():
        pytest.skip("reference generator not built on this machine")
    want = orc.ref_kron_edges(scale, edgef, *seeds, initiator=ini)
    got = orc.kron_edges(scale, edgef, *seeds, initiator=ini)
    assert np.array_equal(got, want)


def test_restated_generator_stages(orc):
    """Stage 1 is stage 0 under one vertex permutation, each pair stored as
    (min, max); stage 2 reorders stage 1."""
    n = 1 << 12
    s0 = orc.kron_edges(12, 8, stage=0)
    s1 = orc.kron_edges(12, 8, stage=1)
    s2 = orc.kron_edges(12, 8, stage=2)
    assert (s1[:, 0] <= s1[:, 1]).all()
    key = lambda e: np.sort(e[:, 0] * (1 << 32) + e[:, 1])
    assert np.array_equal(key(s1), key(s2))
    # recover the permutation from self-loops and edges to already-mapped
    # vertices, then check every edge against it
    img = -np.ones(n, np.int64)
    loops = s0[:, 0] == s0[:, 1]
    img[s0[loops, 0]] = s1[loops, 0]
    for _ in range(8):
        for (a, b), (c, d) in zip(s0, s1):
            if img[a] >= 0 and img[b] < 0:
                img[b] = d if img[a] == c else c
            elif img[b] >= 0 and img[a] < 0:
                img[a] = d if img[b] == c else c
    ok = (img[s0[:, 0]] >= 0) & (img[s0[:, 1]] >= 0)
    assert ok.mean() > 0.9
    a, b = img[s0[ok, 0]], img[s0[ok, 1]]
    assert np.array_equal(np.minimum(a, b), s1[ok, 0]) and np.array_equal(np.maximum(a, b), s1[ok, 1])
    mapped = img[img >= 0]
    assert len(np.unique(mapped)) == len(mapped)


def _hprefix_py(w):
    """The two-level prefix in plain Python floats (IEEE double, left to right
    at every level): runs of 32 inside blocks of 1024, groups of 32 blocks."""
    n = len(w)
    nb = (n + 1023) // 1024
    local = [0.0] * n
    csum = [0.0] * nb
    G = L = 0.0
    for b in range(nb):
        P = 0.0
        for j in range(b * 1024, min(n, (b + 1) * 1024), 32):
            s = 0.0
            for i in range(j, min(j + 32, (b + 1) * 1024, n)):
                s = s + float(w[i])
                local[i] = P + s
            P = P + s
        if b % 32 == 0:
            L = 0.0
        L = L + P
        csum[b] = G + L
        if b % 32 == 31 or b == nb - 1:
            G = G + L
    return np.array(local), np.array(csum)


@pytest.mark.parametrize("n", [1, 31, 33, 1024, 1025, 5000, 33 * 1024 + 77])
def test_hprefix_definition(orc, n):
    rng = np.random.default_rng(n)
    w = (rng.random(n) * rng.choice([1e-3, 1.0, 1e6], n)).astype(np.float32)
    w[rng.random(n) < 0.2] = 0.0
    local, csum = orc.hprefix(w)
    wl, wc = _hprefix_py(w)
    assert np.array_equal(local, wl) and np.array_equal(csum, wc)
    assert (np.diff(csum) >= 0).all()
    for b in range(len(csum)):
        blk = local[b * 1024:(b + 1) * 1024]
        assert (np.diff(blk) >= 0).all()
    np.testing.assert_allclose(csum[-1], np.sum(w, dtype=np.float64), rtol=1e-12)
    # the search returns the first index whose (exact) prefix reaches r
    for r in rng.random(50) * csum[-1]:
        i, found = orc.hsearch(local, csum, float(r))
        assert found
        b = i // 1024
        full = (csum[b - 1] if b else 0.0) + local[i]
        assert full >= r * (1 - 1e-12)
