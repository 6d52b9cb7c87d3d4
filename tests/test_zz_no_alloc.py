"""axbc_bc_pivot_static: the one entry point that allocates no device memory.

It serves callers that cannot call cudaMalloc -- applications whose device
memory belongs to another allocator or budget, loops that must not
synchronise the device through allocation, plug-ins restricted to the buffers
they are handed.  Its scratch is a fixed array inside the library; the caller
passes the graph and the bc output as device buffers.  Here it is called
through the C ABI twice in a row and compared with axbc_run_pivot, the
allocating entry point, within the float tolerance the parity tests use.
This file is collected last so a failure here comes after every other test."""
import ctypes as C
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu
GOLDEN = os.path.join(os.path.dirname(__file__), "golden")


def _dev(torch, arr, dtype):
    return torch.from_numpy(np.ascontiguousarray(arr).view(dtype)).cuda()


@pytest.mark.parametrize("H", [1, 0])
def test_static_pivot_matches_allocating_entry_point(axbc, orc, H):
    torch = pytest.importorskip("torch")
    e = np.load(os.path.join(GOLDEN, "kron_s10_ef16.npz"))["edges"].astype(np.uint64)
    g = orc.pipeline(e, 1024, True, H)
    G = axbc.Graph.from_csc(g.col, g.row, g.reach)
    ctx = axbc.Context(G)
    col = _dev(torch, g.col, np.int32)
    row = _dev(torch, g.row, np.int32)
    reach = _dev(torch, g.reach, np.int32) if H else None
    bc = torch.zeros(1024, dtype=torch.float32, device="cuda")
    torch.cuda.synchronize()
    L = axbc.lib()
    deg = g.deg
    pivots = [int(np.argmax(deg)), int(np.flatnonzero(deg > 0)[17])]
    for v0 in pivots:  # two calls in a row; bc accumulates in both paths
        st = axbc.PivotStats()
        rc = L.axbc_bc_pivot_static(col.data_ptr(), row.data_ptr(),
                                    None if reach is None else reach.data_ptr(),
                                    1024, g.m, v0, 1.0 / 1024, H, bc.data_ptr(), None,
                                    C.byref(st))
        assert rc == 0, L.axbc_last_error().decode()
        want = ctx.run_pivot(v0, 1.0 / 1024, H)
        got = bc.cpu().numpy()
        ref = ctx.bc()
        np.testing.assert_allclose(got, ref, rtol=1e-4, atol=1e-6)
        assert np.array_equal(got, ref)
        assert st.nvisited == want["nvisited"] and st.te == want["te"]
        assert st.levels == want["levels"] and st.all == want["all"]


def test_static_pivot_rejects_oversized_graph(axbc):
    L = axbc.lib()
    dummy = C.c_uint32(0)
    fbuf = C.c_float(0)
    rc = L.axbc_bc_pivot_static(C.addressof(dummy), C.addressof(dummy), None, 1 << 19, 1, 0,
                                1.0, 0, C.addressof(fbuf), None, None)
    assert rc == 5  # AXBC_ERR_RANGE, refused before any device work
    assert b"at most" in L.axbc_last_error()


@pytest.mark.parametrize("case", range(20))
def test_static_pivot_on_random_graphs(axbc, orc, case):
    """Random multigraphs (directed or not, with or without the one-degree
    reduction) against the oracle, several pivots accumulating in one bc."""
    torch = pytest.importorskip("torch")
    rng = np.random.default_rng(500 + case)
    n = int(rng.integers(2, 3000))
    e = rng.integers(0, n, size=(int(rng.integers(0, 8 * n)), 2)).astype(np.uint64)
    undirected = bool(rng.random() < 0.7)
    H = int(rng.random() < 0.4) if undirected else 0
    g = orc.pipeline(e, n, undirected, H)
    col = _dev(torch, g.col, np.int32)
    row = _dev(torch, g.row if g.m else np.zeros(1, np.uint32), np.int32)
    reach = _dev(torch, g.reach, np.int32) if H else None
    bc = torch.zeros(n, dtype=torch.float32, device="cuda")
    torch.cuda.synchronize()
    L = axbc.lib()
    piv = rng.integers(0, n, size=5).astype(np.uint32)
    p = rng.random(5) * 0.5 + 1e-3
    for v0, pp in zip(piv, p):
        st = axbc.PivotStats()
        rc = L.axbc_bc_pivot_static(col.data_ptr(), row.data_ptr(),
                                    None if reach is None else reach.data_ptr(),
                                    n, g.m, int(v0), float(pp), H, bc.data_ptr(), None,
                                    C.byref(st))
        assert rc == 0, L.axbc_last_error().decode()
    want, _, _ = orc.bc_pivots(g, piv, p, H)
    got = bc.cpu().numpy()
    same = (got == want) | (np.isnan(got) & np.isnan(want))
    assert same.all(), f"case {case}: n={n} m={g.m} H={H}: {np.count_nonzero(~same)} differ"
