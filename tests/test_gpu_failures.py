"""Device-allocation failures injected on the host, one allocation at a time,
into the context's lazily allocated state: the failing call reports
AXBC_ERR_NOMEM, the same context then runs the call to the right result, and
closing it returns every device byte."""
import gc
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu
GOLDEN = os.path.join(os.path.dirname(__file__), "golden")


@pytest.fixture(scope="module")
def golden(axbc, orc):
    e = np.load(os.path.join(GOLDEN, "kron_s10_ef16.npz"))["edges"].astype(np.uint64)
    g = orc.pipeline(e, 1024, True, 0)
    return g, axbc.Graph.from_csc(g.col, g.row, g.reach)


def same_bits(got, want, what):
    same = (got == want) | (np.isnan(got) & np.isnan(want))
    assert same.all(), f"{what}: {np.count_nonzero(~same)} values differ"


RUNS = {
    "sampled z=3 W=32": lambda ctx: ctx.run_sampled(z=3, nbfs=64, bader_c=0, nchecks=1, seed=3, W=32),
    "sampled z=2 W=64 Bader": lambda ctx: ctx.run_sampled(z=2, nbfs=96, bader_c=1, nchecks=4, seed=4, W=64),
    "batch": lambda ctx: ctx.run_batch(np.arange(1, 33, dtype=np.uint32), np.full(32, 1 / 1024.0)),
    "plain": lambda ctx: ctx.run_pivot(5, 1 / 1024.0, 0),
}


@pytest.mark.parametrize("name", list(RUNS))
def test_failed_allocation_leaves_a_usable_context(axbc, golden, name):
    g, G = golden
    run = RUNS[name]
    ref = axbc.Context(G)
    run(ref)
    want = ref.bc()
    ref.close()
    # objects of earlier tests freed by the collector would move the counter
    gc.collect()
    gc.disable()
    try:
        _failure_loop(axbc, G, run, want, name)
    finally:
        gc.enable()


def _failure_loop(axbc, G, run, want, name):
    L = axbc.lib()
    base = L.axbc_device_bytes_live()
    failures = 0
    for k in range(60):
        ctx = axbc.Context(G)
        L.axbc_inject_alloc_failure_after(k)
        try:
            run(ctx)
            ok = True
        except axbc.AxbcError as ex:
            assert ex.status == 3, ex
            ok = False
        finally:
            L.axbc_inject_alloc_failure_after(-1)
        if not ok:
            failures += 1
            ctx.reset()
            run(ctx)  # the same context, now with room
        same_bits(ctx.bc(), want, f"{name}, failure after {k} allocations")
        ctx.close()
        assert L.axbc_device_bytes_live() == base, f"{name}: leak after failing allocation {k}"
        if ok:
            break
    assert failures >= 1


def test_server_recovers_from_each_failed_allocation(axbc, golden):
    """A device allocation made to fail at each point of adding a graph (its
    static sampling distributions included) and serving a request (the
    server's worker thread included): the call or the request fails with
    AXBC_ERR_NOMEM, a second request on the same server gets the exact result,
    and closing the server and the graph frees every byte."""
    g, G = golden
    prm = dict(z=3, nbfs=48, bader_c=0, nchecks=1, H=0, seed=9, W=8)
    ref = axbc.Context(G)
    ref.run_sampled(**prm)
    want = ref.bc()
    ref.close()
    gc.collect()
    gc.disable()
    try:
        L = axbc.lib()
        base = L.axbc_device_bytes_live()
        for k in range(60):
            # a fresh graph each time: adding it builds its distributions
            Gk = axbc.Graph.from_csc(g.col, g.row, g.reach)
            srv = axbc.Server()
            L.axbc_inject_alloc_failure_after(k)
            failed = False
            try:
                gid = srv.add_graph(Gk, H=0)
                info = srv.wait(srv.submit(gid, **prm), timeout_ms=60000)
                if info["state"] == "failed":
                    assert info["status"] == 3, info
                    failed = True
                else:
                    assert info["state"] == "done", info
            except axbc.AxbcError as ex:
                assert ex.status == 3, ex
                failed = True
                gid = None
            finally:
                L.axbc_inject_alloc_failure_after(-1)
            if gid is None:
                gid = srv.add_graph(Gk, H=0)
            rid = srv.submit(gid, **prm)
            info = srv.wait(rid, timeout_ms=60000)
            assert info["state"] == "done", (k, info)
            bc, _, _ = srv.result(rid, Gk.n)
            same_bits(bc, want, f"server, failure after {k} allocations")
            srv.close()
            Gk.close()
            assert L.axbc_device_bytes_live() == base, f"server: leak after failing allocation {k}"
            if not failed:
                break
    finally:
        gc.enable()
