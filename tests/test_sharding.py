"""Pivot sharding over two gloo ranks on CPU: each rank computes the oracle's
bc for its share of a pivot list, the shares are summed, and the result equals
the single-process bc (to float rounding: the summation order differs)."""
import os
import socket

import numpy as np
import pytest

GOLDEN = os.path.join(os.path.dirname(__file__), "golden")


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _worker(rank, world, port, out_dir):
    import sys
    sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
    import torch
    import torch.distributed as dist
    import oracle
    from axbc_gb300 import sharding
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    e = np.load(os.path.join(GOLDEN, "kron_s10_ef16.npz"))["edges"].astype(np.uint64)
    g = oracle.pipeline(e, 1024, True, 1)
    piv = np.flatnonzero(g.deg > 0)[::9][:40].astype(np.uint32)
    p = np.full(len(piv), 1.0 / 1024)
    mine = sharding.shard(np.arange(len(piv)), rank, world)
    bc, _, te = oracle.bc_pivots(g, piv[mine], p[mine], 1)
    t = torch.from_numpy(bc.copy())
    sharding.sum_bc(t)
    tmax = sharding.max_time(float(rank + 1))
    te_all = sharding.total(float(te))
    if rank == 0:
        np.save(os.path.join(out_dir, "bc.npy"), t.numpy())
        np.save(os.path.join(out_dir, "meta.npy"), np.array([tmax, te_all]))
    dist.barrier()
    dist.destroy_process_group()


def test_two_rank_pivot_sharding(orc, tmp_path):
    import torch.multiprocessing as mp
    port = _free_port()
    mp.spawn(_worker, args=(2, port, str(tmp_path)), nprocs=2, join=True)
    e = np.load(os.path.join(GOLDEN, "kron_s10_ef16.npz"))["edges"].astype(np.uint64)
    g = orc.pipeline(e, 1024, True, 1)
    piv = np.flatnonzero(g.deg > 0)[::9][:40].astype(np.uint32)
    want, _, te = orc.bc_pivots(g, piv, np.full(len(piv), 1.0 / 1024), 1)
    got = np.load(tmp_path / "bc.npy")
    tmax, te_all = np.load(tmp_path / "meta.npy")
    np.testing.assert_allclose(got, want, rtol=1e-5, atol=1e-3)
    assert tmax == 2.0 and te_all == te


def test_shard_partitions_the_pivots():
    from axbc_gb300 import sharding
    seq = list(range(11))
    parts = [sharding.shard(seq, r, 3) for r in range(3)]
    assert sorted(x for p in parts for x in p) == seq
    assert parts[1] == [1, 4, 7, 10]
