#!/usr/bin/env python3
"""Benchmark: BC traversed-edges/s (forward + backward) on GB300, and the
serving configuration's p50/p99 request latency.

Workload (the headline configuration): the Graph500 generator's Kronecker graph
at scale 23, edgefactor 16 (seeds 23/24), undirected, heuristic 3 (bc-based
dynamic sampling), 1024 pivots per step in batches of 32, Bader test off.  One
step is one sampled BC run of 1024 pivots: device sampling, the batched
forward/backward passes and the bc updates.  TE per pivot = 2 * degree sum of
the vertices it reaches (Graph500 counting).  After the headline timing a
serving phase runs the request server under Poisson arrivals (resident graphs:
Kronecker scales 16/18/20/22 and a 1024^2 grid) and reports p50/p99 latency.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference]

--impl reference times the oracle (oracle/, a C restatement of the reference
path; the reference needs MPI and a Kepler-era toolchain and is not run on the
GPU machine) on the host cores with OpenMP, on a bounded pivot sample of the same
graph and pivot list.

Input generation (device generator + CSC build) is set-up and is not timed.
The graph (~1.1 GB of adjacency) is larger than L2, so no L2 flush is needed.
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--scale", type=int, default=23)
    ap.add_argument("--graph", default="kron",
                    help="headline graph: kron (Graph500 generator at --scale) or grid:SIDE "
                         "(SIDE x SIDE grid, 2%% of edges dropped, 0.01%% long-range, seed 7)")
    ap.add_argument("--edgefactor", type=int, default=16)
    ap.add_argument("--pivots", type=int, default=1024, help="pivots per step")
    ap.add_argument("--width", type=int, default=32, help="batch width (the headline configuration: batches of 32)")
    ap.add_argument("--z", type=int, default=3, help="sampling heuristic")
    ap.add_argument("--cpu-seconds", type=float, default=15.0,
                    help="target CPU time of the oracle baseline sample")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--skip-e2e", action="store_true", help="profiling runs: no e2e pass")
    ap.add_argument("--skip-plain", action="store_true", help="profiling runs: no plain pass")
    ap.add_argument("--skip-serving", action="store_true", help="no serving phase after the headline")
    ap.add_argument("--skip-count", action="store_true", help="no counted step (roofline bytes)")
    ap.add_argument("--skip-wide", action="store_true", help="no width-64 leg after the headline")
    ap.add_argument("--persistent", default="auto", choices=["auto", "on", "off"],
                    help="level loop: one cooperative launch per pass (on), per-level launches (off), "
                         "or the library's rule (auto: narrow batches on deep graphs)")
    ap.add_argument("--workload", default="headline",
                    choices=["headline", "serving", "config1", "config2", "config3"],
                    help="serving: the request server on resident graphs (p50/p99 latency); "
                         "config1..3: the other benchmark configurations, one sampled run "
                         "per step, with the oracle on the host beside it")
    ap.add_argument("--requests", type=int, default=48, help="serving: requests submitted")
    ap.add_argument("--rate", type=float, default=2.0, help="serving: mean arrivals per second")
    ap.add_argument("--push-factor", type=float, default=None,
                    help="fixed batched push/pull factor instead of autotuning (profiling runs)")
    return ap.parse_args()


class ClockSampler:
    """nvidia-smi clock / throttle samples during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = str(index)
        self.rows = []
        self.proc = None

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except OSError:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            parts = [x.strip() for x in line.split(",")]
            if len(parts) >= 9 and parts[0] == self.index:
                self.rows.append(parts)

    def stop(self):
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        self.thread.join(timeout=2)
        sm = sorted(float(r[1]) for r in self.rows if r[1].replace(".", "").isdigit())
        mx = [float(r[2]) for r in self.rows if r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = set()
        for r in self.rows:
            for i, nm in enumerate(names):
                if r[5 + i].lower() == "active":
                    reasons.add(nm)
        return {"sm_mhz": sm[len(sm) // 2] if sm else None,
                "sm_max_mhz": max(mx) if mx else None,
                "samples": len(self.rows), "reasons": sorted(reasons)}


def peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            pk = json.load(f)
        return float(pk["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def kernel_source_digest():
    """SHA-256 of the traversal kernels' source file with its comments and blank
    lines taken out: a DRAM figure taken from an ncu capture of other kernel code
    is stale (an edit of comments alone keeps it)."""
    import hashlib
    import re
    with open(os.path.join(ROOT, "axbc_gb300", "csrc", "batch.cu")) as f:
        src = f.read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    src = re.sub(r"//[^\n]*", "", src)
    code = "\n".join(line.rstrip() for line in src.splitlines() if line.strip())
    return hashlib.sha256(code.encode()).hexdigest()


def traffic_for(kernel, graph_key, must_per_launch, words):
    """(per-launch DRAM bytes of `kernel`, note) from the committed ncu capture in
    profiles/traffic.json.  The capture is of a smaller graph of the same family
    (a few GB on the device); it records, per traversal kernel, DRAM bytes per
    byte the kernel must move (its counting build over the same steps), and the
    figure here is that ratio times this launch's must-move bytes.  None when
    there is no capture for this graph family and kernel, when it was taken of
    other kernel source, or without a must-move count.  `words`: mask words per
    vertex of the passes (1 up to 32 pivots, 2 up to 64), the kernel build the
    capture must be of."""
    path = os.path.join(ROOT, "profiles", "traffic.json")
    try:
        with open(path) as f:
            t = json.load(f)
    except Exception:
        return None, "no ncu capture committed"
    family = graph_key.split("-")[0]
    ent = t.get(family, {})
    k = ent.get("kernels", {}).get(f"{kernel}<{words}>")
    if k is None or "dram_per_must_move_byte" not in k:
        return None, f"no ncu capture of {kernel}<{words}> on a {family} graph"
    if ent.get("kernel_source_sha256") != kernel_source_digest():
        return None, "the committed ncu capture is of other kernel source (stale)"
    if not must_per_launch:
        return None, "no must-move count in this run"
    r = float(k["dram_per_must_move_byte"])
    return r * must_per_launch, (f"ncu capture of {kernel}<{words}> on {ent.get('graph')} at "
                                 f"{ent.get('commit', '?')}: "
                                 f"{r:.3f} DRAM bytes per must-move byte, times this launch's "
                                 f"must-move bytes")


class _DeviceArray:
    """A float32 device vector owned by the library, seen through
    __cuda_array_interface__ (no copy)."""

    def __init__(self, ptr, n):
        self.__cuda_array_interface__ = {"shape": (n,), "typestr": "<f4", "data": (ptr, False),
                                         "version": 3}


def cpu_threads():
    try:
        return len(os.sched_getaffinity(0))
    except Exception:
        return os.cpu_count() or 1


def oracle_sample(g_csc, pivots, probs, seconds, threads):
    """Time the oracle (OpenMP over pivots) on a bounded pivot sample."""
    import numpy as np
    import oracle
    oracle.build()
    g = oracle.CSC(*g_csc)
    # size the sample: one pivot per thread first, then scale to the budget
    k0 = min(len(pivots), threads)
    t0 = time.perf_counter()
    _, te0 = oracle.bc_pivots_omp(g, pivots[:k0], probs[:k0], 0, threads)
    dt0 = time.perf_counter() - t0
    k = k0
    if dt0 < seconds:
        k = int(min(len(pivots), max(k0, k0 * (seconds / max(dt0, 1e-3)))))
        k = max(threads, (k // threads) * threads) if k >= threads else k
    if k == k0:
        return te0 / dt0, k0, dt0
    t0 = time.perf_counter()
    _, te = oracle.bc_pivots_omp(g, pivots[:k], probs[:k], 0, threads)
    dt = time.perf_counter() - t0
    return te / dt, k, dt


def oracle_single(g_csc, pivots, probs):
    """The oracle on one thread over a few pivots: (TE/s, seconds)."""
    import oracle
    g = oracle.CSC(*g_csc)
    t0 = time.perf_counter()
    _, _, te = oracle.bc_pivots(g, pivots, probs, 0)
    dt = time.perf_counter() - t0
    return te / dt, dt


# The other benchmark configurations: graph, heuristic, budget, stop rule, width
# (None: from the autotuner), one-degree reduction.
CONFIGS = {
    "config1": dict(graph=("kron", 14), H=0, z=0, nbfs=256, c=0, x=1, seed=1, W=32,
                    desc="Kronecker scale 14 (Graph500 generator, seeds 23/24), -H 0 -z 0 -N 256 -c 0"),
    "config2": dict(graph=("kron", 20), H=1, z=1, nbfs=4096, c=0, x=1, seed=1, W=64,
                    desc="Kronecker scale 20, -H 1 -z 1 -N 4096 -c 0, width 64"),
    "config3": dict(graph=("grid", 2048), H=0, z=4, nbfs=2048, c=1, x=8, seed=1, W=None,
                    desc="2048x2048 grid (2% edges dropped, seed 7; 0.01% long-range), "
                         "-z 4 -N 2048 -c 1 -x 8, width from the autotuner"),
}


# --persistent: the library's level-loop modes (axbc_set_persistent)
PERSIST_MODES = {"off": -1, "auto": 0, "on": 1}


def config_bench(args):
    """One of the other benchmark configurations: each step is one whole
    sampled run on the GPU (CUDA events on the context's stream); the oracle
    times the same run's pivots on the host (OpenMP over pivots), all of them
    when that fits the CPU budget, else a sample scaled per pivot."""
    import numpy as np
    import torch
    import axbc_gb300 as ax
    cf = CONFIGS[args.workload]
    torch.cuda.init()
    kind, size = cf["graph"]
    t_graph = time.perf_counter()
    G = ax.Graph.kronecker(size, 16, 23, 24, H=cf["H"]) if kind == "kron" else \
        ax.Graph.grid(size, 0.02, 1e-4, seed=7)
    build_s = time.perf_counter() - t_graph
    stream = torch.cuda.Stream()
    ctx = ax.Context(G, stream=stream.cuda_stream)
    ctx.set_persistent(PERSIST_MODES[args.persistent])
    W = cf["W"]
    if W is None:
        deg = G.deg()
        rng = np.random.default_rng(1234)
        trial = rng.choice(np.flatnonzero(deg > 0), size=64, replace=False).astype(np.uint32)
        W = int(ctx.autotune(trial)["batch_width"])

    def run():
        ctx.reset()
        return ctx.run_sampled(z=cf["z"], nbfs=cf["nbfs"], bader_c=cf["c"], nchecks=cf["x"], H=cf["H"],
                               seed=cf["seed"], W=W)

    for _ in range(max(1, args.warmup)):
        r = run()
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    ev0.record(stream)
    te = 0
    for _ in range(args.steps):
        r = run()
        te += r["te"]
    ev1.record(stream)
    torch.cuda.synchronize()
    t = ev0.elapsed_time(ev1) / 1000.0
    out = {"metric": "BC traversed-edges/s (fwd+bwd)", "value": te / t, "unit": "TE/s", "n_gpus": 1,
           "steps": args.steps, "warmup": args.warmup, "ms_per_step": t * 1000 / args.steps,
           "higher_is_better": True, "impl": "gb300", "workload": args.workload,
           "config": {"workload": cf["desc"], "batch_width": W, "graph_build_s": round(build_s, 3),
                      "n": G.n, "m": G.m, "level_loop": args.persistent},
           "rounds": int(r["nrounds"]), "stopped": bool(r["stopped"]), "te_per_run": int(r["te"])}
    if not args.no_cpu_baseline:
        col, row, reach = G.csc()
        piv, pr = r["pivots"], r["probs"]
        threads = cpu_threads()
        import oracle
        oracle.build()
        g = oracle.CSC(col, row, reach)
        # the whole pivot list when a first chunk says it fits the budget
        k0 = min(len(piv), threads)
        t0 = time.perf_counter()
        _, te0 = oracle.bc_pivots_omp(g, piv[:k0], pr[:k0], cf["H"], threads)
        dt0 = time.perf_counter() - t0
        per_pivot = dt0 / max(k0, 1)
        if per_pivot * len(piv) <= args.cpu_seconds * 4:
            t0 = time.perf_counter()
            _, te_all = oracle.bc_pivots_omp(g, piv, pr, cf["H"], threads)
            dt = time.perf_counter() - t0
            out["cpu_baseline"] = {"value": te_all / dt, "unit": "TE/s", "cores": threads, "kind": "port",
                                   "sample": f"all {len(piv)} pivots of the run in {dt:.1f} s"}
        else:
            out["cpu_baseline"] = {"value": te0 / dt0, "unit": "TE/s", "cores": threads, "kind": "port",
                                   "sample": f"{k0} of the run's {len(piv)} pivots in {dt0:.1f} s "
                                             f"(whole run extrapolated: {per_pivot * len(piv):.0f} s)"}
    print(json.dumps(out), flush=True)


def serve_bench(args, emit=True):
    """The request server under Poisson arrivals (seed 11) over resident graphs:
    Kronecker scales 16, 18, 20, 22 (edgefactor 16) and a 1024x1024 grid.  Each
    request picks a graph and a heuristic -z 0..5 uniformly, width 8, and either
    a budget of -N pivots log-uniform in [64, 2048] or Bader's adaptive stop
    (-c 1, -x uniform in 4..16, at most 2048 pivots).  Latency = finish - submit
    on the server's steady clock; throughput = traversed edges of all requests
    over the span from the first submit to the last finish."""
    import numpy as np
    import torch
    import axbc_gb300 as ax
    torch.cuda.init()
    graphs = [("kronecker-s16", ax.Graph.kronecker(16, 16)),
              ("kronecker-s18", ax.Graph.kronecker(18, 16)),
              ("kronecker-s20", ax.Graph.kronecker(20, 16)),
              ("kronecker-s22", ax.Graph.kronecker(22, 16)),
              ("grid-1024", ax.Graph.grid(1024, 0.02, 1e-4, seed=7))]
    srv = ax.Server()
    gids = [srv.add_graph(G, H=0) for _, G in graphs]
    rng = np.random.default_rng(11)
    jobs = []
    t = 0.0
    for i in range(args.requests):
        t += rng.exponential(1.0 / args.rate)
        gi = int(rng.integers(len(graphs)))
        z = int(rng.integers(0, 6))
        if rng.random() < 0.5:
            nbfs = int(round(np.exp(rng.uniform(np.log(64), np.log(2048)))))
            c, x = 0, 1
        else:
            nbfs, c, x = 2048, 1, int(rng.integers(4, 17))
        jobs.append((t, gi, z, nbfs, c, x, 1000 + i))
    clocks = ClockSampler(0)
    clocks.start()
    t0 = time.perf_counter()
    ids = []
    for (ta, gi, z, nbfs, c, x, seed) in jobs:
        d = ta - (time.perf_counter() - t0)
        if d > 0:
            time.sleep(d)
        ids.append(srv.submit(gids[gi], z=z, nbfs=nbfs, bader_c=c, nchecks=x, H=0, seed=seed, W=8))
    infos = [srv.wait(r) for r in ids]
    clk = clocks.stop()
    st = srv.stats()
    failed = [i["error"] for i in infos if i["state"] != "done"]
    lat = np.array([(i["finish_ns"] - i["submit_ns"]) / 1e9 for i in infos])
    wait = np.array([(i["start_ns"] - i["submit_ns"]) / 1e9 for i in infos])
    span = (max(i["finish_ns"] for i in infos) - min(i["submit_ns"] for i in infos)) / 1e9
    te = sum(i["te"] for i in infos)
    per_graph = {}
    for (ta, gi, *_), i, l in zip(jobs, infos, lat):
        per_graph.setdefault(graphs[gi][0], []).append(float(l))
    out = {"metric": "serving p99 request latency", "value": float(np.percentile(lat, 99)),
           "unit": "s", "n_gpus": 1, "higher_is_better": False, "impl": "gb300",
           "p50_s": float(np.percentile(lat, 50)), "p99_s": float(np.percentile(lat, 99)),
           "mean_queue_wait_s": float(wait.mean()), "requests": len(infos),
           "failed": len(failed), "throughput_te_per_s": te / span, "requests_per_s": len(infos) / span,
           "span_s": span, "passes": st["passes"], "lanes_per_pass": st["lanes"] / max(1, st["passes"]),
           "p50_by_graph_s": {k: float(np.median(v)) for k, v in per_graph.items()},
           "worker_by_graph": {graphs[i][0]: srv.graph_stats(g) for i, g in enumerate(gids)},
           "slowest": [{"graph": graphs[jobs[k][1]][0], "z": jobs[k][2], "N": jobs[k][3], "c": jobs[k][4],
                        "x": jobs[k][5], "latency_s": round(float(lat[k]), 3),
                        "queue_wait_s": round(float(wait[k]), 3), "rounds": int(infos[k]["nrounds"]),
                        "stopped": bool(infos[k]["stopped"])}
                       for k in np.argsort(-lat)[:3]],
           "dtype": "u32 path counts, f32 dependencies", "data": "synthetic (Graph500 generator, seeds 23/24, on the device; grid)",
           "config": {"workload": "serving: resident kronecker s16/s18/s20/s22 ef16 + grid 1024^2; "
                                  "Poisson arrivals (seed 11); -z 0..5; width 8; -N log-uniform "
                                  "64-2048 or -c 1 -x 4..16",
                      "rate_per_s": args.rate, "requests": args.requests,
                      "hbm_budget_bytes": st["budget"]},
           "clocks": clk}
    if failed:
        out["errors"] = failed[:3]
    srv.close()
    for _, G in graphs:
        G.close()
    if emit:
        print(json.dumps(out), flush=True)
    return out


def main():
    args = parse()
    if args.workload == "serving":
        return serve_bench(args)
    if args.workload in CONFIGS:
        return config_bench(args)
    from axbc_gb300 import sharding
    rank, world, local = sharding.env()
    import numpy as np

    workload = (f"kronecker-s{args.scale}-ef{args.edgefactor} undirected, -z {args.z} "
                f"-N {args.pivots} -c 0, batch width {args.width}")
    metric = "BC traversed-edges/s (fwd+bwd)"
    config = {"workload": workload, "scale": args.scale, "edgefactor": args.edgefactor,
              "pivots_per_step": args.pivots, "batch_width": args.width,
              "heuristic": args.z, "bader_c": 0,
              "l2": "inputs larger than L2 (adjacency ~4*m bytes, no flush)",
              "parallelism": f"pivot-sharded replicas x{world}"}

    import torch
    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    import axbc_gb300 as ax
    ax.lib()

    # the reference's own input: the Graph500 generator with gen_graph's seeds
    # (23, 24) and initiator, generated and built on the device (set-up, untimed)
    t_graph = time.perf_counter()
    if args.graph == "kron":
        G = ax.Graph.kronecker(args.scale, args.edgefactor, 23, 24)
        gen = "Graph500 (seeds 23/24, initiator .57/.19/.19/.05)"
    else:
        side = int(args.graph.split(":")[1])
        G = ax.Graph.grid(side, 0.02, 1e-4, seed=7)
        gen = f"{side}x{side} grid, 2% of edges dropped, 0.01% long-range edges, seed 7"
        config["workload"] = workload.replace(f"kronecker-s{args.scale}-ef{args.edgefactor}", f"grid-{side}")
    config["graph"] = {"generator": gen, "n": G.n, "m": G.m,
                       "build_s": round(time.perf_counter() - t_graph, 3)}
    stream = torch.cuda.Stream()
    ctx = ax.Context(G, stream=stream.cuda_stream)
    ctx.set_persistent(PERSIST_MODES[args.persistent])
    config["level_loop"] = args.persistent

    def step(seed):
        return ctx.run_sampled(z=args.z, nbfs=args.pivots, bader_c=0, nchecks=1, H=0, seed=seed,
                               W=args.width)

    seed = sharding.rank_seed(4343543, rank)
    # autotune the direction-switch factors on 64 trial pivots (set-up, untimed)
    deg = G.deg()
    rng = np.random.default_rng(1234)
    trial = rng.choice(np.flatnonzero(deg > 0), size=64, replace=False).astype(np.uint32)
    tuning = None
    if args.impl == "gb300" and args.push_factor is not None:
        ctx.set_tuning(32.0, args.push_factor)
        tuning = {"push_factor_single": 32.0, "push_factor_batch": args.push_factor,
                  "batch_width": args.width, "fixed": True}
    elif args.impl == "gb300":
        tuning = ctx.autotune(trial)
    if tuning:
        config["tuning"] = {k: (round(v, 4) if isinstance(v, float) else v)
                            for k, v in tuning.items() if "factor" in k or k == "batch_width"}

    if args.impl == "reference":
        if rank != 0:
            return
        # the graph and the pivot list of the gb300 arm; the oracle is timed
        first = step(seed)
        csc = G.csc()
        piv, pr = first["pivots"], first["probs"]
        threads = cpu_threads()
        vals = []
        for _ in range(args.warmup):
            oracle_sample(csc, piv, pr, args.cpu_seconds / 3, threads)
        t_all = time.perf_counter()
        ks = []
        for _ in range(args.steps):
            v, k, dt = oracle_sample(csc, piv, pr, args.cpu_seconds / 3, threads)
            vals.append(v)
            ks.append(k)
        wall = time.perf_counter() - t_all
        val = float(np.mean(vals))
        out = {"metric": metric, "value": val, "unit": "TE/s", "n_gpus": 1, "steps": args.steps,
               "warmup": args.warmup, "ms_per_step": wall * 1000 / max(args.steps, 1),
               "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
               "dtype": "u32 path counts, f32 dependencies/bc",
               "data": "synthetic: the Graph500 generator's graph (seeds 23/24), generated on the device",
               "config": config, "impl": "reference",
               "cpu_baseline": {"value": val, "unit": "TE/s", "cores": threads, "kind": "port",
                                "sample": f"{ks[0]} pivots of the step's pivot list per step, "
                                          "OpenMP over pivots (oracle/ C restatement; the "
                                          "reference program needs MPI and a GPU, and its "
                                          "one-rank host build exists only where its "
                                          "sources are)"},
               "e2e": {"value": val, "unit": "TE/s", "h2d_bytes_per_step": 0,
                       "d2h_bytes_per_step": 0}}
        print(json.dumps(out), flush=True)
        return

    # ---------------------------------------------------------------- gb300
    # warm-up steps run profiled too, so the CUDA events the timed region's
    # profiling records are created here, not inside the timed region
    ctx.profile(True)
    for _ in range(args.warmup):
        step(seed)
    torch.cuda.synchronize()
    if world > 1:
        dist.barrier()
    clocks = ClockSampler(os.environ.get("CUDA_VISIBLE_DEVICES", str(local)).split(",")[local]
                          if "CUDA_VISIBLE_DEVICES" in os.environ else local)
    clocks.start()
    ctx.profile(True)
    l0 = ctx.launches
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    ev0.record(stream)
    te = 0
    last = None
    for _ in range(args.steps):
        last = step(seed)
        te += last["te"]
    if world > 1:
        # the one exchange of the sharded path: sum the ranks' bc (a device copy
        # of the context's bc, reduced on the same stream)
        bc_t = torch.empty(G.n, dtype=torch.float32, device="cuda")
        with torch.cuda.stream(stream):
            bc_t.copy_(torch.as_tensor(_DeviceArray(ctx.bc_device_ptr(), G.n), device="cuda"))
            sharding.sum_bc(bc_t)
    ev1.record(stream)
    torch.cuda.synchronize()
    launches = ctx.launches - l0
    prof = ctx.profile_read()
    ctx.profile(False)
    clk = clocks.stop()
    t = ev0.elapsed_time(ev1) / 1000.0
    t = sharding.max_time(t, device="cuda")
    te_all = sharding.total(float(te), device="cuda")
    value = te_all / t

    # ---- roofline of the dominant kernel kind (largest live CUDA-event time)
    peak, peak_kind = peaks()
    kind = max(prof, key=lambda k: prof[k][0])
    ms, cnt, model_by = prof[kind]
    avg_s = ms / max(cnt, 1) / 1000.0
    kernel = ax.PROF_KERNELS[kind]
    graph_key = (f"kronecker-s{args.scale}-ef{args.edgefactor}" if args.graph == "kron"
                 else f"grid-{args.graph.split(':')[1]}")
    # the bytes it must move: one more step through the counting builds of the
    # traversal kernels (every step draws the same pivots: same seed, bc reset)
    counts = {}
    if not args.skip_count:
        ctx.count(True)
        step(seed)
        counts = ctx.count_read()
        ctx.count(False)
    must = counts.get(kind, {}).get("bytes")
    must_per_launch = must * args.steps / max(cnt, 1) if must else None
    traffic, traffic_note = traffic_for(kernel, graph_key, must_per_launch, 1 if args.width <= 32 else 2)
    if must_per_launch:
        achieved = must_per_launch / avg_s / 1e9
        basis = ("bytes the kernel must move, counted on the device by its counting build over "
                 "one step: each 4-byte word read or written once (adjacency entries, level "
                 "masks, neighbours' per-pivot values, results); 32-byte sectors not counted")
    else:
        achieved = (model_by / (ms / 1000.0)) / 1e9 if ms > 0 else 0.0
        basis = "traversed-edge byte model (no counting build for this kernel kind)"
    model_gbs = (model_by / (ms / 1000.0)) / 1e9 if ms > 0 else 0.0
    roofline = {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                "frac": achieved / peak, "traffic": traffic, "kernel": kernel,
                "achieved_basis": basis,
                "must_move_bytes_per_launch": must_per_launch,
                "work_per_step": counts.get(kind),
                "dram_gbs": (traffic / avg_s / 1e9) if traffic else None,
                "dram_frac": (traffic / avg_s / 1e9 / peak) if traffic else None,
                "traffic_source": traffic_note,
                "model": "traversed-edge byte model, Graph500 counting: (4/W+8) B/TE backward, "
                         "(4/W+4) forward, charged to every edge of a reached vertex (over-counts: "
                         "the backward gathers only successors)",
                "model_bytes_per_launch": model_by / max(cnt, 1),
                "model_frac": model_gbs / peak,
                "launches": cnt, "avg_launch_ms": ms / max(cnt, 1),
                "peak_source": f"{peak_kind} hbm_gbs",
                "share_of_kernel_time": ms / max(sum(v[0] for v in prof.values()), 1e-9),
                "kernel_ms": {k: round(v[0], 3) for k, v in prof.items() if v[1]},
                "work_per_step_by_kind": counts}

    # ---- e2e: the plugin call a user makes for this workload, host side:
    # axbc_run_sampled with the request in host memory, then the pivot list and
    # bc read back into host memory (pinned), every step
    piv = last["pivots"]
    pr = last["probs"]
    import ctypes
    h_bc = torch.empty(G.n, dtype=torch.float32).pin_memory()
    bc_ptr = ctypes.c_void_p(h_bc.data_ptr())

    def e2e_step_():
        r = step(seed)  # run_sampled + axbc_get_pivots (host vectors)
        ax._check(ax.lib().axbc_get_bc(ctx._h, bc_ptr))
        return r["te"], len(r["pivots"])

    e2e = None
    if not args.skip_e2e:
        ctx.profile(False)
        e2e_step_()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        e2e_te = 0
        k_piv = 0
        for _ in range(args.steps):
            te_i, k_piv = e2e_step_()
            e2e_te += te_i
        torch.cuda.synchronize()
        e2e_t = time.perf_counter() - t0
        e2e = {"value": e2e_te * world / e2e_t, "unit": "TE/s",
               "h2d_bytes_per_step": int(ctypes.sizeof(ax.RunParams)),
               "d2h_bytes_per_step": int(G.n * 4 + k_piv * 12),
               "api": "axbc_run_sampled (request parameters from host memory; device sampler, "
                      "batched passes, bc updates) + axbc_get_pivots + axbc_get_bc into pinned "
                      "host memory; wall clock, profiling off"}

    # the plain form (one pivot per launch sequence, host-driven levels) on a
    # sample of the same pivots: the denominator of the batched form's speed-up
    k_plain = 0 if args.skip_plain else min(len(piv), 64)
    ctx.reset()
    torch.cuda.synchronize()
    ev2, ev3 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    ev2.record(stream)
    plain_te = 0
    for v0, p0 in zip(piv[:k_plain], pr[:k_plain]):
        plain_te += ctx.run_pivot(int(v0), float(p0), 0)["te"]
    ev3.record(stream)
    torch.cuda.synchronize()
    plain_t = ev2.elapsed_time(ev3) / 1000.0
    plain = None
    if k_plain:
        plain = {"value": plain_te / plain_t, "unit": "TE/s", "pivots": k_plain,
                 "speedup_of_value": value / world / (plain_te / plain_t)}

    # the same workload in batches of 64 (one 64-pivot pass per batch): a
    # different pivot sequence under the dynamic heuristics (the bc they sample
    # from is refreshed per batch), so beside the headline, not in it
    wide = None
    if not args.skip_wide and args.width == 32:
        def step64():
            return ctx.run_sampled(z=args.z, nbfs=args.pivots, bader_c=0, nchecks=1, H=0, seed=seed, W=64)
        step64()
        ctx.profile(True)
        torch.cuda.synchronize()
        ev4, ev5 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        ev4.record(stream)
        te64 = 0
        for _ in range(args.steps):
            r64 = step64()
            te64 += r64["te"]
        ev5.record(stream)
        torch.cuda.synchronize()
        prof64 = ctx.profile_read()
        ctx.profile(False)
        t64 = ev4.elapsed_time(ev5) / 1000.0
        wide = {"value": te64 / t64, "unit": "TE/s", "batch_width": 64,
                "ms_per_step": t64 * 1000 / args.steps, "te_per_step": te64 / args.steps,
                "pivots_applied_per_step": int(r64["nrounds"]),
                "kernel_ms": {k: round(v[0], 3) for k, v in prof64.items() if v[1]}}

    out = {"metric": metric, "value": value, "unit": "TE/s", "n_gpus": world,
           "steps": args.steps, "warmup": args.warmup, "ms_per_step": t * 1000 / args.steps,
           "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
           "dtype": "u32 path counts, f32 dependencies/bc",
               "data": "synthetic: the Graph500 generator's graph (seeds 23/24), generated on the device",
           "config": config, "e2e": e2e, "roofline": roofline, "clocks": clk,
           "gpu_launches": int(launches), "plain_form": plain, "width_64": wide,
           "te_per_step": te_all / args.steps, "pivots_applied_per_step": int(last["nrounds"])}

    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        csc = G.csc()
        threads = cpu_threads()
        v, k, dt = oracle_sample(csc, piv, pr, args.cpu_seconds, threads)
        v1, dt1 = oracle_single(csc, piv[:1], pr[:1])
        out["cpu_baseline"] = {"value": v, "unit": "TE/s", "cores": threads, "kind": "port",
                               "sample": f"{k} pivots of the step's pivot list in {dt:.1f} s, "
                                         "OpenMP over pivots (oracle/ C restatement)",
                               "single_thread": {"value": v1, "unit": "TE/s", "cores": 1,
                                                 "sample": f"the first pivot of the list in {dt1:.1f} s"}}
    if rank == 0 and world == 1 and not args.skip_serving:
        # the serving configuration after the headline: resident graphs,
        # Poisson arrivals, continuous batching; p50/p99 request latency
        ctx.close()
        G.close()
        torch.cuda.synchronize()
        srv = serve_bench(args, emit=False)
        out["serving"] = {k: srv[k] for k in ("p50_s", "p99_s", "mean_queue_wait_s", "requests",
                                             "failed", "throughput_te_per_s", "requests_per_s",
                                             "span_s", "passes", "lanes_per_pass", "p50_by_graph_s",
                                             "config", "clocks") if k in srv}
    if rank == 0:
        print(json.dumps(out), flush=True)
    if world > 1:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
