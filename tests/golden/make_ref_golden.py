"""Golden fixtures from the reference program itself (run in the build
container only; the committed .npz files are what the tests read).

The reference's single-GPU program is built for a host without GPU or MPI by
`make -C oracle refbc` (src/axbc2d.c and its Graph500 generator compiled
unchanged against a one-rank MPI stand-in; its mono kernels, copied unedited
from src/cuda_kernels.cu, run thread after thread on the host).  Each case
below runs it with the given command line and records, from the record file
the host boundary writes (AXBC_REF_DUMP) and from its stdout:

  - the CSC it built (SHA-256 of col, row, reach),
  - the pivot sequence with probabilities and nvisited+all per pivot,
  - per pivot the SHA-256 of its final levels and uint32 path counts,
  - the dependencies of the first and the last pivot,
  - the final bc vector (before the output's division by 2 * nrounds),
  - rounds, skipped rounds, Bader stop, check vertices,
  - for the first case, the -o output file.

    python tests/golden/make_ref_golden.py [--only NAME]
"""
import hashlib
import os
import re
import struct
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

# name: (command-line arguments after -p 1x1, graph source)
# graph source: ("kron", scale) for -S scale -E 16, ("grid", side) for a grid
# edge file read with -f / -n
CASES = {
    "s10_z0": (["-S", "10", "-E", "16", "-z", "0", "-N", "64", "-c", "0"], ("kron", 10)),
    "s10_H1_z1": (["-S", "10", "-E", "16", "-H", "1", "-z", "1", "-N", "64", "-c", "0"], ("kron", 10)),
    "s10_z2": (["-S", "10", "-E", "16", "-z", "2", "-N", "48", "-c", "0"], ("kron", 10)),
    "s10_z3": (["-S", "10", "-E", "16", "-z", "3", "-N", "64", "-c", "0"], ("kron", 10)),
    "s10_z4": (["-S", "10", "-E", "16", "-z", "4", "-N", "64", "-c", "0"], ("kron", 10)),
    "s10_z5": (["-S", "10", "-E", "16", "-z", "5", "-N", "48", "-c", "0"], ("kron", 10)),
    "s10_z6": (["-S", "10", "-E", "16", "-z", "6", "-N", "48", "-c", "0"], ("kron", 10)),
    "s10_U_z0": (["-S", "10", "-E", "16", "-U", "-z", "0", "-N", "48", "-c", "0"], ("kron", 10)),
    "s12_H1_z3": (["-S", "12", "-E", "16", "-H", "1", "-z", "3", "-N", "64", "-c", "0"], ("kron", 12)),
    "s14_z0_N256": (["-S", "14", "-E", "16", "-z", "0", "-N", "256", "-c", "0"], ("kron", 14)),
    "grid64_z4_bader": (["-z", "4", "-N", "2048", "-c", "1", "-x", "8"], ("grid", 64)),
    "grid64_H1_z0_bader": (["-H", "1", "-z", "0", "-N", "2048", "-c", "1", "-x", "4"], ("grid", 64)),
}


def grid_edges(side, drop=0.02, longrange=8, seed=7):
    """side x side four-neighbour grid, each edge dropped with probability
    `drop`, plus `longrange` uniform random edges (seeded numpy draws)."""
    rng = np.random.default_rng(seed)
    v = np.arange(side * side, dtype=np.int64).reshape(side, side)
    e = np.concatenate([np.stack([v[:, :-1].ravel(), v[:, 1:].ravel()], 1),
                        np.stack([v[:-1, :].ravel(), v[1:, :].ravel()], 1)])
    e = e[rng.random(len(e)) >= drop]
    extra = rng.integers(0, side * side, size=(longrange, 2))
    return np.concatenate([e, extra]).astype(np.uint16)


def parse_dump(path):
    d = open(path, "rb").read()
    off, out, piv = 0, {}, []
    while off < len(d):
        tag, ln = struct.unpack_from("<IQ", d, off)
        off += 12
        body = d[off:off + ln]
        off += ln
        if tag == 1:
            n, m = struct.unpack_from("<QQ", body, 0)
            out["n"], out["m"] = n, m
            out["col"] = np.frombuffer(body, np.uint32, n + 1, 16)
            out["row"] = np.frombuffer(body, np.uint32, m, 16 + 4 * (n + 1))
        elif tag == 2:
            out["reach"] = np.frombuffer(body, np.uint32)
        elif tag == 3:
            n = out["n"]
            v0, r0, p, nv = struct.unpack_from("<IIdQ", body, 0)
            lvl = np.frombuffer(body, np.int32, n, 24)
            sig = np.frombuffer(body, np.uint32, n, 24 + 4 * n)
            dl = np.frombuffer(body, np.float32, n, 24 + 8 * n)
            piv.append((v0, p, nv, lvl, sig, dl))
        elif tag == 4:
            out["bc"] = np.frombuffer(body, np.float32).copy()
        elif tag == 5:
            break
    out["pivots"] = piv
    return out


def sha(a):
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def pivot_digest(lvl, sig):
    return np.frombuffer(hashlib.sha256(lvl.tobytes() + sig.tobytes()).digest(), np.uint8)


def run_case(exe, name, args, src, tmp):
    argv = [exe, "-p", "1x1"] + list(args)
    extra = {}
    if src[0] == "grid":
        e = grid_edges(src[1])
        gpath = os.path.join(tmp, f"{name}.txt")
        with open(gpath, "w") as f:
            for a, b in e:
                f.write(f"{a} {b}\n")
        argv += ["-f", gpath, "-n", str(src[1] * src[1])]
        extra["edges"] = e
    dump = os.path.join(tmp, f"{name}.bin")
    oprefix = os.path.join(tmp, name)
    argv += ["-o", oprefix]
    env = dict(os.environ, AXBC_REF_DUMP=dump)
    r = subprocess.run(argv, capture_output=True, text=True, env=env, timeout=1800)
    if r.returncode != 0:
        raise SystemExit(f"{name}: reference exited {r.returncode}\n{r.stdout[-2000:]}\n{r.stderr[-2000:]}")
    d = parse_dump(dump)
    out = r.stdout
    rounds = int(re.search(r"BC rounds: (\d+)", out).group(1))
    skipped = int(re.search(r"BC skipped: (\d+)", out).group(1))
    stopped = "exit bader criterion" in out
    m = re.search(r"Selected Verts to Approximate \(TODO REMOVE PRINT\): ([0-9 ]*)\n", out)
    checks = np.array([int(x) for x in m.group(1).split()], np.uint32) if m and m.group(1).strip() else \
        np.zeros(0, np.uint32)
    piv = d["pivots"]
    assert len(piv) == rounds, (name, len(piv), rounds)
    fx = dict(
        argv=np.array(["-p", "1x1"] + list(args)),
        graph=np.array([src[0], str(src[1])]),
        n=np.uint64(d["n"]), m=np.uint64(d["m"]),
        col_sha=np.array(sha(d["col"])), row_sha=np.array(sha(d["row"])), reach_sha=np.array(sha(d["reach"])),
        pivots=np.array([p[0] for p in piv], np.uint32),
        probs=np.array([p[1] for p in piv], np.float64),
        nvisited_all=np.array([p[2] for p in piv], np.uint64),
        pivot_digest=np.stack([pivot_digest(p[3], p[4]) for p in piv]) if piv else np.zeros((0, 32), np.uint8),
        delta_first=piv[0][5].copy() if piv else np.zeros(0, np.float32),
        delta_last=piv[-1][5].copy() if piv else np.zeros(0, np.float32),
        bc=d["bc"], rounds=np.uint64(rounds), skipped=np.uint64(skipped), stopped=np.bool_(stopped),
        checks=checks, **extra)
    if name == "s10_z0":
        fx["output_file"] = np.array(open(f"{oprefix}_1X1_0.log").read())
    return fx


def main():
    import oracle
    only = sys.argv[sys.argv.index("--only") + 1] if "--only" in sys.argv else None
    rd = oracle.reference_dir()
    if rd is None:
        raise SystemExit("the reference sources are not present on this machine")
    subprocess.run(["make", "-s", "-C", os.path.join(ROOT, "oracle"), "refbc", f"REF={rd}"], check=True)
    exe = os.path.join(ROOT, "oracle", "_ref", "axbc_ref")
    with tempfile.TemporaryDirectory() as tmp:
        for name, (args, src) in CASES.items():
            if only and name != only:
                continue
            fx = run_case(exe, name, args, src, tmp)
            np.savez_compressed(os.path.join(HERE, f"ref_{name}.npz"), **fx)
            print(f"{name}: n={int(fx['n'])} m={int(fx['m'])} rounds={int(fx['rounds'])} "
                  f"skipped={int(fx['skipped'])} stopped={bool(fx['stopped'])}")


if __name__ == "__main__":
    main()
