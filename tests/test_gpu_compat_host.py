"""The reference's driver order in C (tests/compat_host.c) linked against
libaxbc_gb300.so: the vertex count comes from the host's global N, every call
goes through the reference-named entry points, and the bc equals the oracle's
bit for bit."""
import os
import subprocess

import numpy as np
import pytest

pytestmark = pytest.mark.gpu
HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
GOLDEN = os.path.join(HERE, "golden")


@pytest.fixture(scope="module")
def host_exe(axbc, tmp_path_factory):
    out = tmp_path_factory.mktemp("compat") / "compat_host"
    libdir = os.path.join(ROOT, "axbc_gb300")
    cmd = ["gcc", "-std=c99", "-O2", "-Wall", "-Werror", "-I", os.path.join(ROOT, "include"),
           os.path.join(HERE, "compat_host.c"), "-o", str(out), "-L", libdir, "-laxbc_gb300",
           f"-Wl,-rpath,{libdir}"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return str(out)


@pytest.mark.parametrize("H", [0, 1])
def test_c_host_drives_the_compat_boundary(host_exe, orc, tmp_path, H):
    e = np.load(os.path.join(GOLDEN, "kron_s10_ef16.npz"))["edges"].astype(np.uint64)
    g = orc.pipeline(e, 1024, True, H)
    rng = np.random.default_rng(17 + H)
    piv = rng.choice(np.flatnonzero(g.deg > 0), 24, replace=False).astype(np.uint32)
    gf, pf, of = tmp_path / "g.bin", tmp_path / "p.bin", tmp_path / "o.bin"
    with open(gf, "wb") as f:
        np.array([g.n, g.m], np.uint64).tofile(f)
        g.col.astype(np.uint32).tofile(f)
        g.row[: g.m].astype(np.uint32).tofile(f)
        g.reach.astype(np.uint32).tofile(f)
    with open(pf, "wb") as f:
        np.array([len(piv)], np.uint64).tofile(f)
        piv.tofile(f)
    r = subprocess.run([host_exe, str(gf), str(pf), str(of), str(H)], capture_output=True, text=True,
                       timeout=300)
    assert r.returncode == 0, r.stderr
    out = np.fromfile(of, np.uint8)
    bc = out[: 4 * g.n].view(np.float32)
    deg = out[4 * g.n:].view(np.uint32)
    want, _, _ = orc.bc_pivots(g, piv, np.full(len(piv), 1.0 / g.n), H)
    same = (bc == want) | (np.isnan(bc) & np.isnan(want))
    assert same.all(), f"{np.count_nonzero(~same)} bc values differ"
    assert np.array_equal(deg, g.deg)
