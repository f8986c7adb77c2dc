"""The C boundary exercised from C: tests/c/step_driver.c, compiled with gcc against
include/nsg.h and libnsg.so, runs the integration sequence (nsg_params_default,
nsg_create, nsg_upload_particles on a double *particles[5] table, nsg_step,
nsg_gather every step, nsg_download_particles, nsg_sync, nsg_destroy) on a state
read from a reference initial-conditions file (nsphere.c:2386-2487), and writes its
arrays to a file that is compared bit for bit with the oracle.
"""
import os
import subprocess

import numpy as np
import pytest

from conftest import ROOT
from nsphere_gb300 import ics

DRIVER = os.path.join(ROOT, "tests", "c", "step_driver.c")


def build_driver(out_dir):
    from nsphere_gb300 import build as nbuild

    lib = nbuild.build()
    exe = os.path.join(str(out_dir), "step_driver")
    cmd = ["gcc", "-O2", "-Wall", "-Wextra", "-Werror", "-I", os.path.join(ROOT, "include"), DRIVER,
           "-L", os.path.dirname(lib), "-lnsg", "-Wl,-rpath," + os.path.dirname(lib), "-o", exe]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return exe


def write_init(path, r, vr, ell, ids, mu=None):
    """The reference's initial-conditions file: int32 N, N x (r, v_r, ell, id, mu)."""
    n = len(r)
    rec = np.empty((n, 5))
    rec[:, 0], rec[:, 1], rec[:, 2], rec[:, 3] = r, vr, ell, ids
    rec[:, 4] = 0.0 if mu is None else mu
    with open(path, "wb") as f:
        np.array([n], dtype=np.int32).tofile(f)
        rec.tofile(f)


def read_out(path):
    with open(path, "rb") as f:
        n, steps, k = (int(x) for x in np.fromfile(f, np.int32, 3))
        status = int(np.fromfile(f, np.uint32, 1)[0])
        rows = np.fromfile(f, np.float64, 4 * n).reshape(4, n)
        track = []
        for _ in range(steps):
            vals = np.fromfile(f, np.float64, 3 * k).reshape(3, k)
            rank = np.fromfile(f, np.int32, k)
            track.append((vals, rank))
    return rows, track, status


def test_c_driver_compiles_against_the_header(tmp_path):
    """gcc builds and links the C driver against include/nsg.h and libnsg.so (no GPU)."""
    exe = build_driver(tmp_path)
    assert os.access(exe, os.X_OK)


@pytest.mark.gpu
@pytest.mark.parametrize("method", [5, 2], ids=["adaptive_lc", "kdk"])
def test_c_driver_matches_oracle(tmp_path, oracle, method):
    n, steps = 20_000, 12
    r, vr, ell, ids = ics.hernquist(n, seed=21)
    perm = np.random.default_rng(21).permutation(n)
    r, vr, ell, ids = r[perm], vr[perm], ell[perm], ids[perm]
    init, out = str(tmp_path / "init.dat"), str(tmp_path / "out.dat")
    write_init(init, r, vr, ell, ids)
    exe = build_driver(tmp_path)
    dt = 5e-4
    res = subprocess.run([exe, init, out, str(steps), str(method), repr(dt), "128", "1", "1e-3"],
                         capture_output=True, text=True, timeout=300)
    assert res.returncode == 0, res.stderr
    rows, track, status = read_out(out)
    assert status & 0x2 == 0    # no tau-step cap

    if method == 5:
        p = oracle.params(dt=dt, max_subdiv=128, lc_rule=1, lc_radius=1e-3)
        step = lambda cur: oracle.step_adaptive(p, *cur)[:4]   # noqa: E731
    else:
        p = oracle.params(dt=dt)
        step = lambda cur: oracle.step_kdk(p, *cur)            # noqa: E731
    cur = (r, vr, ell, ids) if method == 5 else oracle.sort(r, vr, ell, ids)
    for j in range(steps):
        cur = step(cur)
        vals, rank = track[j]
        pos = np.argsort(cur[3])[:10]      # array index of ids 0..9
        assert np.array_equal(rank, pos)
        assert np.array_equal(vals[0], cur[0][pos]) and np.array_equal(vals[1], cur[1][pos])
        assert np.array_equal(vals[2], cur[2][pos])
    assert np.array_equal(rows[0], cur[0]) and np.array_equal(rows[1], cur[1])
    assert np.array_equal(rows[2], cur[2]) and np.array_equal(rows[3].astype(np.int32), cur[3])
