"""Generates the golden fixtures of tests/golden/ from the reference's own functions.

The reference (kris-sigurdson/NSphere) ships no tests, fixtures or known-answer
vectors for its step path, so the fixtures come from running its own functions
(forces, doAdaptiveFullLeap, doAdaptiveFullLeviCivita, sort_particles, and the
method-5 / method-2 step bodies) on seeded inputs.  Those functions are extracted
from src/c/nsphere.c and built by oracle/build_oracle.py into oracle/_ref/libnsref.so
with -O2 -fno-fast-math -ffp-contract=off.  Units: G = M = 1 (VEL_CONV_SQ = 1).

Run from the repository root:  python tests/golden/make_golden.py
"""
from __future__ import annotations

import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

from nsphere_gb300 import ics  # noqa: E402
from oracle import build_oracle  # noqa: E402
from oracle.oracle import Reference  # noqa: E402

OUT = os.path.dirname(os.path.abspath(__file__))


def main():
    build_oracle.build_reference()
    R = Reference()
    rng = np.random.default_rng(12345)

    # 1. single-particle integrators on a Hernquist sample plus hand-picked hard cases
    n = 4096
    r, vr, ell, ids = ics.hernquist(n, seed=11)
    pick = np.sort(rng.choice(n, 256, replace=False))
    extra_r = np.array([1e-4, 3e-4, 1e-3, 2e-3, 0.05, 0.5, 5.0, 50.0])
    extra_v = np.array([-0.5, 0.3, -0.1, 0.0, 1.2, -0.9, 0.2, -0.05])
    extra_l = np.array([1e-5, 1e-4, 1e-3, 1e-2, 0.03, 0.3, 1.0, 2.0])
    extra_i = np.array([1, 2, 5, 10, 200, 1500, 3500, 4090])
    pr = np.concatenate([r[pick], extra_r])
    pv = np.concatenate([vr[pick], extra_v])
    pl = np.concatenate([ell[pick], extra_l])
    pi = np.concatenate([pick, extra_i]).astype(np.int32)
    cases = []
    for dt, msub in ((5e-4, 128), (1e-2, 128), (1e-2, 1 << 12)):
        out = np.array([R.adaptive_leap(int(i), n, a, b, c, dt, max_subdiv=msub)
                        for i, a, b, c in zip(pi, pr, pv, pl)])
        cases.append((dt, msub, out))
    lc_out = np.array([R.adaptive_lc(int(i), n, a, b, c, 5e-4, max_subdiv=128)
                       for i, a, b, c in zip(pi, pr, pv, pl)])
    np.savez_compressed(os.path.join(OUT, "integrators.npz"), n=n, idx=pi, r=pr, vr=pv, ell=pl,
                        leap_dt=np.array([c[0] for c in cases]),
                        leap_msub=np.array([c[1] for c in cases]),
                        leap_out=np.stack([c[2] for c in cases]), lc_dt=5e-4, lc_msub=128,
                        lc_out=lc_out)

    # 2. sort_particles (exact quadsort) on a shuffled state with distinct radii
    n = 3000
    r, vr, ell, ids = ics.plummer(n, seed=13)
    perm = rng.permutation(n)
    mu = rng.uniform(-1, 1, n)
    tab = R.sort_particles(r[perm], vr[perm], ell[perm], ids[perm], mu[perm])
    np.savez_compressed(os.path.join(OUT, "sort.npz"), r=r[perm], vr=vr[perm], ell=ell[perm],
                        ids=ids[perm], mu=mu[perm], out=tab)

    # 3. one method-5 step (r_crit rule), one with the fixed-radius rule, and 5 KDK steps
    n = 5000
    r, vr, ell, ids = ics.hernquist(n, seed=17)
    perm = rng.permutation(n)
    r, vr, ell, ids = r[perm], vr[perm], ell[perm], ids[perm]
    # a few near-radial orbits so that the Levi-Civita path is exercised
    lowl = rng.choice(n, 40, replace=False)
    ell = ell.copy()
    ell[lowl] = rng.uniform(0.0, 1e-4, lowl.size)
    # and inner particles whose centrifugal term dominates (r < 0.05 ell^2 / (G M_i))
    inner = np.flatnonzero(r < 0.2)[:30]
    ell[inner] = np.sqrt(40.0 * r[inner] ** 3 / (1.0 + r[inner]) ** 2)
    t5, _ = R.step_method5(r, vr, ell, ids, 5e-4, max_subdiv=128, lc_rule=0)
    t5b, _ = R.step_method5(r, vr, ell, ids, 5e-4, max_subdiv=128, lc_rule=1, lc_radius=1e-1)
    cur = np.array([r, vr, ell, ids.astype(np.float64), np.zeros(n)])
    cur = R.sort_particles(cur[0], cur[1], cur[2], cur[3])  # the reference's initial sort
    start = cur.copy()
    for _ in range(5):
        cur, _ = R.step_kdk(cur[0], cur[1], cur[2], cur[3], 1e-3)
    np.savez_compressed(os.path.join(OUT, "steps.npz"), r=r, vr=vr, ell=ell, ids=ids,
                        method5_rcrit=t5, method5_radius=t5b, kdk_start=start, kdk5=cur,
                        dt5=5e-4, dt_kdk=1e-3, lc_radius=1e-1)
    print("fixtures written to", OUT)


if __name__ == "__main__":
    main()
