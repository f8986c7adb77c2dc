"""Generates the golden fixtures of tests/golden/ from the reference's own functions.

The reference (kris-sigurdson/NSphere) ships no tests, fixtures or known-answer
vectors for its step path, so the fixtures come from running its own functions
(forces, doAdaptiveFullLeap, doAdaptiveFullLeviCivita, doLeviCivitaLeapfrog,
sort_particles, and the method-5 / method-4 / method-2 step bodies) on seeded inputs.  Those functions are extracted
from src/c/nsphere.c and built by oracle/build_oracle.py into oracle/_ref/libnsref.so
with -O2 -fno-fast-math -ffp-contract=off.  Units: G = M = 1 (VEL_CONV_SQ = 1).

Run from the repository root:  python tests/golden/make_golden.py  (all fixtures), or
python tests/golden/make_golden.py method4  (method4.npz alone).
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
    method4_fixture(R)
    print("fixtures written to", OUT)


def method4_fixture(R):
    """4. method 4 (CLI --method 2): the fixed-dtau Levi-Civita leapfrog of single
    particles (doLeviCivitaLeapfrog) and one step body (nsphere.c:5661-5745)."""
    rng = np.random.default_rng(4242)
    n = 4096
    idx = np.sort(rng.choice(np.arange(1, n), 64, replace=False)).astype(np.int32)
    r = 10.0 ** rng.uniform(-4.0, -1.0, idx.size)
    v = rng.normal(0.0, 0.3, idx.size)
    ell = 10.0 ** rng.uniform(-5.0, -2.0, idx.size)
    fixed = np.array([R.lc_fixed(int(i), n, a, b, c, 1e-3, 1000) for i, a, b, c in zip(idx, r, v, ell)])
    m = 5000
    sr, sv, sl, sid = ics.hernquist(m, seed=19)
    perm = rng.permutation(m)
    sr, sv, sl, sid = sr[perm], sv[perm], sl[perm], sid[perm]
    sl = sl.copy()
    low = rng.choice(m, 50, replace=False)
    sl[low] = rng.uniform(0.0, 1e-4, low.size)
    t4, _ = R.step_method4(sr, sv, sl, sid, 1e-3, max_subdiv=128, tol=1e-8, N_taumin=1000)
    np.savez_compressed(os.path.join(OUT, "method4.npz"), n=n, idx=idx, r=r, vr=v, ell=ell, dt=1e-3,
                        N_taumin=1000, fixed_out=fixed, step_r=sr, step_vr=sv, step_ell=sl, step_ids=sid,
                        step_out=t4, step_msub=128, step_tol=1e-8)


if __name__ == "__main__":
    if len(sys.argv) > 1 and sys.argv[1] == "method4":
        build_oracle.build_reference()
        method4_fixture(Reference())
    else:
        main()
