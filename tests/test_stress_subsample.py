"""The stress configuration checked on the CPU at a 1e6-particle subsample.

Workload: an N = 1e6 Hernquist halo (a = 1, truncated at r = 100, isotropic f(E)) with
20 % of the particles moved to near-radial orbits (ell uniform in [0, 1e-4]), the
default method (adaptive leapfrog with at most 8 levels, adaptive Levi-Civita below
r = 1e-3) at dt = 5e-4, and a central point mass ramped from 0 by 0.01 over 500 steps.

* GPU (plain schedule) against the oracle over 40 steps: the state bit for bit (NaN
  where both have NaN), the energy with the point-mass term to 1e-12 relative, and the
  binned density profile (the reference's 200 linear bins on [0, 10 a), 60 logarithmic
  bins) bin for bin.
* GPU learned schedule against the plain one: the same state bit for bit, so the same
  drift and profile.
* The reference has no central point mass: without it (rate 0, the reference's
  nonfinite behaviour and tau-step cap), the GPU state after 40 steps equals that of
  the reference's own functions bit for bit.
Tolerance: none on the state (bit-exact); 1e-12 relative on energies, which differ by
the order of the GPU's parallel sums only.
"""
import numpy as np
import pytest

from nsphere_gb300 import ics
from test_long_horizon import log_histogram, radial_histogram

pytestmark = pytest.mark.gpu

N, K, DT = 1_000_000, 40, 5e-4
RATE = 0.01 / (500 * DT)


def stress_state(n=N, seed=5):
    r, vr, ell, ids = ics.hernquist(n, seed=seed)
    rng = np.random.default_rng(seed)
    pick = rng.random(n) < 0.2
    ell = ell.copy()
    ell[pick] = rng.uniform(0.0, 1e-4, int(pick.sum()))
    return r, vr, ell, ids


def _same(a, b):
    return np.array_equal(a, b, equal_nan=True)


def _gpu_run(nsg, state, sched, **kw):
    p = nsg.default_params(method=nsg.METHOD_ADAPTIVE_LC, **kw)
    p.sched = sched
    with nsg.Context(p) as c:
        if sched == nsg.SCHED_LEARNED:
            c.mlp_init(3)
        c.upload(*state)
        E0 = sum(c.energy())
        c.step(K)
        out = c.download()
        E1 = sum(c.energy())
        st = c.status()
    return out, E0, E1, st


def test_stress_subsample_gpu_matches_oracle_and_learned_matches_plain(nsg, oracle):
    state = stress_state()
    kw = dict(dt=DT, max_subdiv=128, lc_rule=1, lc_radius=1e-3, max_tau_steps=1_000_000)
    gpu, gE0, gE1, st = _gpu_run(nsg, state, nsg.SCHED_PLAIN, point_mass_rate=RATE, **kw)
    lrn, lE0, lE1, _ = _gpu_run(nsg, state, nsg.SCHED_LEARNED, point_mass_rate=RATE, **kw)

    p = oracle.params(**kw)
    s0 = oracle.sort(*state)
    E0 = sum(oracle.energy(p, s0[0], s0[1], s0[2]))
    cur = state
    for _ in range(K):
        cur = oracle.step_adaptive(p, *cur)[:4]
        p.point_mass = p.point_mass + RATE * DT
    for g, o, q in zip(gpu, cur, lrn):
        assert _same(g, o)
        assert _same(g, q)
    assert abs(gE0 - E0) <= 1e-12 * abs(E0)
    fin = np.isfinite(cur[0]) & np.isfinite(cur[1])
    if fin.all():
        srt = oracle.sort(*cur)
        E1 = sum(oracle.energy(p, srt[0], srt[1], srt[2]))
        assert abs(gE1 - E1) <= 1e-12 * abs(E1)
        assert lE1 == gE1
    assert np.array_equal(radial_histogram(gpu[0], 10.0), radial_histogram(cur[0], 10.0))
    assert np.array_equal(log_histogram(gpu[0]), log_histogram(cur[0]))


def test_stress_subsample_without_point_mass_matches_reference(nsg, reference):
    state = stress_state()
    kw = dict(dt=DT, max_subdiv=128, lc_rule=1, lc_radius=1e-3, max_tau_steps=100_000_000, nonfinite_stop=0)
    gpu, _, _, _ = _gpu_run(nsg, state, nsg.SCHED_PLAIN, **kw)
    ref = (state[0], state[1], state[2], state[3].astype(np.float64))
    for _ in range(K):
        tab, _ = reference.step_method5(*ref, DT, max_subdiv=128, lc_rule=1, lc_radius=1e-3)
        ref = (tab[0], tab[1], tab[2], tab[3])
    assert _same(gpu[0], ref[0]) and _same(gpu[1], ref[1]) and _same(gpu[2], ref[2])
    assert np.array_equal(gpu[3], ref[3].astype(np.int32))
    assert np.array_equal(radial_histogram(gpu[0], 10.0), radial_histogram(ref[0], 10.0))
