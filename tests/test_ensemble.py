"""Ensembles of independent halos in one state (one sort, scan and integrate launch
per step): every halo must evolve exactly as it would alone."""
import numpy as np
import pytest

from nsphere_gb300 import ics

pytestmark = pytest.mark.gpu


def _halos(seed=5, nhalo=6, nmin=800, nmax=20000):
    r, vr, ell, ids, hn = ics.plummer_ensemble(nhalo, nmin, nmax, seed=seed)
    start = np.concatenate([[0], np.cumsum(hn)])
    return r, vr, ell, ids, hn, start


def _shuffle_within(start, seed, *cols):
    rng = np.random.default_rng(seed)
    perm = np.concatenate([start[h] + rng.permutation(start[h + 1] - start[h]) for h in range(len(start) - 1)])
    return tuple(c[perm] for c in cols)


@pytest.mark.parametrize("method", ["adaptive", "kdk"])
def test_ensemble_steps_equal_single_halo_runs(nsg, oracle, method):
    r, vr, ell, ids, hn, start = _halos()
    r, vr, ell, ids = _shuffle_within(start, 1, r, vr, ell, ids)
    steps = 4
    if method == "adaptive":
        kw = dict(dt=2e-3, max_subdiv=128, lc_rule=1, lc_radius=2e-2, max_tau_steps=1_000_000)
        p = oracle.params(dt=2e-3, max_subdiv=128, lc_rule=1, lc_radius=2e-2)
    else:
        kw = dict(dt=2e-3, method=nsg.METHOD_KDK)
        p = oracle.params(dt=2e-3)
    with nsg.Context(nsg.default_params(**kw)) as c:
        c.upload_ensemble(r, vr, ell, ids, hn)
        c.step(steps)
        gr, gv, gl, gid = c.download()
        K, W = c.energy_halos()
    for h in range(len(hn)):
        a, b = start[h], start[h + 1]
        cur = (r[a:b], vr[a:b], ell[a:b], ids[a:b] - a)
        if method == "kdk":
            cur = oracle.sort(*cur)
        for _ in range(steps):
            cur = oracle.step_adaptive(p, *cur)[:4] if method == "adaptive" else oracle.step_kdk(p, *cur)
        assert np.array_equal(gid[a:b] - a, cur[3]), h
        assert np.array_equal(gr[a:b], cur[0]) and np.array_equal(gv[a:b], cur[1]), h
        # per-halo energy of the state, sorted (the ensemble energy call sorts first)
        s = oracle.sort(*cur)
        oK, oW = oracle.energy(p, s[0], s[1], s[2])
        assert abs(K[h] - oK) <= 1e-12 * abs(oK) and abs(W[h] - oW) <= 1e-12 * abs(oW)


@pytest.mark.parametrize("lc_radius,nmax,steps", [(0.1, 20000, 3), (0.3, 20000, 1), (1.0, 4000, 1)])
def test_ensemble_levi_civita_list_before_the_sort(nsg, oracle, lc_radius, nmax, steps):
    """The fixed-radius Levi-Civita list of an ensemble is made before the sort, each
    candidate ranked within its own halo; with more candidates than the list holds
    (lc_radius 1.0) the list made after the sort takes over.  Every halo evolves as it
    would alone."""
    r, vr, ell, ids, hn, start = _halos(seed=11, nhalo=6, nmin=1500, nmax=nmax)
    r, vr, ell, ids = _shuffle_within(start, 2, r, vr, ell, ids)
    kw = dict(dt=1e-3, max_subdiv=64, lc_rule=1, lc_radius=lc_radius, max_tau_steps=1_000_000)
    p = oracle.params(dt=1e-3, max_subdiv=64, lc_rule=1, lc_radius=lc_radius)
    with nsg.Context(nsg.default_params(**kw)) as c:
        c.upload_ensemble(r, vr, ell, ids, hn)
        c.step(steps)
        gr, gv, gl, gid = c.download()
        glv = c.levels()
    n_lc = 0
    for h in range(len(hn)):
        a, b = start[h], start[h + 1]
        cur = (r[a:b], vr[a:b], ell[a:b], ids[a:b] - a)
        for _ in range(steps):
            out = oracle.step_adaptive(p, *cur)
            cur, olv = out[:4], out[4]
        n_lc += int(np.sum(olv >= 99))
        assert np.array_equal(gid[a:b] - a, cur[3]), h
        assert np.array_equal(glv[a:b], olv), h
        assert np.array_equal(gr[a:b], cur[0]) and np.array_equal(gv[a:b], cur[1]), h
    assert n_lc > (4096 if lc_radius == 1.0 else 10)


def test_ensemble_radix_fallback_and_bucket_path(nsg, oracle):
    """First sort of shuffled halos runs the radix sort with the halo passes; the
    second runs the near-sorted bucket path per halo; both give per-halo order."""
    r, vr, ell, ids, hn, start = _halos(seed=9, nhalo=40, nmin=300, nmax=6000)
    r, vr, ell, ids = _shuffle_within(start, 2, r, vr, ell, ids)
    with nsg.Context(nsg.default_params()) as c:
        c.upload_ensemble(r, vr, ell, ids, hn)
        c.sort()
        s1 = c.download()
        c.sort()
        s2 = c.download()
    for h in range(len(hn)):
        a, b = start[h], start[h + 1]
        o = oracle.sort(r[a:b], vr[a:b], ell[a:b], ids[a:b] - a)
        for s in (s1, s2):
            assert np.array_equal(s[3][a:b] - a, o[3]) and np.array_equal(s[0][a:b], o[0])


def test_ensemble_rejects_ids_outside_their_halo(nsg):
    r, vr, ell, ids, hn, start = _halos(nhalo=3, nmin=100, nmax=200)
    ids = ids.copy()
    ids[start[1]], ids[start[1] - 1] = ids[start[1] - 1], ids[start[1]]   # swap across a boundary
    with nsg.Context(nsg.default_params()) as c:
        with pytest.raises(nsg.NsgError) as e:
            c.upload_ensemble(r, vr, ell, ids, hn)
        assert e.value.code == nsg.NSG_EIDS
