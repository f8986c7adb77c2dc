"""Tracking energies (nsphere.c:6384-6450) and the static potential they use.

CPU: the oracle's closed-form Psi(r) against the reference's own construction
(nsphere.c:4575-4592: M(r) and the outer integral by quadrature of the
mass-normalised profile, then Psi = G M(r)/r + G M/norm * int_r^inf r' f dr'), and
the clamps of evaluatespline (nsphere.c:8205-8236) and of the low-ell group.
GPU: the device recorder, run inside graph-replayed steps, against the oracle's
records of the oracle's own steps, bit for bit for the Plummer and Hernquist
potentials and to a few ulp of Psi for the cored one (atan differs between the two
maths libraries).
"""
import math

import numpy as np
import pytest

from nsphere_gb300 import ics

PROFILES = {  # model: f(r) with scale a
    0: lambda r, a: (1.0 + (r / a) ** 2) ** -3,
    1: lambda r, a: (1.0 + (r / a) ** 2) ** -2.5,
    2: lambda r, a: 1.0 / ((r / a) * (1.0 + r / a) ** 3),
}


def _psi_quadrature(model, a, r_trunc, r, G=1.0, M=1.0):
    integrate = pytest.importorskip("scipy.integrate")
    f = PROFILES[model]
    kw = dict(epsabs=0.0, epsrel=1e-13, limit=400)
    norm = integrate.quad(lambda x: x * x * f(x, a), 0.0, r_trunc, points=[a], **kw)[0]
    inner = integrate.quad(lambda x: x * x * f(x, a), 0.0, r, **kw)[0]
    outer = integrate.quad(lambda x: x * f(x, a), r, np.inf, **kw)[0]
    return G * (M * inner / norm / r + M / norm * outer)


@pytest.mark.parametrize("model,a,r_trunc", [(0, 100.0, 1000.0), (1, 1.0, 30.0), (2, 1.0, 100.0)])
def test_closed_form_psi_matches_quadrature(oracle, model, a, r_trunc):
    for r in [1e-3 * a, 0.07 * a, 0.5 * a, a, 3.3 * a, 0.9 * r_trunc]:
        ref = _psi_quadrature(model, a, r_trunc, r, G=2.5, M=3.0)
        got = oracle.psi(model, a, r_trunc, 0.0, 0.0, r, G=2.5, M=3.0)
        assert got == pytest.approx(ref, rel=1e-10), (model, r)


def test_untruncated_limits(oracle):
    # r_trunc <= 0: the untruncated normalisation
    assert oracle.psi(1, 2.0, 0.0, 0.0, 0.0, 0.0) == pytest.approx(1.0 / 2.0, rel=1e-15)
    assert oracle.psi(2, 2.0, 0.0, 0.0, 0.0, 0.0) == pytest.approx(1.0 / 2.0, rel=1e-15)
    # cored, m(inf) = pi/16, Psi(0) = G M / (a pi/16) / 4
    assert oracle.psi(0, 1.0, 0.0, 0.0, 0.0, 1e-12) == pytest.approx(4.0 / math.pi, rel=1e-12)
    # the series below x = 1e-3 joins the closed form
    lo = oracle.psi(0, 1.0, 10.0, 0.0, 0.0, 1e-3 * (1 - 1e-12))
    hi = oracle.psi(0, 1.0, 10.0, 0.0, 0.0, 1e-3 * (1 + 1e-12))
    assert lo == pytest.approx(hi, rel=1e-13)


def test_evaluatespline_clamps(oracle):
    rc = 100.0
    rmax, rhi = 10 * rc, 9999.0 / 10000.0 * 10 * rc
    at_hi = oracle.psi(0, rc, rmax, 0.0, rhi, rhi - 1e-10)
    assert oracle.psi(0, rc, rmax, 0.0, rhi, 5 * rmax) == at_hi
    assert oracle.psi(0, rc, rmax, 0.0, rhi, -3.0) == oracle.psi(0, rc, rmax, 0.0, rhi, 1e-10)


def test_track_records_and_clamps(oracle):
    r = np.array([0.5, 2.0, -1.0, 50.0])
    v = np.array([0.1, -0.3, 0.2, 0.0])
    l = np.array([0.2, 0.4, 0.1, 0.3])
    out = oracle.track(2, 1.0, 10.0, 0.0, 0.0, r, v, l, k_clamped=2)
    # the low-ell group (last two) is clamped to [1e-10, r_trunc] and stored clamped
    assert out[0, 2] == 1e-10 and out[0, 3] == 10.0
    assert out[0, 0] == 0.5 and out[0, 1] == 2.0
    w = v[0] ** 2 + l[0] ** 2 / r[0] ** 2
    assert out[3, 0] == oracle.psi(2, 1.0, 10.0, 0.0, 0.0, 0.5) - 0.5 * w
    assert out[4, 0] == v[0] / math.sqrt(w)


def _expected_records(oracle, states, ids, psi_args, k_clamped):
    recs = []
    for st in states:
        pos = np.empty(len(ids), dtype=np.int64)
        where = np.empty(len(st[3]), dtype=np.int64)
        where[st[3]] = np.arange(len(st[3]))
        pos[:] = where[ids]
        recs.append(oracle.track(*psi_args, st[0][pos], st[1][pos], st[2][pos], k_clamped=k_clamped))
    return np.stack(recs, axis=-1)   # (5, k, steps)


@pytest.mark.gpu
@pytest.mark.parametrize("method", [2, 5])
@pytest.mark.parametrize("model", [0, 1, 2])
def test_recorder_matches_oracle(nsg, oracle, method, model):
    n, dt, steps = 6000, 1e-3, 7
    r, vr, ell, ids = oracle.sort(*ics.plummer(n, seed=12))
    low = np.argsort(ell, kind="stable")[:5]
    track_ids = np.concatenate([np.arange(10), ids[low]]).astype(np.int32)
    a, r_trunc = (1.0, 30.0) if model else (0.5, 5.0)
    psi = nsg.Psi(model, 0, a, r_trunc, 0.0, 0.9999 * r_trunc)
    kw = dict(dt=dt, max_subdiv=64, lc_rule=1, lc_radius=2e-2) if method == 5 else dict(dt=dt)
    p = oracle.params(**kw)
    states, cur = [], (r, vr, ell, ids)
    for _ in range(steps):
        cur = (oracle.step_adaptive(p, *cur) if method == 5 else oracle.step_kdk(p, *cur))[:4]
        states.append(cur)
    want = _expected_records(oracle, states, track_ids, (model, a, r_trunc, 0.0, 0.9999 * r_trunc), 5)
    with nsg.Context(nsg.default_params(method=method, max_tau_steps=1_000_000, **kw)) as c:
        c.upload(r, vr, ell, ids)
        c.track_open(track_ids, psi, capacity=steps - 2, k_clamped=5)
        c.step(steps - 2)          # graph replays
        got, seen = c.track_read()
        assert seen == steps - 2 and got.shape == (5, 15, steps - 2)
        c.step(2)                  # buffer full: counted, not stored
        got2, seen2 = c.track_read()
        assert seen2 == steps and np.array_equal(got2, got)
        gr, gv, gl, gid = c.download()
    assert np.array_equal(gid, states[-1][3]) and np.array_equal(gr, states[-1][0])
    w = want[:, :, :steps - 2]
    assert np.array_equal(got[:3], w[:3])
    if model == 0:
        scale = np.abs(np.array([oracle.psi(0, a, r_trunc, 0.0, 0.0, 0.0)]))
        assert np.max(np.abs(got[3] - w[3])) <= 8 * np.finfo(float).eps * scale[0]
        assert np.array_equal(got[4], w[4])
    else:
        assert np.array_equal(got[3:], w[3:])


@pytest.mark.gpu
def test_recorder_bad_ids_and_reopen(nsg):
    r, vr, ell, ids = ics.plummer(2000, seed=3)
    with nsg.Context(nsg.default_params(dt=1e-3, method=nsg.METHOD_KDK)) as c:
        c.upload(r, vr, ell, ids)
        psi = nsg.Psi(1, 0, 1.0, 0.0, 0.0, 0.0)
        c.track_open(np.array([5, -1, 2000], dtype=np.int32), psi, capacity=4)
        c.step(3)
        got, seen = c.track_read()
        assert seen == 3 and np.all(np.isfinite(got[:, 0])) and np.all(np.isnan(got[:, 1:]))
        c.track_open(np.array([7], dtype=np.int32), psi, capacity=2)   # replaces the recorder
        c.step(1)
        got, seen = c.track_read()
        assert seen == 1 and got.shape == (5, 1, 1)
        c.track_close()
        with pytest.raises(nsg.NsgError):
            c.track_read()
        with pytest.raises(nsg.NsgError):
            c.track_open(np.array([1], dtype=np.int32), nsg.Psi(7, 0, 1.0, 0.0, 0.0, 0.0), capacity=1)


@pytest.mark.gpu
def test_recorder_equals_gather_on_an_ensemble(nsg):
    """Ids are global over the halos of an ensemble: the recorder's r, v_r, ell after
    each step equal nsg_gather's for the same ids."""
    r, vr, ell, ids, sizes = ics.plummer_ensemble(4, 2000, 8000, seed=5)
    track = np.array([0, 5, int(sizes[0]) + 3, int(ids.size) - 1], dtype=np.int32)
    with nsg.Context(nsg.default_params(dt=1e-3, max_subdiv=64, lc_rule=1, lc_radius=1e-2)) as c:
        c.upload_ensemble(r, vr, ell, ids, sizes)
        c.track_open(track, nsg.Psi(1, 0, 1.0, 0.0, 0.0, 0.0), capacity=4)
        want = []
        for _ in range(4):
            c.step(1)
            gr, gv, gl, _ = c.gather(track)
            want.append((gr, gv, gl))
        got, seen = c.track_read()
    assert seen == 4
    for s, (gr, gv, gl) in enumerate(want):
        assert np.array_equal(got[0, :, s], gr) and np.array_equal(got[1, :, s], gv)
        assert np.array_equal(got[2, :, s], gl)
