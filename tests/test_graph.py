"""Steps replayed from a captured CUDA graph equal steps launched one kernel at a
time, bit for bit, for every method and for ensembles."""
import numpy as np
import pytest

from nsphere_gb300 import ics

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("kw", [
    dict(dt=1e-3, max_subdiv=128, lc_rule=1, lc_radius=3e-2),
    dict(dt=1e-3, max_subdiv=128, lc_rule=0),
    dict(dt=1e-3, method=2),
    dict(dt=1e-3, method=2, point_mass=1e-3, point_mass_rate=0.5),
    dict(dt=1e-3, max_subdiv=64, lc_rule=1, lc_radius=1e-2, point_mass_rate=0.2),
])
def test_graph_replay_equals_eager(nsg, kw):
    n = 30000
    r, vr, ell, ids = ics.hernquist(n, seed=21)
    out = []
    for graph in (0, 1):
        with nsg.Context(nsg.default_params(graph=graph, max_tau_steps=1_000_000, **kw)) as c:
            c.upload(r, vr, ell, ids)
            c.step(9)
            out.append(c.download() + (c.energy(),))
            launches, steps = c.counters()
            assert steps == 9
    for a, b in zip(out[0], out[1]):
        if isinstance(a, tuple):
            assert a == b
        else:
            assert np.array_equal(a, b)


def test_graph_replay_ensemble(nsg):
    r, vr, ell, ids, hn = ics.plummer_ensemble(12, 500, 8000, seed=4)
    out = []
    for graph in (0, 1):
        with nsg.Context(nsg.default_params(graph=graph, dt=2e-3, max_subdiv=128, lc_rule=1, lc_radius=1e-2,
                                            max_tau_steps=1_000_000)) as c:
            c.upload_ensemble(r, vr, ell, ids, hn)
            c.step(7)
            out.append(c.download())
    for a, b in zip(out[0], out[1]):
        assert np.array_equal(a, b)


@pytest.mark.parametrize("cond", [1, 0], ids=["conditional_node", "direct"])
@pytest.mark.parametrize("method", [2, 5])
def test_graph_replay_with_radix_fallback(nsg, method, cond, monkeypatch):
    """10000 particles at rest at r = 1 without gravity keep equal radii, so every
    near-sorted sort overflows its bucket and the radix sort runs: in a replayed graph
    it sits in a conditional node that the overflow opens (or, where the driver builds
    no conditional nodes -- forced here by NSG_NO_CONDITIONAL_NODES -- its kernels are
    captured directly and return at once when not needed).  Replay equals eager
    launches either way, and the equal radii stay ordered by id."""
    if not cond:
        monkeypatch.setenv("NSG_NO_CONDITIONAL_NODES", "1")
    rng = np.random.default_rng(8)
    n, ntie = 30000, 10000
    r = rng.uniform(0.1, 3.0, n)
    vr = rng.normal(0.0, 0.1, n)
    ell = rng.uniform(0.0, 0.5, n)
    tie = rng.choice(n, ntie, replace=False)
    r[tie], vr[tie], ell[tie] = 1.0, 0.0, 0.0
    ids = rng.permutation(n).astype(np.int32)
    kw = dict(dt=1e-3, G=0.0, method=method, max_subdiv=64, lc_rule=2, max_tau_steps=1_000_000)
    out = []
    for graph in (0, 1):
        with nsg.Context(nsg.default_params(graph=graph, **kw)) as c:
            c.upload(r, vr, ell, ids)
            c.step(8)
            out.append(c.download())
    for a, b in zip(out[0], out[1]):
        assert np.array_equal(a, b)
    gr, _, _, gid = out[1]
    at1 = gr == 1.0
    assert at1.sum() == ntie and np.all(np.diff(gid[at1]) > 0)
    if method == 2:   # the fixed-step body ends with the sort; the adaptive one integrates after it
        assert np.all(np.diff(gr) >= 0)


def test_step_download_with_radix_fallback(nsg):
    """nsg_step_download runs its last step eagerly and reads the overflow flag on the
    host, launching the radix sort only when the near-sorted path overflowed: with
    10000 equal radii (no gravity) every sort overflows, and the result equals
    nsg_step followed by nsg_download."""
    rng = np.random.default_rng(9)
    n, ntie = 30000, 10000
    r = rng.uniform(0.1, 3.0, n)
    vr = rng.normal(0.0, 0.1, n)
    ell = rng.uniform(0.0, 0.5, n)
    tie = rng.choice(n, ntie, replace=False)
    r[tie], vr[tie], ell[tie] = 1.0, 0.0, 0.0
    ids = rng.permutation(n).astype(np.int32)
    kw = dict(dt=1e-3, G=0.0, max_subdiv=64, lc_rule=1, lc_radius=0.2, max_tau_steps=1_000_000)
    outs = []
    for overlapped in (False, True):
        with nsg.Context(nsg.default_params(**kw)) as c:
            c.upload(r, vr, ell, ids)
            if overlapped:
                outs.append(c.step_download(6))
            else:
                c.step(6)
                outs.append(c.download())
            assert c.status() & nsg.ST_SORT_FALLBACK
    for a, b in zip(*outs):
        assert np.array_equal(a, b)
