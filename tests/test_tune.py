"""Launch-shape tuning: the autotuner leaves the state untouched, every shape gives
the same results bit for bit, and bad shapes are rejected."""
import numpy as np
import pytest

from nsphere_gb300 import ics

pytestmark = pytest.mark.gpu

KW = dict(dt=1e-3, max_subdiv=128, lc_rule=1, lc_radius=2e-2, max_tau_steps=1_000_000)


def test_autotune_restores_state(nsg):
    r, vr, ell, ids = ics.hernquist(60000, seed=31)
    with nsg.Context(nsg.default_params(**KW)) as c:
        c.upload(r, vr, ell, ids)
        c.step(2)
        before = c.download()
        cnt, st = c.counters(), c.status()
        rep = c.autotune(steps=1)
        assert set(rep) == {"gather_level0", "bucket_shift", "levels", "chosen"}
        assert tuple(rep["chosen"]) == c.tune_get()
        assert c.counters() == cnt
        assert c.status() == st
        after = c.download()
        for a, b in zip(before, after):
            assert np.array_equal(a, b)


def test_shapes_do_not_change_results(nsg):
    r, vr, ell, ids = ics.hernquist(40000, seed=32)
    out = []
    for shape in [None, (128, 16, 10, 2), (512, 2, 12, 8), (256, 4, 8, 1), (256, 8, 9, 4), (256, 8, 11, 4)]:
        with nsg.Context(nsg.default_params(**KW)) as c:
            if shape is not None:
                c.tune_set(shape)
                assert c.tune_get() == shape
            c.upload(r, vr, ell, ids)
            c.step(3)
            if shape is not None:
                c.tune_set(shape[:2] + (shape[2] - 1 if shape[2] > 8 else 9,) + shape[3:])
            c.step(3)
            out.append(c.download())
    for o in out[1:]:
        for a, b in zip(out[0], o):
            assert np.array_equal(a, b)


def test_tuned_run_equals_default(nsg):
    r, vr, ell, ids = ics.hernquist(50000, seed=33)
    out = []
    for tune in (False, True):
        with nsg.Context(nsg.default_params(**KW)) as c:
            c.upload(r, vr, ell, ids)
            c.step(1)
            if tune:
                c.autotune(steps=1)
            c.step(4)
            out.append(c.download())
    for a, b in zip(*out):
        assert np.array_equal(a, b)


@pytest.mark.parametrize("bad", [(64, 4, 11, 4), (256, 0, 11, 4), (256, 4, 13, 4), (256, 4, 11, 65)])
def test_bad_shapes_rejected(nsg, bad):
    with nsg.Context(nsg.default_params()) as c:
        with pytest.raises(nsg.NsgError):
            c.tune_set(bad)
