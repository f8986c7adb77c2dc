"""The learned level scheduler: the network's gradients against the CPU oracle,
the learned step against the plain step, and what training gains."""
import numpy as np
import pytest

from nsphere_gb300 import ics
from oracle import mlp_oracle as mo


def _batch(nb, seed):
    rng = np.random.default_rng(seed)
    X = rng.normal(0, 0.6, (nb, 4)).astype(np.float32)
    y = rng.integers(0, 8, nb).astype(np.int8)
    return X, y


def test_oracle_backward_matches_finite_differences():
    X, y = _batch(24, 1)
    cw = np.array([0.5, 1, 1, 2, 1, 1, 1, 3.0])
    w = mo.random_weights(3)
    loss, g = mo.forward_backward(w, X.astype(np.float64), y, cw, mode="exact")
    rng = np.random.default_rng(4)
    live = [k for k in range(mo.NPARAMS) if not (k < mo.H * mo.IN and k % mo.IN >= 4)]
    for k in rng.choice(live, 60, replace=False):
        e = 1e-6
        wp, wm = w.copy(), w.copy()
        wp[k] += e
        wm[k] -= e
        fd = (mo.forward_backward(wp, X.astype(np.float64), y, cw)[0] -
              mo.forward_backward(wm, X.astype(np.float64), y, cw)[0]) / (2 * e)
        assert abs(fd - g[k]) <= 1e-5 * max(1.0, abs(fd)), (k, fd, g[k])


def test_bf16_rounding_helper():
    x = np.array([1.0, 1.0 + 2 ** -8, 1.0 + 2 ** -7 + 2 ** -9, -3.14159, 0.0], dtype=np.float32)
    r = mo.bf16(x)
    assert r[0] == 1.0 and r[1] == 1.0          # tie rounds to even
    assert r[2] == 1.0 + 2 ** -7                # below the halfway point 1 + 2^-7 + 2^-8
    assert abs(r[3] + 3.140625) < 1e-12


@pytest.mark.gpu
def test_gpu_gradients_match_oracle(nsg):
    with nsg.Context(nsg.default_params()) as c:
        w = mo.random_weights(7).astype(np.float32)
        c.mlp_set_weights(w)
        w = c.mlp_weights().astype(np.float64)
        for nb, seed in ((16, 1), (100, 2), (4096, 3)):
            X, y = _batch(nb, seed)
            cw = np.array([0.25, 1, 1, 1, 2, 1, 1, 4.0], dtype=np.float32)
            gl, gg = c.mlp_grad(X, y, cw)
            ol, og = mo.forward_backward(w, X.astype(np.float64), y, cw.astype(np.float64), mode="bf16")
            assert abs(gl - ol) <= 1e-4 * abs(ol)
            for name, (a, b) in zip([s[0] for s in mo.SIZES],
                                    zip(np.split(gg.astype(np.float64), np.cumsum([np.prod(s[1]) for s in mo.SIZES])[:-1]),
                                        np.split(og, np.cumsum([np.prod(s[1]) for s in mo.SIZES])[:-1]))):
                err = np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-12)
                assert err < 2e-2, (name, nb, err)


@pytest.mark.gpu
def test_gpu_predictions_match_oracle(nsg):
    with nsg.Context(nsg.default_params()) as c:
        w = mo.random_weights(9).astype(np.float32)
        c.mlp_set_weights(w)
        X, _ = _batch(5000, 5)
        cls, lg = c.mlp_predict(X)
        ocls, olg = mo.predict(w.astype(np.float64), X.astype(np.float64))
        assert np.max(np.abs(lg - olg)) < 2e-2 * max(1.0, np.max(np.abs(olg)))
        top2 = np.sort(olg, axis=1)
        clear = (top2[:, -1] - top2[:, -2]) > 1e-2
        assert np.array_equal(cls[clear], ocls[clear])


@pytest.mark.gpu
@pytest.mark.parametrize("seed", [11, 12])
def test_learned_step_bit_identical_to_plain(nsg, oracle, seed):
    """Random networks send many particles straight to the level-parallel kernel;
    the results must equal the plain schedule and the oracle bit for bit."""
    n = 20000
    r, vr, ell, ids = ics.hernquist(n, seed=seed)
    perm = np.random.default_rng(seed).permutation(n)
    r, vr, ell, ids = r[perm], vr[perm], ell[perm], ids[perm]
    kw = dict(dt=5e-3, max_subdiv=256, lc_rule=1, lc_radius=3e-2, max_tau_steps=1_000_000)
    p = oracle.params(dt=5e-3, max_subdiv=256, lc_rule=1, lc_radius=3e-2)
    orr, ov, _, oid, olv, _ = oracle.step_adaptive(p, r, vr, ell, ids)
    with nsg.Context(nsg.default_params(sched=nsg.SCHED_LEARNED, **kw)) as c:
        c.mlp_set_weights(mo.random_weights(seed, scale=3.0).astype(np.float32))
        c.upload(r, vr, ell, ids)
        c.step(1)
        gr, gv, _, gid = c.download()
        glv = c.levels()
    assert np.array_equal(gid, oid)
    assert np.array_equal(glv, olv)
    assert np.array_equal(gr, orr) and np.array_equal(gv, ov)


@pytest.mark.gpu
def test_collect_train_and_gain(nsg):
    """Levels logged from plain steps train the network on the GPU; the trained
    network predicts deep particles far better than chance, and the learned
    schedule reproduces the plain step exactly."""
    n = 400_000
    r, vr, ell, ids = ics.hernquist(n, seed=4, r_a=1.0)
    kw = dict(dt=2e-3, max_subdiv=128, lc_rule=1, lc_radius=1e-3, max_tau_steps=1_000_000)
    with nsg.Context(nsg.default_params(**kw)) as c:
        c.upload(r, vr, ell, ids)
        c.mlp_init(3)
        c.mlp_collect(20, keep_level0=0.02, capacity=1 << 20)
        X, y = c.mlp_dataset()
        assert len(y) > 1000 and (y >= 1).sum() > 100
        loss0 = c.mlp_train(1, batch=1024, lr=3e-3)
        loss = c.mlp_train(20, batch=1024, lr=3e-3)
        assert loss < loss0
        cls, _ = c.mlp_predict(X)
        deep = y >= 1
        # recall of deep samples and precision of deep predictions
        recall = np.mean(cls[deep] >= 1)
        assert recall > 0.3
        w = c.mlp_weights()
        # learned and plain schedules agree exactly on the next step
        st = c.download()
    res = []
    for sched in (nsg.SCHED_PLAIN, nsg.SCHED_LEARNED):
        with nsg.Context(nsg.default_params(sched=sched, **kw)) as c:
            c.mlp_set_weights(w)
            c.upload(st[0], st[1], st[2], st[3])
            c.step(2)
            res.append(c.download())
    assert all(np.array_equal(a, b) for a, b in zip(res[0], res[1]))
