"""Initial conditions generated on the GPU (nsg_generate) against the numpy
restatement of the same counter-based generators, and against the models'
analytic distributions."""
import numpy as np
import pytest

from nsphere_gb300 import ics


def test_counter_draws_are_uniform():
    u = ics.counter_uniform(7, np.arange(200_000, dtype=np.uint64), 3)
    assert 0.0 <= u.min() and u.max() < 1.0
    assert abs(u.mean() - 0.5) < 3e-3 and abs(u.var() - 1 / 12) < 2e-3
    # different draw indices and seeds are different streams
    assert not np.array_equal(u, ics.counter_uniform(7, np.arange(200_000, dtype=np.uint64), 4))
    assert not np.array_equal(u, ics.counter_uniform(8, np.arange(200_000, dtype=np.uint64), 3))


def test_restated_generators_follow_the_models():
    r, vr, ell, ids, mu = ics.hernquist_counter(200_000, seed=5, r_max=100.0)
    m = (r / (1 + r)) ** 2 / (100.0 / 101.0) ** 2           # M(<r) / M(<r_max), uniform if right
    assert abs(np.sort(m) - (np.arange(m.size) + 0.5) / m.size).max() < 5e-3
    # isotropy: <v_r^2> = <v_t^2> / 2 with v_t = ell / r
    assert abs(np.mean(vr ** 2) / np.mean((ell / r) ** 2) - 0.5) < 0.02
    r, vr, ell, ids, mu = ics.plummer_counter(200_000, seed=5)
    m = r ** 3 / (1 + r * r) ** 1.5
    assert abs(np.sort(m) - (np.arange(m.size) + 0.5) / m.size).max() < 5e-3
    # virial equilibrium: 2K + W = 0 with W = -3 pi / 32 for the Plummer sphere
    K = 0.5 * np.mean(vr ** 2 + (ell / r) ** 2)
    assert abs(2 * K / (3 * np.pi / 32) - 1) < 0.02


@pytest.mark.gpu
@pytest.mark.parametrize("model,n", [(1, 100_003), (2, 150_001), (2, 300)])
def test_gpu_generator_matches_restatement(nsg, model, n):
    seed = 11 + model
    with nsg.Context(nsg.default_params(carry_aux=1)) as c:
        c.generate(model, n, seed, 100.0)
        assert c.status() & nsg.ST_IC_REJECT == 0
        r, vr, ell, ids, mu = c.download(with_aux=True)
    want = ics.plummer_counter(n, seed) if model == 1 else ics.hernquist_counter(n, seed, 100.0)
    assert np.array_equal(ids, np.arange(n))
    # pow (Plummer radii) and asin (Hernquist f(E)) are not correctly rounded on either
    # side.  Hernquist radii use only correctly rounded operations; the Plummer radius
    # r = (u^(-2/3) - 1)^(-1/2) amplifies pow's few-ulp difference by up to
    # 1 / (2 (u^(-2/3) - 1)) = r^2 / 2, about 1e5 at the largest radii of 1e5 draws.
    rtol = 1e-10 if model == 1 else 1e-13
    if model == 2:
        # every value is a chain of correctly rounded operations on the same draws
        # (asin only decides acceptances, which agree): bit-identical
        for got, w in zip((r, vr, ell), want[:3]):
            assert np.array_equal(got, w)
    np.testing.assert_allclose(r, want[0], rtol=rtol, atol=0)
    assert np.array_equal(mu, want[4])
    np.testing.assert_allclose(vr, want[1], rtol=rtol, atol=1e-300)
    np.testing.assert_allclose(ell, want[2], rtol=rtol, atol=1e-300)


@pytest.mark.gpu
def test_generated_state_steps(nsg, oracle):
    """A generated state is an ordinary resident state: one adaptive step equals the
    oracle's step of the downloaded state."""
    with nsg.Context(nsg.default_params(dt=1e-3, max_subdiv=64, lc_rule=1, lc_radius=1e-2,
                                        max_tau_steps=1_000_000)) as c:
        c.generate(nsg.IC_HERNQUIST, 20_000, 3, 100.0)
        r, vr, ell, ids = c.download()
        c.step(1)
        gr, gv, gl, gid = c.download()
    p = oracle.params(dt=1e-3, max_subdiv=64, lc_rule=1, lc_radius=1e-2)
    orr, ov, ol, oid, olv, cap = oracle.step_adaptive(p, r, vr, ell, ids)
    assert np.array_equal(gid, oid) and np.array_equal(gr, orr) and np.array_equal(gv, ov)


def test_om_closed_form_matches_eddington_inversion():
    """The Osipkov-Merritt f(Q) of nsg_generate_om against a numerical Eddington
    inversion of rho_Q = (1 + r^2/r_a^2) rho (ics._om_df_table)."""
    Q = np.array([0.05, 0.1, 0.2, 0.4, 0.6, 0.8])
    for r_a in (0.75, 1.0, 3.0):
        Qt, ft = ics._om_df_table(r_a)
        want = np.interp(Q, Qt, ft)
        got = ics.hernquist_df(Q) + np.sqrt(Q) * (1 - 2 * Q) / (np.sqrt(2) * np.pi ** 3 * r_a ** 2)
        np.testing.assert_allclose(got, want, rtol=2e-3)


def test_om_restatement_has_the_model_anisotropy():
    r_a = 1.0
    r, vr, ell, ids, mu = ics.hernquist_om_counter(300_000, seed=9, r_max=100.0, r_a=r_a)
    m = (r / (1 + r)) ** 2 / (100.0 / 101.0) ** 2
    assert abs(np.sort(m) - (np.arange(m.size) + 0.5) / m.size).max() < 5e-3
    # beta(r) = 1 - <v_t^2> / (2 <v_r^2>) = r^2 / (r^2 + r_a^2) for Osipkov-Merritt
    vt2 = (ell / r) ** 2
    for lo, hi in ((0.1, 0.3), (0.8, 1.25), (3.0, 6.0)):
        sel = (r > lo) & (r < hi)
        beta = 1 - np.mean(vt2[sel]) / (2 * np.mean(vr[sel] ** 2))
        rm = np.sqrt(lo * hi)
        assert abs(beta - rm ** 2 / (rm ** 2 + r_a ** 2)) < 0.05, (lo, hi, beta)


@pytest.mark.gpu
@pytest.mark.parametrize("r_a,n", [(1.0, 150_001), (2.5, 20_000)])
def test_gpu_om_generator_matches_restatement(nsg, r_a, n):
    seed = 17
    with nsg.Context(nsg.default_params(carry_aux=1)) as c:
        c.generate_om(n, seed, 100.0, r_a)
        assert c.status() & nsg.ST_IC_REJECT == 0
        r, vr, ell, ids, mu = c.download(with_aux=True)
    want = ics.hernquist_om_counter(n, seed, 100.0, r_a)
    assert np.array_equal(ids, np.arange(n))
    for got, w in zip((r, vr, ell, mu), (want[0], want[1], want[2], want[4])):
        assert np.array_equal(got, w)
