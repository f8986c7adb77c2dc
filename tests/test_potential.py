"""Post-processing potential and energies (nsg_potential) against the reference's
sequential formulas (nsphere.c:7697-7846) restated in oracle.potential_energy."""
import numpy as np
import pytest

from nsphere_gb300 import ics
from oracle.oracle import potential_energy


def test_restatement_on_a_tiny_case():
    r = np.array([0.5, 1.0, 2.0])
    vr = np.array([0.1, -0.2, 0.3])
    ell = np.array([0.0, 0.5, 1.0])
    psi, E, psi0 = potential_energy(r, vr, ell)
    dM = 1.0 / 3
    assert psi[2] == pytest.approx(3 * dM / 2.0)
    assert psi[0] == pytest.approx(dM / 0.5 + dM * (1 / 1.0 + 1 / 2.0))
    assert psi0 == pytest.approx(dM * (2 + 1 + 0.5))
    assert E[1] == pytest.approx(psi[1] - 0.25 / 2 - 0.02)


@pytest.mark.gpu
@pytest.mark.parametrize("n", [1, 1000, 1023, 1024, 1025, 100_003])
def test_potential_matches_reference_formula(nsg, n):
    r, vr, ell, ids = ics.hernquist(n, seed=50 + n)
    with nsg.Context(nsg.default_params(dt=1e-3, max_subdiv=64, lc_rule=1, lc_radius=1e-2,
                                        max_tau_steps=1_000_000)) as c:
        c.upload(r, vr, ell, ids)
        if n > 1:
            c.step(2)                           # the state is no longer sorted: the call sorts it
        psi, E, psi0 = c.potential()
        sr, sv, sl, sid = c.download()
    assert np.all(np.diff(sr) >= 0)
    wpsi, wE, wpsi0 = potential_energy(sr, sv, sl)
    # the suffix sums are accumulated in a different order: agreement to rounding
    np.testing.assert_allclose(psi, wpsi, rtol=1e-12, atol=0)
    assert abs(psi0 / wpsi0 - 1) < 1e-12
    assert np.all(np.abs(E - wE) <= 1e-12 * np.abs(wpsi))
