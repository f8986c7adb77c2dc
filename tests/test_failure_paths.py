"""Failure detection through the C ABI, in forms that fault, trap or hang no GPU:

* a Levi-Civita particle that exhausts a small max_tau_steps: the kernel stops at the
  cap with the reference's "best available result" (nsphere.c:2320-2329), sets
  NSG_ST_TAU_CAP, and nsg_sync reports NSG_EDEVICE; the result equals the oracle's
  under the same cap;
* an absurd particle count: nsg_upload / nsg_generate return NSG_ENOMEM before any
  device allocation or copy, and the context stays usable and destroyable;
* nsg_sync with a zero timeout while steps are queued returns NSG_ETIMEOUT, and a
  later unbounded sync succeeds.
The host-side argument checks (null pointers, bad ids, bad parameters) need no GPU
beyond context creation and are covered in test_abi.py / test_gpu_parity.py.
"""
import ctypes as C

import numpy as np
import pytest

from nsphere_gb300 import ics

pytestmark = pytest.mark.gpu


def test_tau_cap_sets_status_and_sync_reports_edevice(nsg, oracle):
    n = 3000
    r, vr, ell, ids = ics.hernquist(n, seed=31)
    # three particles inside the Levi-Civita radius on near-radial orbits
    r[:3] = [2e-4, 5e-4, 8e-4]
    ell[:3] = [1e-7, 0.0, 3e-6]
    vr[:3] = [0.5, -0.3, 0.1]
    cap = 4      # a step takes ~2 N_taumin = 20 tau-steps
    kw = dict(dt=5e-4, max_subdiv=128, lc_rule=1, lc_radius=1e-3)
    p = nsg.default_params(method=nsg.METHOD_ADAPTIVE_LC, max_tau_steps=cap, **kw)
    with nsg.Context(p) as c:
        c.upload(r, vr, ell, ids)
        c.step(1)
        with pytest.raises(nsg.NsgError) as ei:
            c.sync(-1)
        assert ei.value.code == nsg.NSG_EDEVICE
        assert c.status() & nsg.ST_TAU_CAP
        gpu = c.download()
        # the status word is sticky until cleared; afterwards sync succeeds again
        c.clear_status()
        c.sync(-1)
    op = oracle.params(max_tau_steps=cap, **kw)
    orc = oracle.step_adaptive(op, r, vr, ell, ids)
    assert orc[5] > 0              # the oracle hit the cap too
    for g, o in zip(gpu, orc[:4]):
        assert np.array_equal(g, o)


def test_absurd_n_returns_enomem_and_context_survives(nsg):
    L = nsg.lib()
    small = np.zeros(16)
    with nsg.Context(nsg.default_params()) as c:
        # 2^31 - 1 particles need ~390 GB of device buffers: refused before allocating
        # (the host columns are never read: the count is checked first)
        P = C.c_void_p(small.ctypes.data)
        rc = L.nsg_upload(c.handle, P, P, P, P, None, (1 << 31) - 1)
        assert rc == nsg.NSG_ENOMEM, L.nsg_last_error(c.handle)
        assert b"device" in L.nsg_last_error(c.handle)
        rc = L.nsg_generate(c.handle, nsg.IC_PLUMMER, (1 << 31) - 1, 1, 100.0)
        assert rc == nsg.NSG_ENOMEM
        # still usable
        r, vr, ell, ids = ics.plummer(1000, seed=3)
        c.upload(r, vr, ell, ids)
        c.step(2)
        assert len(c.download()[0]) == 1000
    # a context that never held a state is destroyable after the failure too
    c2 = nsg.Context(nsg.default_params())
    P = C.c_void_p(small.ctypes.data)
    assert L.nsg_upload(c2.handle, P, P, P, P, None, (1 << 31) - 1) == nsg.NSG_ENOMEM
    c2.close()


def test_sync_timeout_then_normal_sync(nsg):
    n = 2_000_000
    with nsg.Context(nsg.default_params(dt=5e-4, max_subdiv=128, lc_rule=1, lc_radius=1e-3,
                                        max_tau_steps=1_000_000)) as c:
        c.generate(nsg.IC_HERNQUIST, n, 5, 100.0)
        c.step(2)
        c.sync(-1)
        c.step(200)                # queued; ~0.5 ms of GPU work per step
        with pytest.raises(nsg.NsgError) as ei:
            c.sync(0)
        assert ei.value.code == nsg.NSG_ETIMEOUT
        c.sync(-1)
        assert len(c.download()[0]) == n
