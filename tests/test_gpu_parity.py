"""GPU parity: libnsg through its C ABI against the CPU oracle on identical inputs.

Bar: bit equality (sort permutation, r, v_r, levels) at sizes the oracle runs in
seconds, plus size-independent properties (sortedness, permutation, idempotence,
energy) at the full workload size.
"""
import numpy as np
import pytest

from conftest import golden
from nsphere_gb300 import ics

pytestmark = pytest.mark.gpu


def _shuffle(seed, *cols):
    perm = np.random.default_rng(seed).permutation(len(cols[0]))
    return tuple(c[perm] for c in cols)


def _ctx(nsg, **kw):
    # a finite Levi-Civita tau-step cap bounds the worst-case kernel time; none of
    # these cases comes near it, so results equal the oracle's (cap 1e8)
    kw.setdefault("max_tau_steps", 1_000_000)
    return nsg.Context(nsg.default_params(**kw))


# ------------------------------------------------------------------ sort

@pytest.mark.parametrize("n", [1, 2, 31, 4096, 4097, 100003])
def test_sort_matches_oracle_random(nsg, oracle, n):
    rng = np.random.default_rng(n)
    r = rng.lognormal(0, 2, n)
    vr, ell = rng.normal(size=n), rng.uniform(0, 1, n)
    ids = rng.permutation(n).astype(np.int32)
    with _ctx(nsg) as c:
        c.upload(r, vr, ell, ids)
        c.sort()
        gr, gv, gl, gid = c.download()
    orr, ov, ol, oid = oracle.sort(r, vr, ell, ids)
    assert np.array_equal(gid, oid)
    assert np.array_equal(gr, orr) and np.array_equal(gv, ov) and np.array_equal(gl, ol)


def test_sort_edge_keys(nsg, oracle):
    """ties (broken by id), -0.0 == +0.0, negative radii, inf, NaN last."""
    rng = np.random.default_rng(9)
    n = 50000
    r = rng.choice(np.array([0.0, -0.0, 1.0, 2.5, -3.0, np.inf, 1e-300, 5e-324]), n)
    r[rng.choice(n, 10, replace=False)] = np.nan
    ids = rng.permutation(n).astype(np.int32)
    z = np.zeros(n)
    with _ctx(nsg) as c:
        c.upload(r, z, z, ids)
        c.sort()
        gr, _, _, gid = c.download()
        assert c.status() & nsg.ST_NAN
    orr, _, _, oid = oracle.sort(r, z, z, ids)
    assert np.array_equal(gid, oid)
    assert np.array_equal(gr.view(np.uint64), orr.view(np.uint64))  # keeps -0.0 bits


def test_sort_matches_golden(nsg):
    g = golden("sort.npz")
    with nsg.Context(nsg.default_params(carry_aux=1)) as c:
        c.upload(g["r"], g["vr"], g["ell"], g["ids"], aux=g["mu"])
        c.sort()
        r, vr, ell, ids, mu = c.download(with_aux=True)
    out = g["out"]
    assert np.array_equal(r, out[0]) and np.array_equal(vr, out[1]) and np.array_equal(ell, out[2])
    assert np.array_equal(ids, out[3].astype(np.int32)) and np.array_equal(mu, out[4])


def test_sort_particles_dropin(nsg, oracle):
    rng = np.random.default_rng(4)
    n = 10000
    tab = np.ascontiguousarray(np.stack([rng.uniform(0, 5, n), rng.normal(size=n), rng.uniform(0, 1, n),
                                         rng.permutation(n).astype(np.float64), rng.uniform(-1, 1, n)]))
    want = oracle.sort(tab[0], tab[1], tab[2], tab[3].astype(np.int32), tab[4])
    with nsg.Context(nsg.default_params(carry_aux=1)) as c:
        nsg.sort_particles(c, tab)
    assert np.array_equal(tab[0], want[0]) and np.array_equal(tab[4], want[4])
    assert np.array_equal(tab[3].astype(np.int32), want[3])


def test_bad_ids_rejected(nsg):
    n = 100
    r = np.linspace(1, 2, n)
    ids = np.arange(n)
    ids[5] = 7  # duplicate
    with _ctx(nsg) as c:
        with pytest.raises(nsg.NsgError) as e:
            c.upload(r, r, r, ids)
        assert e.value.code == nsg.NSG_EIDS
        with pytest.raises(nsg.NsgError):
            c.upload(r, r, r, np.arange(n) + 0.5)


# ------------------------------------------------------------------ steps

def _adaptive_case(n, seed, lowl=0):
    r, vr, ell, ids = ics.hernquist(n, seed=seed)
    r, vr, ell, ids = _shuffle(seed, r, vr, ell, ids)
    ell = ell.copy()
    rng = np.random.default_rng(seed + 1)
    if lowl:
        k = rng.choice(n, lowl, replace=False)
        ell[k] = rng.uniform(0, 1e-4, lowl)
    inner = np.flatnonzero(r < 0.2)[:20]
    ell[inner] = np.sqrt(40.0 * r[inner] ** 3 / (1.0 + r[inner]) ** 2)
    return r, vr, ell, ids


@pytest.mark.parametrize("lc_rule,lc_radius,dt,msub,out_type", [
    (0, 1e-3, 5e-4, 128, 2),      # reference r_crit rule
    (1, 1e-1, 5e-4, 128, 2),      # fixed radius rule (many Levi-Civita particles)
    (1, 1.0, 5e-4, 128, 2),       # 5015 below the radius: more than the list before the sort holds
    (0, 1e-3, 5e-3, 1 << 12, 2),  # deeper levels (single-warp Levi-Civita kernel)
    (2, 1e-3, 2e-2, 64, 2),       # leapfrog only, level cap reached
    (1, 3e-2, 5e-4, 128, 0),      # coarse-pass output
    (1, 3e-2, 5e-4, 128, 1),      # fine-pass output
])
def test_adaptive_step_bit_exact(nsg, oracle, lc_rule, lc_radius, dt, msub, out_type):
    n = 20000
    r, vr, ell, ids = _adaptive_case(n, 21, lowl=100)
    with _ctx(nsg, dt=dt, max_subdiv=msub, lc_rule=lc_rule, lc_radius=lc_radius, out_type=out_type) as c:
        c.upload(r, vr, ell, ids)
        c.step(1)
        gr, gv, gl, gid = c.download()
        glv = c.levels()
        hist = c.level_hist(10)
    p = oracle.params(dt=dt, max_subdiv=msub, lc_rule=lc_rule, lc_radius=lc_radius, out_type=out_type)
    orr, ov, ol, oid, olv, cap = oracle.step_adaptive(p, r, vr, ell, ids)
    assert np.array_equal(gid, oid)
    assert np.array_equal(glv, olv), "accepted levels differ"
    bad = np.flatnonzero((gr != orr) | (gv != ov))
    assert bad.size == 0, "first mismatches at %s: gpu %s oracle %s" % (
        bad[:5], list(zip(gr[bad[:3]], gv[bad[:3]])), list(zip(orr[bad[:3]], ov[bad[:3]])))
    assert hist.sum() == n
    assert hist[-1] == np.sum(olv >= 99)


@pytest.mark.parametrize("lc_rule,lc_radius", [(0, 1e-3), (1, 5e-2)])
def test_method4_fixed_levi_civita_matches_oracle(nsg, oracle, lc_rule, lc_radius):
    """Method 4: adaptive leapfrog at tol 1e-8, fixed-dtau Levi-Civita leapfrog
    (N_taumin 1000) below r_crit (no rank-0 special case) or below lc_radius; three
    steps, graph replay included."""
    n, dt = 20000, 1e-3
    r, vr, ell, ids = _adaptive_case(n, 27, lowl=100)
    kw = dict(dt=dt, max_subdiv=128, tol_r=1e-8, tol_v=1e-8, N_taumin=1000, lc_rule=lc_rule, lc_radius=lc_radius)
    p = oracle.params(lc_fixed=1, **kw)
    cur = (r, vr, ell, ids)
    for _ in range(3):
        o = oracle.step_adaptive(p, *cur)
        cur = o[:4]
    with _ctx(nsg, method=nsg.METHOD_FULL_LC, **kw) as c:
        c.upload(r, vr, ell, ids)
        c.step(3)
        gr, gv, gl, gid = c.download()
        glv = c.levels()
    assert np.array_equal(gid, cur[3])
    assert np.array_equal(gr, cur[0]) and np.array_equal(gv, cur[1])
    assert np.array_equal(glv, o[4]) and np.sum(glv == 100) > 0


def test_method3_adaptive_leapfrog_only(nsg, oracle):
    """Method 3 (CLI --method 3, nsphere.c:5560-5615): adaptive leapfrog for every
    particle, with the reference's constants tol 1e-5, max_subdiv 1, coarse output."""
    n, dt = 20000, 1e-3
    r, vr, ell, ids = _adaptive_case(n, 29, lowl=100)
    kw = dict(dt=dt, max_subdiv=1, tol_r=1e-5, tol_v=1e-5, out_type=0)
    p = oracle.params(lc_rule=2, **kw)
    cur = (r, vr, ell, ids)
    for _ in range(4):
        cur = oracle.step_adaptive(p, *cur)[:4]
    with _ctx(nsg, method=nsg.METHOD_ADAPTIVE, **kw) as c:
        c.upload(r, vr, ell, ids)
        c.step(4)
        gr, gv, gl, gid = c.download()
    assert np.array_equal(gid, cur[3])
    assert np.array_equal(gr, cur[0]) and np.array_equal(gv, cur[1])


def test_method4_matches_golden(nsg):
    g = golden("method4.npz")
    tol = float(g["step_tol"])
    with _ctx(nsg, method=nsg.METHOD_FULL_LC, dt=float(g["dt"]), max_subdiv=int(g["step_msub"]), tol_r=tol,
              tol_v=tol, N_taumin=int(g["N_taumin"]), lc_rule=0) as c:
        c.upload(g["step_r"], g["step_vr"], g["step_ell"], g["step_ids"])
        c.step(1)
        r, vr, ell, ids = c.download()
    t = g["step_out"]
    assert np.array_equal(ids, t[3].astype(np.int32))
    assert np.array_equal(r, t[0]) and np.array_equal(vr, t[1])


def test_method5_matches_golden(nsg):
    g = golden("steps.npz")
    with _ctx(nsg, dt=float(g["dt5"]), max_subdiv=128, lc_rule=0) as c:
        c.upload(g["r"], g["vr"], g["ell"], g["ids"])
        c.step(1)
        r, vr, ell, ids = c.download()
        assert c.level_hist(10)[-1] > 0
    t = g["method5_rcrit"]
    assert np.array_equal(ids, t[3].astype(np.int32))
    assert np.array_equal(r, t[0]) and np.array_equal(vr, t[1])


def test_kdk_matches_golden_and_oracle(nsg, oracle):
    g = golden("steps.npz")
    s = g["kdk_start"]
    with _ctx(nsg, dt=float(g["dt_kdk"]), method=nsg.METHOD_KDK) as c:
        c.upload(s[0], s[1], s[2], s[3])
        c.step(5)
        r, vr, ell, ids = c.download()
    t = g["kdk5"]
    assert np.array_equal(ids, t[3].astype(np.int32))
    assert np.array_equal(r, t[0]) and np.array_equal(vr, t[1])
    # longer run against the oracle on a Plummer sphere
    n = 30000
    r0, v0, l0, i0 = ics.plummer(n, seed=1)
    p = oracle.params(dt=1e-3)
    cur = (r0, v0, l0, i0)
    for _ in range(20):
        cur = oracle.step_kdk(p, *cur)
    with _ctx(nsg, dt=1e-3, method=nsg.METHOD_KDK) as c:
        c.upload(r0, v0, l0, i0)
        c.step(20)
        r, vr, ell, ids = c.download()
    assert np.array_equal(ids, cur[3]) and np.array_equal(r, cur[0]) and np.array_equal(vr, cur[1])


def test_multi_step_adaptive(nsg, oracle):
    n = 8000
    r, vr, ell, ids = _adaptive_case(n, 33)
    p = oracle.params(dt=1e-3, max_subdiv=128, lc_rule=1, lc_radius=3e-2)
    cur = (r, vr, ell, ids)
    for _ in range(10):
        o = oracle.step_adaptive(p, *cur)
        cur = o[:4]
    with _ctx(nsg, dt=1e-3, max_subdiv=128, lc_rule=1, lc_radius=3e-2) as c:
        c.upload(r, vr, ell, ids)
        c.step(10)
        gr, gv, gl, gid = c.download()
    assert np.array_equal(gid, cur[3]) and np.array_equal(gr, cur[0]) and np.array_equal(gv, cur[1])


@pytest.mark.parametrize("method", [2, 5])
def test_point_mass_ramp_matches_oracle(nsg, oracle, method):
    """Central point mass (the stress configuration; not in the reference): every step
    uses the current mass in the gravity numerator, then the mass grows by rate*dt."""
    n, dt, m0, rate = 12000, 1e-3, 1e-3, 0.5
    # in radial order, as the reference sorts once before its time loop (nsphere.c:5339-5342)
    r, vr, ell, ids = oracle.sort(*_adaptive_case(n, 44, lowl=200))
    kw = dict(dt=dt, max_subdiv=64, lc_rule=1, lc_radius=2e-2) if method == 5 else dict(dt=dt)
    p = oracle.params(point_mass=m0, **kw)
    cur = (r, vr, ell, ids)
    for _ in range(6):
        cur = (oracle.step_adaptive(p, *cur) if method == 5 else oracle.step_kdk(p, *cur))[:4]
        p.point_mass = p.point_mass + rate * dt
    srt = oracle.sort(*cur)                  # energies are taken over the current radial order
    K, W = oracle.energy(p, srt[0], srt[1], srt[2])
    with _ctx(nsg, method=method, point_mass=m0, point_mass_rate=rate, **kw) as c:
        c.upload(r, vr, ell, ids)
        c.step(6)
        gr, gv, gl, gid = c.download()
        gK, gW = c.energy()
    assert np.array_equal(gid, cur[3]) and np.array_equal(gr, cur[0]) and np.array_equal(gv, cur[1])
    assert gK == pytest.approx(K, rel=1e-12) and gW == pytest.approx(W, rel=1e-12)


@pytest.mark.parametrize("nf_stop", [1, 0])
@pytest.mark.parametrize("lc_rule", [1, 2])
def test_nonfinite_rule_matches_oracle(nsg, oracle, nf_stop, lc_rule):
    """A near-radial particle at the centre with a central mass (found in the N = 1e8
    point-mass run): its Levi-Civita tau-step overflows in the coarse passes.  With
    nonfinite_stop = 1 the climb ends there (non-finite radius); with 0 it climbs on to
    the fallback pass as the reference does (finite result).  lc_rule 2 sends the same
    particle, and one at r = 0, through the leapfrog.  GPU and oracle agree either way."""
    pm = float.fromhex("0x1.f75104d551d69p-14")
    n = 2000
    r, vr, ell, ids = ics.hernquist(n, seed=9)
    r, vr, ell = r.copy(), vr.copy(), ell.copy()
    r[0] = float.fromhex("0x1.0aa796db64b39p-19")
    vr[0] = float.fromhex("-0x1.24c0ac2752822p+3")
    ell[0] = float.fromhex("0x1.d1834db7f4eddp-20")
    if lc_rule == 2:
        r[1] = 0.0
    kw = dict(dt=5e-4, max_subdiv=128, lc_rule=lc_rule, lc_radius=1e-3, max_tau_steps=2000, point_mass=pm)
    p = oracle.params(nonfinite_stop=nf_stop, **kw)
    orr, ov, ol, oid, olv, cap = oracle.step_adaptive(p, r, vr, ell, ids)
    with _ctx(nsg, nonfinite_stop=nf_stop, **kw) as c:
        c.upload(r, vr, ell, ids)
        c.step(1)
        gr, gv, gl, gid = c.download()
        glv = c.levels()
    assert np.array_equal(gid, oid) and np.array_equal(glv, olv)
    assert np.array_equal(gr, orr, equal_nan=True) and np.array_equal(gv, ov, equal_nan=True)
    if lc_rule == 1:
        k = np.flatnonzero(gid == 0)[0]
        assert np.isnan(gr[k]) == bool(nf_stop)


def test_energy_and_gather(nsg, oracle):
    n = 50000
    r, vr, ell, ids = ics.plummer(n, seed=5)
    r, vr, ell, ids = _shuffle(5, r, vr, ell, ids)
    with _ctx(nsg) as c:
        c.upload(r, vr, ell, ids)
        K, W = c.energy()
        sr, sv, sl, sid = c.download()
        q = np.array([0, 1, 2, 17, n - 1], dtype=np.int32)
        gr, gv, gl, rank = c.gather(q)
    p = oracle.params()
    oK, oW = oracle.energy(p, sr, sv, sl)
    assert abs(K - oK) <= 1e-12 * abs(oK) and abs(W - oW) <= 1e-12 * abs(oW)
    # virial ratio of an equilibrium Plummer sphere is close to 1
    assert 0.9 < 2 * K / abs(W) < 1.1
    assert np.array_equal(sid[rank], q)
    assert np.array_equal(gr, sr[rank]) and np.array_equal(gv, sv[rank])


def test_gather_before_any_sort(nsg):
    n = 1000
    rng = np.random.default_rng(0)
    r = rng.uniform(0, 1, n)
    ids = rng.permutation(n)
    with _ctx(nsg) as c:
        c.upload(r, r, r, ids)
        gr, _, _, rank = c.gather(np.array([ids[10], ids[500]], dtype=np.int32))
    assert list(rank) == [10, 500] and gr[0] == r[10]


# ----------------------------------------------------------- large sizes

def test_large_sort_properties(nsg):
    """At the workload size: output sorted by (r, id), a permutation, idempotent."""
    n = 10_000_000
    r, vr, ell, ids = ics.hernquist(n, seed=2)
    r, vr, ell, ids = _shuffle(2, r, vr, ell, ids)
    with _ctx(nsg) as c:
        c.upload(r, vr, ell, ids)
        c.sort()
        sr, sv, sl, sid = c.download()
        c.sort()
        sr2, _, _, sid2 = c.download()
    assert np.all(np.diff(sr) >= 0)
    eq = np.flatnonzero(np.diff(sr) == 0)
    assert np.all(sid[eq] < sid[eq + 1])
    assert np.array_equal(np.sort(sid), np.arange(n))
    assert np.array_equal(sid, sid2) and np.array_equal(sr, sr2)
    # the payload travelled with its key
    src = np.empty(n, dtype=np.int64)
    src[ids] = np.arange(n)
    assert np.array_equal(sv, vr[src[sid]]) and np.array_equal(sl, ell[src[sid]])


@pytest.mark.parametrize("dt, bound", [(5e-4, 3e-6), (4e-5, 2e-8)])
def test_energy_drift_matches_oracle_n1e6(nsg, oracle, dt, bound):
    """N = 1e6 Hernquist, 20 adaptive steps: the state equals the oracle's bit for bit,
    so its drift is the oracle's; the drift grows as dt^2 per step (about 1e-7 per step
    at dt = 5e-4, 6e-10 at the bench's 4e-5), and stays within that bound."""
    n = 1_000_000
    r, vr, ell, ids = ics.hernquist(n, seed=2)
    kw = dict(dt=dt, max_subdiv=128, lc_rule=1, lc_radius=1e-3)
    with _ctx(nsg, **kw) as c:
        c.upload(r, vr, ell, ids)
        E0 = sum(c.energy())
        c.step(20)
        gpu = c.download()
        E1 = sum(c.energy())
        st = c.status()
    p = oracle.params(**kw)
    cur = (r, vr, ell, ids)
    for _ in range(20):
        cur = oracle.step_adaptive(p, *cur)[:4]
    for g, o in zip(gpu, cur):
        assert np.array_equal(g, o)
    srt = oracle.sort(*cur)
    s0 = oracle.sort(r, vr, ell, ids)
    e0 = sum(oracle.energy(p, s0[0], s0[1], s0[2]))
    e1 = sum(oracle.energy(p, srt[0], srt[1], srt[2]))
    assert abs(abs(E1 - E0) / abs(E0) - abs(e1 - e0) / abs(e0)) <= 2e-12
    assert abs(E1 - E0) / abs(E0) < bound
    assert not (st & nsg.ST_TAU_CAP)


def test_integer_pipe_division_matches_ieee(nsg):
    """The integrators divide on the integer/FP32 pipes; every result must carry the
    same bits as the hardware IEEE division."""
    total = 0
    for seed in (1, 2, 3):
        mism, fast, first = nsg.selftest_division(200_000_000, seed=seed)
        assert mism == 0, "first mismatch a=%r b=%r" % first
        total += fast
    assert total > 0.5 * 600_000_000  # most pairs take the integer path


@pytest.mark.parametrize("ntie", [100, 30000])
def test_near_sorted_sort_ties_and_overflow(nsg, oracle, ntie):
    """Second sort of a state runs the near-sorted bucket path: equal radii are
    ordered by id inside a bucket; a tie run larger than a bucket overflows it and
    the radix sort takes over."""
    rng = np.random.default_rng(ntie)
    n = 120_000
    r = rng.uniform(0.0, 2.0, n)
    r[rng.choice(n, ntie, replace=False)] = 1.0
    ids = rng.permutation(n).astype(np.int32)
    z = rng.normal(size=n)
    with _ctx(nsg) as c:
        c.upload(r, z, z, ids)
        c.sort()
        c.clear_status()
        c.sort()
        gr, gv, _, gid = c.download()
        st = c.status()
    orr, ov, _, oid = oracle.sort(r, z, z, ids)
    assert np.array_equal(gid, oid) and np.array_equal(gr, orr) and np.array_equal(gv, ov)
    assert bool(st & nsg.ST_SORT_FALLBACK) == (ntie > 6144)


def test_near_sorted_sort_after_moves(nsg, oracle):
    """Sorts after each of 30 KDK steps with a large dt (many rank crossings) use
    the bucket path and stay bit-exact."""
    n = 50_000
    r0, v0, l0, i0 = ics.plummer(n, seed=8)
    p = oracle.params(dt=2e-2)
    cur = (r0, v0, l0, i0)
    for _ in range(30):
        cur = oracle.step_kdk(p, *cur)
    with _ctx(nsg, dt=2e-2, method=nsg.METHOD_KDK) as c:
        c.upload(r0, v0, l0, i0)
        c.step(30)
        r, vr, ell, ids = c.download()
    assert np.array_equal(ids, cur[3]) and np.array_equal(r, cur[0]) and np.array_equal(vr, cur[1])


@pytest.mark.gpu
@pytest.mark.parametrize("method", [5, 4, 2])
def test_step_download_equals_step_then_download(nsg, method):
    """nsg_step_download overlaps the last step's copy with its Levi-Civita chains and
    patches the chains' particles in: the arrays equal nsg_step + nsg_download."""
    n = 50000
    r, vr, ell, ids = _adaptive_case(n, 51, lowl=200)
    kw = dict(dt=1e-3, max_subdiv=64, lc_rule=1, lc_radius=5e-2) if method != 2 else dict(dt=1e-3)
    outs = []
    for overlapped in (False, True):
        with _ctx(nsg, method=method, **kw) as c:
            c.upload(r, vr, ell, ids)
            if overlapped:
                outs.append(c.step_download(3))
            else:
                c.step(3)
                outs.append(c.download())
    for a, b in zip(*outs):
        assert np.array_equal(a, b)


def test_config1_full_run_matches_oracle(nsg, oracle):
    """The whole fixed-step configuration: N = 1e5 Plummer, dt = 1e-3, 1000 KDK steps,
    bit for bit against the oracle (which the reference's functions pin)."""
    n, steps = 100_000, 1000
    r0, v0, l0, i0 = oracle.sort(*ics.plummer(n, seed=1))
    p = oracle.params(dt=1e-3)
    cur = (r0, v0, l0, i0)
    for _ in range(steps):
        cur = oracle.step_kdk(p, *cur)
    with _ctx(nsg, dt=1e-3, method=nsg.METHOD_KDK) as c:
        c.upload(r0, v0, l0, i0)
        c.step(steps)
        r, vr, ell, ids = c.download()
        assert c.status() == 0
    assert np.array_equal(ids, cur[3]) and np.array_equal(r, cur[0]) and np.array_equal(vr, cur[1])


def test_step_download_carries_aux(nsg):
    n = 30000
    r, vr, ell, ids = _adaptive_case(n, 53, lowl=100)
    mu = np.random.default_rng(3).uniform(-1, 1, n)
    outs = []
    for overlapped in (False, True):
        with _ctx(nsg, dt=1e-3, max_subdiv=64, lc_rule=1, lc_radius=5e-2, carry_aux=1) as c:
            c.upload(r, vr, ell, ids, mu)
            if overlapped:
                outs.append(c.step_download(2, with_aux=True))
            else:
                c.step(2)
                outs.append(c.download(with_aux=True))
    for a, b in zip(*outs):
        assert np.array_equal(a, b)


def test_reupload_keeps_splitters_and_results(nsg, oracle):
    """A driver that uploads its host state every step: the previous sort's splitters
    stay in use when the halo table is unchanged.  Re-uploading the downloaded state
    continues bit for bit like uninterrupted steps.  The buckets are key ranges, so a
    shuffled state of the same distribution sorts through them as well; a state whose
    radii lie elsewhere overflows them and the radix sort takes over.  Both are exact."""
    n = 60_000
    r, vr, ell, ids = _adaptive_case(n, 61, lowl=150)
    kw = dict(dt=1e-3, max_subdiv=64, lc_rule=1, lc_radius=5e-2)
    p = oracle.params(**kw)
    cur = (r, vr, ell, ids)
    for _ in range(5):
        cur = oracle.step_adaptive(p, *cur)[:4]
    with _ctx(nsg, **kw) as c:
        c.upload(r, vr, ell, ids)
        c.step(2)
        mid = c.download()
        for _ in range(3):
            c.upload(*mid)
            c.step(1)
            mid = c.download()
        for g, o in zip(mid, cur):
            assert np.array_equal(g, o)
        # unrelated states of the same size: shuffled, same distribution; then radii
        # twenty times larger (all above the old splitters but the last few)
        r2, v2, l2, i2 = _shuffle(7, *_adaptive_case(n, 62, lowl=0))
        for scale, fallback in ((1.0, False), (20.0, True)):
            c.clear_status()
            c.upload(r2 * scale, v2, l2, i2)
            c.sort()
            got = c.download()
            assert bool(c.status() & nsg.ST_SORT_FALLBACK) == fallback
            want = oracle.sort(r2 * scale, v2, l2, i2)
            for g, o in zip(got, want):
                assert np.array_equal(g, o)


@pytest.mark.parametrize("method", [2, 5])
def test_aux_column_follows_particles_through_fused_sorts(nsg, oracle, method):
    """carry_aux = 1: the fifth column (mu) is permuted with the state by every sort,
    including the sorts done inside the fused kernels; r, v_r, ell and the order equal
    the oracle's (which has no fifth column) and mu stays attached to its particle."""
    n = 40_000
    r, vr, ell, ids = _adaptive_case(n, 71, lowl=100)
    mu = np.cos(ids.astype(np.float64) * 0.001)          # a function of the id
    kw = dict(dt=1e-3, max_subdiv=64, lc_rule=1, lc_radius=5e-2) if method == 5 else dict(dt=1e-3)
    p = oracle.params(**kw)
    cur = (r, vr, ell, ids) if method == 5 else oracle.sort(r, vr, ell, ids)
    for _ in range(6):
        cur = (oracle.step_adaptive(p, *cur)[:4] if method == 5 else oracle.step_kdk(p, *cur))
    with _ctx(nsg, method=method, carry_aux=1, **kw) as c:
        c.upload(r, vr, ell, ids, mu)
        c.step(6)
        gr, gv, gl, gid, gmu = c.download(with_aux=True)
    assert np.array_equal(gid, cur[3]) and np.array_equal(gr, cur[0]) and np.array_equal(gv, cur[1])
    assert np.array_equal(gl, cur[2])
    assert np.array_equal(gmu, np.cos(gid.astype(np.float64) * 0.001))


@pytest.mark.parametrize("consumer", ["sort", "step"])
def test_fused_sort_with_empty_buckets(nsg, oracle, consumer):
    """Buckets that receive no particle: the sort's own splitters are kept across an
    upload of a state in which every particle of buckets 0, 5 and 20 (1024 sorted
    positions each) moved into the neighbouring buckets' key ranges.  Their blocks sort
    nothing but still publish where the next bucket starts (the look-back over the
    bucket counts); the fused sort (nsg_sort: rank force; nsg_step: adaptive level 0)
    equals the oracle's with no fallback to the radix sort."""
    n, B = 60_000, 1024
    r, vr, ell, ids = _adaptive_case(n, 71, lowl=0)
    kw = dict(dt=1e-3, max_subdiv=64, lc_rule=1, lc_radius=5e-2)
    with _ctx(nsg, **kw) as c:
        c.upload(r, vr, ell, ids)
        c.sort()                                   # splitters: keys at positions b * 1024
        sr, sv, sl, si = (a.copy() for a in c.download())
        rng = np.random.default_rng(5)
        mr = sr.copy()
        for b in (0, 5, 20):
            lo, hi = b * B, (b + 1) * B
            if b == 0:                              # all into bucket 1
                mr[lo:hi] = rng.uniform(sr[B], sr[2 * B], B)
            else:                                   # halves into buckets b - 1 and b + 1
                mr[lo:lo + B // 2] = rng.uniform(sr[(b - 1) * B], sr[b * B], B // 2)
                mr[lo + B // 2:hi] = rng.uniform(sr[(b + 1) * B], sr[(b + 2) * B], B // 2)
        c.clear_status()
        c.upload(mr, sv, sl, si)
        if consumer == "sort":
            c.sort()
            got = c.download()
            want = oracle.sort(mr, sv, sl, si)
        else:
            c.step(1)
            got = c.download()
            want = oracle.step_adaptive(oracle.params(**kw), mr, sv, sl, si)[:4]
        assert not c.status() & nsg.ST_SORT_FALLBACK
    for g, o in zip(got, want):
        assert np.array_equal(g, o)
