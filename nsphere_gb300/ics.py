"""Seeded initial conditions in G = M = a = 1 units (host side, numpy).

Each generator returns ``(r, vr, ell, ids)``: float64 radius, radial velocity,
specific angular momentum, and int32 ids equal to the initial radial rank (the
reference remaps ids to 0..N-1 in sorted order, nsphere.c:4908-4920).  Directions
use the reference's mapping v_r = v mu, ell = r v sqrt(1 - mu^2) with mu uniform in
[-1, 1] (nsphere.c:4805-4808, 4914).

* Plummer: inverse-CDF radii r = (u^(-2/3) - 1)^(-1/2) and the Aarseth, Henon &
  Wielen (1974) rejection for the speed ratio q = v / v_esc.
* Hernquist (1990): inverse-CDF radii of M(r) = r^2/(1+r)^2 truncated at r_max,
  speeds from the isotropic distribution function f(E) by rejection; with
  ``r_a`` set, Osipkov-Merritt anisotropy with f(Q) from a numerical Eddington
  inversion of rho_Q = (1 + r^2/r_a^2) rho.
"""
from __future__ import annotations

import numpy as np


def _finish(r, v, mu, rng=None):
    order = np.argsort(r, kind="stable")
    r, v, mu = r[order], v[order], mu[order]
    vr = v * mu
    ell = r * v * np.sqrt(np.maximum(0.0, 1.0 - mu * mu))
    ids = np.arange(r.shape[0], dtype=np.int32)
    return r.astype(np.float64), vr.astype(np.float64), ell.astype(np.float64), ids


def plummer(n: int, seed: int = 1):
    rng = np.random.Generator(np.random.PCG64(seed))
    u = rng.uniform(1e-10, 1.0, n)
    r = 1.0 / np.sqrt(u ** (-2.0 / 3.0) - 1.0)
    q = np.empty(n)
    todo = np.arange(n)
    while todo.size:
        x1 = rng.uniform(0.0, 1.0, todo.size)
        x2 = rng.uniform(0.0, 1.0, todo.size)
        ok = 0.1 * x2 < x1 * x1 * (1.0 - x1 * x1) ** 3.5
        q[todo[ok]] = x1[ok]
        todo = todo[~ok]
    v = q * np.sqrt(2.0) * (1.0 + r * r) ** -0.25
    mu = rng.uniform(-1.0, 1.0, n)
    return _finish(r, v, mu)


def plummer_ensemble(nhalo: int, nmin: int = 10_000, nmax: int = 1_000_000, seed: int = 3):
    """Independent Plummer halos with N drawn log-uniform in [nmin, nmax] (seeded).

    Returns (r, vr, ell, ids, halo_n): the halos' rows concatenated, each halo in
    radial order, ids = row index (so halo h owns the ids of its own row range)."""
    rng = np.random.Generator(np.random.PCG64(seed))
    sizes = np.floor(10.0 ** rng.uniform(np.log10(nmin), np.log10(nmax), nhalo)).astype(np.int64)
    parts = [plummer(int(nh), seed=seed * 100003 + h) for h, nh in enumerate(sizes)]
    r = np.concatenate([p[0] for p in parts])
    vr = np.concatenate([p[1] for p in parts])
    ell = np.concatenate([p[2] for p in parts])
    ids = np.arange(r.shape[0], dtype=np.int32)
    return r, vr, ell, ids, sizes


def hernquist_df(eps):
    """Isotropic Hernquist f(E) for binding energy eps = -E in (0, 1), G = M = a = 1."""
    q = np.sqrt(np.clip(eps, 0.0, 1.0 - 1e-15))
    q2 = q * q
    val = (3.0 * np.arcsin(q) + q * np.sqrt(1.0 - q2) * (1.0 - 2.0 * q2) * (8.0 * q2 * q2 - 8.0 * q2 - 3.0))
    return val / (8.0 * np.sqrt(2.0) * np.pi ** 3 * (1.0 - q2) ** 2.5)


def _om_df_table(r_a: float, npts: int = 4000):
    """f(Q) of the Osipkov-Merritt Hernquist model by Eddington inversion.

    rho_Q(Psi) = (1 + r^2/r_a^2) rho(r(Psi)), Psi = 1/(1+r), rho = 1/(2 pi r (1+r)^3).
    f(Q) = 1/(sqrt(8) pi^2) d/dQ int_0^Q (d rho_Q/d Psi) / sqrt(Q - Psi) dPsi.
    """
    psi = np.linspace(0.0, 1.0, npts + 1)[1:-1]
    r = 1.0 / psi - 1.0
    rho = 1.0 / (2.0 * np.pi * r * (1.0 + r) ** 3)
    rhoq = (1.0 + (r / r_a) ** 2) * rho
    drho = np.gradient(rhoq, psi)
    # substitute Psi = Q - t^2 to remove the inverse square-root singularity
    Q = psi
    t = np.linspace(0.0, 1.0, 400)
    I = np.empty_like(Q)
    for k, qq in enumerate(Q):
        tt = t * np.sqrt(qq)
        p = qq - tt * tt
        I[k] = 2.0 * np.trapezoid(np.interp(p, psi, drho, left=drho[0]), tt)
    f = np.gradient(I, Q) / (np.sqrt(8.0) * np.pi ** 2)
    return Q, np.maximum(f, 0.0)


def hernquist(n: int, seed: int = 2, r_max: float = 100.0, r_a: float | None = None):
    rng = np.random.Generator(np.random.PCG64(seed))
    umax = (r_max / (1.0 + r_max)) ** 2
    s = np.sqrt(rng.uniform(0.0, umax, n))
    r = s / (1.0 - s)
    r = np.maximum(r, 1e-12)
    psi = 1.0 / (1.0 + r)
    if r_a is None:
        fdf = hernquist_df
    else:
        Qt, ft = _om_df_table(r_a)

        def fdf(Q):
            return np.interp(Q, Qt, ft, left=0.0, right=ft[-1])
    # envelope of x^2 f(psi (1 - x^2)), x = w / w_esc, tabulated over psi
    pg = np.linspace(0.0, 1.0, 513)[1:]
    xg = np.linspace(0.0, 1.0, 257)
    env = np.array([np.max(xg * xg * fdf(p * (1.0 - xg * xg))) for p in pg]) * 1.3 + 1e-300
    bound = np.interp(psi, pg, env)
    bound = np.maximum(bound, np.interp(np.minimum(psi + 1.0 / 512, 1.0), pg, env))
    x = np.empty(n)
    todo = np.arange(n)
    while todo.size:
        xx = rng.uniform(0.0, 1.0, todo.size)
        yy = rng.uniform(0.0, 1.0, todo.size) * bound[todo]
        ok = yy < xx * xx * fdf(psi[todo] * (1.0 - xx * xx))
        x[todo[ok]] = xx[ok]
        todo = todo[~ok]
    w = x * np.sqrt(2.0 * psi)
    mu = rng.uniform(-1.0, 1.0, n)
    if r_a is None:
        return _finish(r, w, mu)
    # Osipkov-Merritt: w is isotropic in (v_r, v_t sqrt(1 + r^2/r_a^2))
    wr = w * mu
    wt = w * np.sqrt(np.maximum(0.0, 1.0 - mu * mu))
    vt = wt / np.sqrt(1.0 + (r / r_a) ** 2)
    v = np.sqrt(wr * wr + vt * vt)
    mu2 = np.where(v > 0, wr / np.where(v > 0, v, 1.0), 0.0)
    return _finish(r, v, mu2)


# ---------------------------------------------------------------- reference file formats

INIT_RECORD = np.dtype([("r", "<f8"), ("v", "<f8"), ("l", "<f8"), ("id", "<f8"), ("mu", "<f8")])
SNAP_RECORD = np.dtype([("rank", "<i4"), ("r", "<f4"), ("v", "<f4"), ("l", "<f4")])


def write_init_file(path, r, vr, ell, ids, mu=None):
    """Writes the initial-conditions file of the reference's write_initial_conditions
    (nsphere.c:2386-2420): int32 npts, then npts records (r, v_r, ell, index, mu)."""
    n = len(r)
    rec = np.empty(n, dtype=INIT_RECORD)
    rec["r"], rec["v"], rec["l"] = r, vr, ell
    rec["id"] = np.asarray(ids, dtype=np.float64)
    rec["mu"] = 0.0 if mu is None else mu
    with open(path, "wb") as f:
        f.write(np.int32(n).tobytes())
        f.write(rec.tobytes())


def read_init_file(path):
    """Reads a file written by write_initial_conditions: (r, v_r, ell, ids, mu)."""
    with open(path, "rb") as f:
        n = int(np.frombuffer(f.read(4), dtype="<i4")[0])
        rec = np.frombuffer(f.read(n * INIT_RECORD.itemsize), dtype=INIT_RECORD)
    if rec.shape[0] != n:
        raise ValueError("%s ends before its %d records" % (path, n))
    return (rec["r"].copy(), rec["v"].copy(), rec["l"].copy(), rec["id"].astype(np.int32), rec["mu"].copy())


def read_snapshots(path, n):
    """Reads an all_particle_data stream (nsphere.c:1295-1324): array (snapshots, n)
    of records (rank, r, v, l) indexed by original particle id."""
    raw = np.fromfile(path, dtype=SNAP_RECORD)
    if raw.size % n:
        raise ValueError("%s does not hold whole snapshots of %d records" % (path, n))
    return raw.reshape(-1, n)


def snapshot_records(r, vr, ell, ids):
    """The snapshot records the reference writes for a state in sorted order
    (nsphere.c:6466-6476): record[id] = (rank, float r, float v_r, float ell)."""
    n = len(r)
    out = np.empty(n, dtype=SNAP_RECORD)
    ids = np.asarray(ids, dtype=np.int64)
    out["rank"][ids] = np.arange(n, dtype=np.int32)
    out["r"][ids] = np.asarray(r).astype(np.float32)
    out["v"][ids] = np.asarray(vr).astype(np.float32)
    out["l"][ids] = np.asarray(ell).astype(np.float32)
    return out


def write_rank_files(sorted_path, unsorted_path, sorted_records, unsorted_records):
    """Writes Rank_Mass_Rad_VRad_sorted / _unsorted files as the reference's fprintf_bin
    does (nsphere.c:2550-2588, 7930-7983): the records back to back, no header."""
    if sorted_path is not None:
        np.ascontiguousarray(sorted_records).tofile(sorted_path)
    if unsorted_path is not None:
        np.ascontiguousarray(unsorted_records).tofile(unsorted_path)


# ---------------------------------------------------------------- counter-based generators
# The restatement, in numpy, of the GPU generators of nsg_generate (csrc/nsg_ics.cu):
# the same counter-based draws and the same arithmetic, for the tests.

_M64 = np.uint64(0xFFFFFFFFFFFFFFFF)


def _mix(x):
    x = x + np.uint64(0x9E3779B97F4A7C15)
    x = (x ^ (x >> np.uint64(30))) * np.uint64(0xBF58476D1CE4E5B9)
    x = (x ^ (x >> np.uint64(27))) * np.uint64(0x94D049BB133111EB)
    return x ^ (x >> np.uint64(31))


def counter_uniform(seed, i, j):
    """Draw j of particle i in [0, 1): SplitMix64 finaliser applied twice."""
    with np.errstate(over="ignore"):
        i = np.asarray(i, dtype=np.uint64)
        h = _mix(_mix(np.uint64(seed) ^ (i * np.uint64(0xD1B54A32D192ED03))) + np.uint64(j))
    return (h >> np.uint64(11)).astype(np.float64) * 2.0 ** -53


def _hq_df_unnormalised(eps):
    e = np.clip(eps, 0.0, 1.0 - 1e-15)
    q = np.sqrt(e)
    q2 = q * q
    val = 3.0 * np.arcsin(q) + q * np.sqrt(1.0 - q2) * (1.0 - 2.0 * q2) * (8.0 * q2 * q2 - 8.0 * q2 - 3.0)
    w = 1.0 - q2
    return val / (w * w * np.sqrt(w))


def _hq_target(psi, x):
    return x * x * _hq_df_unnormalised(psi * (1.0 - x * x))


def _hq_bound(psi):
    """Per-particle rejection bound: best of x_j = (j/64)^2, 40 golden-section steps."""
    gb = np.full(psi.shape, -1.0)
    jb = np.ones(psi.shape, dtype=np.int64)
    for j in range(1, 65):
        t = j / 64.0
        g = _hq_target(psi, t * t)
        better = g > gb
        gb = np.where(better, g, gb)
        jb = np.where(better, j, jb)
    tl = (jb - 1) / 64.0
    th = np.where(jb < 64, jb + 1, 64) / 64.0
    a, b = tl * tl, th * th
    ig = 0.6180339887498949
    c = b - ig * (b - a)
    d = a + ig * (b - a)
    gc, gd = _hq_target(psi, c), _hq_target(psi, d)
    for _ in range(40):
        left = gc > gd
        nb = np.where(left, d, b)
        na = np.where(left, a, c)
        nc = np.where(left, nb - ig * (nb - na), d)
        nd = np.where(left, c, na + ig * (nb - na))
        ngc = np.where(left, _hq_target(psi, nc), gd)
        ngd = np.where(left, gc, _hq_target(psi, nd))
        a, b, c, d, gc, gd = na, nb, nc, nd, ngc, ngd
    return np.maximum(gb, np.maximum(gc, gd)) * 1.3 + 1e-300


def _om_target(psi, x, k):
    q = psi * (1.0 - x * x)
    f = _hq_df_unnormalised(q) + k * np.sqrt(q) * (1.0 - 2.0 * q)
    return x * x * np.where(f > 0.0, f, 0.0)


def _om_bound(psi, k):
    """_hq_bound for the Osipkov-Merritt target."""
    gb = np.full(psi.shape, -1.0)
    jb = np.ones(psi.shape, dtype=np.int64)
    for j in range(1, 65):
        t = j / 64.0
        g = _om_target(psi, t * t, k)
        better = g > gb
        gb = np.where(better, g, gb)
        jb = np.where(better, j, jb)
    tl = (jb - 1) / 64.0
    th = np.where(jb < 64, jb + 1, 64) / 64.0
    a, b = tl * tl, th * th
    ig = 0.6180339887498949
    c = b - ig * (b - a)
    d = a + ig * (b - a)
    gc, gd = _om_target(psi, c, k), _om_target(psi, d, k)
    for _ in range(40):
        left = gc > gd
        nb = np.where(left, d, b)
        na = np.where(left, a, c)
        nc = np.where(left, nb - ig * (nb - na), d)
        nd = np.where(left, c, na + ig * (nb - na))
        ngc = np.where(left, _om_target(psi, nc, k), gd)
        ngd = np.where(left, gc, _om_target(psi, nd, k))
        a, b, c, d, gc, gd = na, nb, nc, nd, ngc, ngd
    return np.maximum(gb, np.maximum(gc, gd)) * 1.3 + 1e-300


def hernquist_om_counter(n: int, seed: int, r_max: float = 100.0, r_a: float = 1.0):
    """(r, vr, ell, ids, mu) of nsg_generate_om(n, seed, r_max, r_a)."""
    i = np.arange(n, dtype=np.uint64)
    k = 8.0 / (r_a * r_a)
    umax = (r_max / (1.0 + r_max)) * (r_max / (1.0 + r_max))
    s = np.sqrt(umax * counter_uniform(seed, i, 0))
    r = np.maximum(s / (1.0 - s), 1e-12)
    psi = 1.0 / (1.0 + r)
    bound = _om_bound(psi, k)
    x = np.zeros(n)
    todo = np.arange(n)
    a = 0
    while todo.size:
        xx = counter_uniform(seed, i[todo], 2 + 2 * a)
        yy = counter_uniform(seed, i[todo], 3 + 2 * a) * bound[todo]
        ok = yy < _om_target(psi[todo], xx, k)
        x[todo[ok]] = xx[ok]
        todo = todo[~ok]
        a += 1
    w = x * np.sqrt(2.0 * psi)
    mu = 2.0 * counter_uniform(seed, i, 1) - 1.0
    wr = w * mu
    wt = w * np.sqrt(np.maximum(0.0, 1.0 - mu * mu))
    ra = r / r_a
    vt = wt / np.sqrt(1.0 + ra * ra)
    return _rank_order(r, wr, r * vt, mu)


def _rank_order(r, vr, ell, mu):
    order = np.lexsort((np.arange(r.shape[0]), r))
    return r[order], vr[order], ell[order], np.arange(r.shape[0], dtype=np.int32), mu[order]


def plummer_counter(n: int, seed: int):
    """(r, vr, ell, ids, mu) of nsg_generate(NSG_IC_PLUMMER, n, seed)."""
    i = np.arange(n, dtype=np.uint64)
    u = 1e-10 + (1.0 - 1e-10) * counter_uniform(seed, i, 0)
    r = 1.0 / np.sqrt(u ** (-2.0 / 3.0) - 1.0)
    q = np.zeros(n)
    todo = np.arange(n)
    a = 0
    while todo.size:
        x1 = counter_uniform(seed, i[todo], 2 + 2 * a)
        x2 = counter_uniform(seed, i[todo], 3 + 2 * a)
        w = 1.0 - x1 * x1
        ok = 0.1 * x2 < x1 * x1 * (w * w * w * np.sqrt(w))
        q[todo[ok]] = x1[ok]
        todo = todo[~ok]
        a += 1
    v = q * np.sqrt(2.0) / np.sqrt(np.sqrt(1.0 + r * r))
    mu = 2.0 * counter_uniform(seed, i, 1) - 1.0
    return _rank_order(r, v * mu, r * v * np.sqrt(np.maximum(0.0, 1.0 - mu * mu)), mu)


def hernquist_counter(n: int, seed: int, r_max: float = 100.0):
    """(r, vr, ell, ids, mu) of nsg_generate(NSG_IC_HERNQUIST, n, seed, r_max)."""
    i = np.arange(n, dtype=np.uint64)
    umax = (r_max / (1.0 + r_max)) * (r_max / (1.0 + r_max))
    s = np.sqrt(umax * counter_uniform(seed, i, 0))
    r = np.maximum(s / (1.0 - s), 1e-12)
    psi = 1.0 / (1.0 + r)
    bound = _hq_bound(psi)
    x = np.zeros(n)
    todo = np.arange(n)
    a = 0
    while todo.size:
        xx = counter_uniform(seed, i[todo], 2 + 2 * a)
        yy = counter_uniform(seed, i[todo], 3 + 2 * a) * bound[todo]
        ok = yy < _hq_target(psi[todo], xx)
        x[todo[ok]] = xx[ok]
        todo = todo[~ok]
        a += 1
    w = x * np.sqrt(2.0 * psi)
    mu = 2.0 * counter_uniform(seed, i, 1) - 1.0
    return _rank_order(r, w * mu, r * w * np.sqrt(np.maximum(0.0, 1.0 - mu * mu)), mu)
