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
