"""Per-snapshot post-processing (nsphere.c:7060-7990): Rank-file records on the GPU.

CPU: the oracle's knot recurrence against a plain loop, and the oracle's density
(direct sums of the one-sided Gaussian) against a numpy/scipy restatement of the
reference's own formulation -- natural cubic splines and the zero-padded FFT
convolution of nsphere.c:2901-3104.
GPU: nsg_post_snapshot against the oracle on the same float records.  Integer and
copied fields are equal; Psi_A, E and the density are doubles rounded to float, equal
to the oracle's within 2 float ulp (the potential's sums and the density's spline
solve and kernel normalisation differ from the oracle's sequential ones in order
only, and pow/exp come from two maths libraries).
"""
import math

import numpy as np
import pytest

from nsphere_gb300 import ics

F32_ULP = np.finfo(np.float32).eps


def _c_round(x):
    f = np.floor(x)
    return f + (x - f >= 0.5)


def _density_fft(R, M=1.0):
    """The reference's density pipeline (nsphere.c:7281-7686) in numpy, with its
    FFT convolution; R sorted."""
    interpolate = pytest.importorskip("scipy.interpolate")
    n = len(R)
    dM = M / n
    keep = np.concatenate([[True], R[1:] > R[:-1]])
    Rf, Mf = R[keep], (np.nonzero(keep)[0] + 1.0) * dM
    F, D = len(Rf), min(math.ceil(n / 100.0), 30000)
    if F <= D:
        Rd, Md = Rf, Mf
    else:
        step = (F - 1) / (D - 1)
        idx = np.minimum(_c_round(np.arange(D) * step).astype(np.int64), F - 1)
        Rd, Md = Rf[idx], Mf[idx]
    G = 131072
    lmin, lmax = math.log10(Rd[0]), math.log10(Rd[-1] * 1.04)
    dlog = (lmax - lmin) / (G - 1)
    lg = lmin + np.arange(G) * dlog
    rg = 10.0 ** lg
    mg = interpolate.CubicSpline(Rd, Md, bc_type="natural")(np.clip(rg, Rd[0], Rd[-1]))
    dg = np.empty(G)
    dg[1:-1] = (mg[2:] - mg[:-2]) / (rg[2:] - rg[:-2])
    dg[1:-1] = np.maximum(dg[1:-1], 1e-10)
    dg[0], dg[-1] = dg[1], dg[-2]
    sigma = 0.08 * (n / 10000.0) ** -0.40
    x = np.arange(G) * (lg[1] - lg[0])
    kn = np.exp(-0.5 * (x / sigma) ** 2) / (sigma * math.sqrt(2 * math.pi))
    kn /= kn.sum()
    pad = 2 * G
    sm = np.fft.irfft(np.fft.rfft(dg, pad) * np.fft.rfft(kn, pad), pad)[:G]
    sm = np.maximum(sm, 1e-10)
    back = interpolate.CubicSpline(rg, sm, bc_type="natural")
    return np.where(R <= rg[0], sm[0], np.where(R >= rg[-1], sm[-1], back(np.clip(R, rg[0], rg[-1]))))


def test_psi_knots_recurrence(oracle):
    rng = np.random.default_rng(4)
    R = np.sort(np.concatenate([[0.0, 0.0], np.round(rng.random(3000), 4), np.full(40, 0.5)]))
    k = oracle.psi_knots(R)
    want = [0.0]
    for x in R:
        want.append(x if x > want[-1] else want[-1] + 1e-5)
    assert np.array_equal(k, np.array(want))


def test_density_matches_fft_formulation(oracle):
    r, _, _, _ = ics.plummer(200_000, seed=21)
    R = np.sort(r.astype(np.float32).astype(np.float64))
    got = oracle.density(R)
    want = _density_fft(R)
    big = want > 1e-6 * want.max()
    assert big.mean() > 0.95
    assert np.allclose(got[big], want[big], rtol=1e-8, atol=0.0)
    # where the FFT's rounding noise dominates, both stay at or near the floor
    assert np.all(got > 0)


def _records(n, seed, nan=0, ties=0):
    r, v, l, ids = ics.hernquist(n, seed=seed) if n > 500_000 else ics.plummer(n, seed=seed)
    rec = ics.snapshot_records(*ics_sorted(r, v, l, ids))
    rng = np.random.default_rng(seed)
    if ties:
        j = rng.choice(n, ties, replace=False)
        rec["r"][j] = rec["r"][rng.choice(n, ties)]
    if nan:   # NaN v_r reads as 0 (nsphere.c:7118); a NaN radius would leave no density
        rec["v"][rng.choice(n, nan, replace=False)] = np.nan
    return rec


def ics_sorted(r, v, l, ids):
    o = np.lexsort((ids, r))
    return r[o], v[o], l[o], ids[o]


def _compare(srt, uns, psi0, want, rec, M):
    n = len(rec)
    dM = M / n
    assert np.array_equal(srt["rank"], np.arange(n, dtype=np.int32))
    assert np.array_equal(srt["mass"], ((np.arange(n) + 1.0) * dM).astype(np.float32))
    assert np.array_equal(srt["r"], want["s_r"].astype(np.float32))
    assert np.array_equal(srt["vr"], want["s_v"].astype(np.float32))
    assert np.array_equal(srt["ell"], want["s_l"].astype(np.float32))
    assert psi0 == pytest.approx(want["psi0"], rel=1e-12)

    def close(a, b, scale):
        return np.all(np.abs(a.astype(np.float64) - b.astype(np.float32).astype(np.float64))
                      <= 2 * F32_ULP * scale)

    psi_scale = np.nanmax(np.abs(want["s_psi"]))
    assert close(srt["psi"], want["s_psi"], np.abs(want["s_psi"]))
    assert close(srt["E"], want["s_E"], np.maximum(np.abs(want["s_E"]), psi_scale))
    assert close(srt["rho"], want["s_rho"], np.abs(want["s_rho"]))
    assert np.array_equal(uns["rank"], rec["rank"])
    assert np.array_equal(uns["mass"], ((rec["rank"] + 1.0) * dM).astype(np.float32))
    assert np.array_equal(uns["r"], rec["r"], equal_nan=True)
    assert np.array_equal(uns["vr"], rec["v"], equal_nan=True)
    assert np.array_equal(uns["ell"], rec["l"])
    fin = np.isfinite(want["u_psi"])
    assert np.array_equal(np.isfinite(uns["psi"]), fin)
    assert close(uns["psi"][fin], want["u_psi"][fin], np.abs(want["u_psi"][fin]))
    fe = np.isfinite(want["u_E"])
    assert close(uns["E"][fe], want["u_E"][fe], np.maximum(np.abs(want["u_E"][fe]), psi_scale))


@pytest.mark.gpu
@pytest.mark.parametrize("n,nan,ties,M,G", [(200_003, 20, 500, 1.0, 1.0), (60_000, 0, 0, 2.5, 0.7),
                                           (250, 0, 0, 1.0, 1.0), (30_001, 0, 3000, 1.0, 1.0)])
def test_post_snapshot_matches_oracle(nsg, oracle, n, nan, ties, M, G):
    rec = _records(n, 31 + n % 7, nan=nan, ties=ties)
    want = oracle.post_snapshot(rec["r"], rec["v"], rec["l"], G=G, M=M)
    assert want["density_ok"]
    with nsg.Context(nsg.default_params(G=G, M_total=M)) as c:
        srt, uns, psi0 = c.post_snapshot(rec)
        # the records are now the resident state, sorted
        r, vr, ell, ids = c.download()
    assert np.array_equal(ids, want["s_idx"].astype(np.int32))
    assert np.array_equal(r, want["s_r"])
    _compare(srt, uns, psi0, want, rec, M)


@pytest.mark.gpu
def test_post_snapshot_full_size(nsg, oracle):
    """N = 1e7 Hernquist snapshot: the knot adjustment cascades over most of the
    halo (float radii tie about once per ten particles near r ~ 1)."""
    n = 10_000_000
    rec = _records(n, 2)
    want = oracle.post_snapshot(rec["r"], rec["v"], rec["l"])
    with nsg.Context(nsg.default_params()) as c:
        srt, uns, psi0 = c.post_snapshot(rec)
    _compare(srt, uns, psi0, want, rec, 1.0)


@pytest.mark.gpu
def test_post_snapshot_rejects_undefined_density(nsg):
    with nsg.Context(nsg.default_params()) as c:
        rec = _records(150, 3)
        with pytest.raises(nsg.NsgError):
            c.post_snapshot(rec)           # fewer than 3 decimated radii
        rec = _records(5000, 3)
        rec["r"][7] = np.nan               # read as radius 0 (nsphere.c:7112-7116)
        with pytest.raises(nsg.NsgError):
            c.post_snapshot(rec)           # smallest radius not positive
