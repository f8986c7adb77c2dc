"""The reference's particle files: the initial-conditions file (int32 npts + npts
records of five doubles) and the all_particle_data snapshot stream (16-byte records
by original id), written and read through the C ABI from the resident GPU state."""
import os

import numpy as np
import pytest

from nsphere_gb300 import ics


def test_init_file_layout(tmp_path):
    r, vr, ell, ids = ics.plummer(1000, seed=3)
    p = str(tmp_path / "ic.bin")
    ics.write_init_file(p, r, vr, ell, ids)
    assert os.path.getsize(p) == 4 + 40 * 1000
    raw = open(p, "rb").read()
    assert np.frombuffer(raw[:4], "<i4")[0] == 1000
    first = np.frombuffer(raw[4:44], "<f8")
    assert np.array_equal(first, [r[0], vr[0], ell[0], ids[0], 0.0])
    r2, v2, l2, i2, mu = ics.read_init_file(p)
    assert np.array_equal(r2, r) and np.array_equal(v2, vr) and np.array_equal(l2, ell) and np.array_equal(i2, ids)


@pytest.mark.gpu
def test_init_file_round_trip(nsg, tmp_path):
    r, vr, ell, ids = ics.hernquist(300_001, seed=41)
    p_in, p_out = str(tmp_path / "in.bin"), str(tmp_path / "out.bin")
    ics.write_init_file(p_in, r, vr, ell, ids)
    with nsg.Context(nsg.default_params(dt=1e-3, method=2)) as c:
        c.read_init(p_in, expected_n=len(r))
        got = c.download()
        assert np.array_equal(got[0], r) and np.array_equal(got[3], ids)
        c.step(2)
        c.write_init(p_out)
        after = c.download()
    rr, vv, ll, ii, mu = ics.read_init_file(p_out)
    assert np.array_equal(rr, after[0]) and np.array_equal(vv, after[1])
    assert np.array_equal(ll, after[2]) and np.array_equal(ii, after[3]) and not mu.any()


@pytest.mark.gpu
def test_init_file_many_chunks_and_mu(nsg, tmp_path):
    n = (1 << 21) + 12345
    rng = np.random.default_rng(5)
    r = rng.random(n) + 1e-3
    vr, ell, mu = rng.normal(size=n), rng.random(n), rng.uniform(-1, 1, n)
    ids = rng.permutation(n).astype(np.int32)
    p = str(tmp_path / "big.bin")
    ics.write_init_file(p, r, vr, ell, ids, mu)
    with nsg.Context(nsg.default_params(carry_aux=1)) as c:
        c.read_init(p)
        got = c.download(with_aux=True)
        q = str(tmp_path / "big_out.bin")
        c.write_init(q)
    assert np.array_equal(got[0], r) and np.array_equal(got[4], mu) and np.array_equal(got[3], ids)
    assert open(p, "rb").read() == open(q, "rb").read()


@pytest.mark.gpu
def test_init_file_errors(nsg, tmp_path):
    r, vr, ell, ids = ics.plummer(2000, seed=3)
    p = str(tmp_path / "ic.bin")
    ics.write_init_file(p, r, vr, ell, ids)
    with nsg.Context(nsg.default_params()) as c:
        with pytest.raises(nsg.NsgError, match="expected"):
            c.read_init(p, expected_n=1999)
        with pytest.raises(nsg.NsgError):
            c.read_init(str(tmp_path / "missing.bin"))
        short = str(tmp_path / "short.bin")
        open(short, "wb").write(open(p, "rb").read()[:4 + 40 * 1000])
        with pytest.raises(nsg.NsgError, match="ends before"):
            c.read_init(short)
        bad = str(tmp_path / "bad_ids.bin")
        ics.write_init_file(bad, r, vr, ell, np.zeros(2000, np.int32))
        with pytest.raises(nsg.NsgError):
            c.read_init(bad)


@pytest.mark.gpu
def test_snapshot_stream(nsg, tmp_path):
    n = 50_000
    r, vr, ell, ids = ics.hernquist(n, seed=42)
    p = str(tmp_path / "apd.bin")
    want = []
    with nsg.Context(nsg.default_params(dt=1e-3, max_subdiv=64, lc_rule=1, lc_radius=1e-2,
                                        max_tau_steps=1_000_000)) as c:
        c.upload(r, vr, ell, ids)
        c.snapshot_open(p)
        c.snapshot()                       # before any step: ranks are the upload order
        want.append(ics.snapshot_records(*c.download()))
        for _ in range(3):
            c.step(2)
            c.snapshot()
            want.append(ics.snapshot_records(*c.download()))
        c.snapshot_close()
        c.snapshot_open(p, append=True)
        c.step(1)
        c.snapshot()
        want.append(ics.snapshot_records(*c.download()))
        c.snapshot_close()
    got = ics.read_snapshots(p, n)
    assert got.shape == (5, n)
    for g, w in zip(got, want):
        assert g.tobytes() == w.tobytes()
