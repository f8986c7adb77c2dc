"""nsphere_gb300: GB300-native step loop of NSphere behind the C ABI of include/nsg.h.

This module is a thin ctypes binding of ``libnsg.so`` (built in-tree by
``nsphere_gb300.build``).  There is no CPU fallback: importing works anywhere, but
``lib()`` raises when the library is missing and every context creation fails
without an sm_103a GPU.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

_PKG = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_PKG, "libnsg.so")

NSG_OK = 0
NSG_EINVAL, NSG_ECUDA, NSG_ENOMEM, NSG_ESTATE, NSG_EIDS, NSG_EDEVICE, NSG_ETIMEOUT = (
    -1, -2, -3, -4, -5, -6, -7)
METHOD_KDK, METHOD_ADAPTIVE, METHOD_FULL_LC, METHOD_ADAPTIVE_LC = 2, 3, 4, 5
LC_RCRIT, LC_RADIUS, LC_OFF = 0, 1, 2
SCHED_PLAIN, SCHED_LEARNED = 0, 1
IC_PLUMMER, IC_HERNQUIST = 1, 2
PSI_CORED, PSI_PLUMMER, PSI_HERNQUIST = 0, 1, 2
ST_IC_REJECT = 0x20
ST_DEVICE_WAIT = 0x40
ST_NAN, ST_TAU_CAP, ST_NOT_CONVERGED, ST_SORT_FALLBACK, ST_QUEUE = 0x1, 0x2, 0x4, 0x8, 0x10

# exported symbols of include/nsg.h (tests check the library exports each one)
EXPORTS = [
    "nsg_params_default", "nsg_create", "nsg_destroy", "nsg_last_error", "nsg_set_params",
    "nsg_get_params", "nsg_upload", "nsg_upload_particles", "nsg_upload_device", "nsg_step",
    "nsg_sort", "nsg_download", "nsg_download_particles", "nsg_device_state",
    "nsg_sort_particles", "nsg_gather", "nsg_energy", "nsg_level_hist", "nsg_levels",
    "nsg_sync", "nsg_status", "nsg_clear_status", "nsg_profile", "nsg_profile_read", "nsg_counters",
    "nsg_selftest_division", "nsg_probe_fp64",
    "nsg_upload_ensemble", "nsg_num_halos", "nsg_energy_halos",
    "nsg_mlp_num_params", "nsg_mlp_init", "nsg_mlp_set_weights", "nsg_mlp_get_weights",
    "nsg_mlp_collect", "nsg_mlp_dataset", "nsg_mlp_train", "nsg_mlp_grad", "nsg_mlp_predict",
    "nsg_tune_get", "nsg_tune_set", "nsg_autotune", "nsg_sort_device_noalloc", "nsg_probe_latency",
    "nsg_write_init", "nsg_read_init", "nsg_snapshot_open", "nsg_snapshot", "nsg_snapshot_close",
    "nsg_generate", "nsg_potential", "nsg_track_open", "nsg_track_read", "nsg_track_close",
    "nsg_post_snapshot", "nsg_step_download", "nsg_generate_om",
]

# records of the reference's Rank files (nsphere.c:7930-7983), as nsg_rank_sorted /
# nsg_rank_unsorted in include/nsg.h
RANK_SORTED = np.dtype([("rank", "<i4"), ("mass", "<f4"), ("r", "<f4"), ("vr", "<f4"), ("psi", "<f4"),
                        ("E", "<f4"), ("ell", "<f4"), ("rho", "<f4")])
RANK_UNSORTED = np.dtype([("rank", "<i4"), ("mass", "<f4"), ("r", "<f4"), ("vr", "<f4"), ("psi", "<f4"),
                          ("E", "<f4"), ("ell", "<f4")])


class Params(C.Structure):
    """Mirror of ``nsg_params`` (include/nsg.h)."""
    _fields_ = [
        ("G", C.c_double), ("M_total", C.c_double), ("dt", C.c_double),
        ("tol_r", C.c_double), ("tol_v", C.c_double), ("max_subdiv", C.c_int64),
        ("out_type", C.c_int32), ("N_taumin", C.c_int32), ("method", C.c_int32),
        ("lc_rule", C.c_int32), ("lc_alpha", C.c_double), ("lc_radius", C.c_double),
        ("max_tau_steps", C.c_int64), ("sched", C.c_int32), ("carry_aux", C.c_int32),
        ("sort_mode", C.c_int32), ("graph", C.c_int32), ("point_mass", C.c_double),
        ("point_mass_rate", C.c_double), ("nonfinite_stop", C.c_int32), ("reserved", C.c_int32),
    ]


class Psi(C.Structure):
    """Mirror of ``nsg_psi`` (include/nsg.h): the static halo potential of tracking."""
    _fields_ = [("model", C.c_int32), ("reserved", C.c_int32), ("a", C.c_double),
                ("r_trunc", C.c_double), ("r_lo", C.c_double), ("r_hi", C.c_double)]


def reference_psi(rc: float = 100.0) -> Psi:
    """The reference's own halo (nsphere.c:366, 4528-4592): cored profile with core
    radius RC, mass normalised within 10 RC, tabulated on [0, 0.9999 * 10 RC]."""
    return Psi(PSI_CORED, 0, rc, 10.0 * rc, 0.0, 9999.0 / 10000.0 * 10.0 * rc)


class KernelStat(C.Structure):
    _fields_ = [("name", C.c_char * 32), ("launches", C.c_int64), ("total_ms", C.c_double),
                ("bytes", C.c_double)]


_lib = None


def lib() -> C.CDLL:
    """Loads libnsg.so; raises if it was not built (no fallback path exists)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise RuntimeError("libnsg.so is not built: run `python -c \"import __graft_entry__ as g; "
                           "g.build()\"` (needs nvcc); there is no CPU fallback")
    L = C.CDLL(LIB_PATH)
    P, I64, I32, D = C.c_void_p, C.c_int64, C.c_int32, C.c_double
    sig = {
        "nsg_params_default": [C.POINTER(Params)],
        "nsg_create": [C.POINTER(P), C.POINTER(Params), P],
        "nsg_set_params": [P, C.POINTER(Params)],
        "nsg_get_params": [P, C.POINTER(Params)],
        "nsg_upload": [P, P, P, P, P, P, I64],
        "nsg_upload_particles": [P, P, I64],
        "nsg_upload_device": [P, P, P, P, P, P, I64],
        "nsg_step": [P, C.c_int],
        "nsg_sort": [P],
        "nsg_download": [P, P, P, P, P, P],
        "nsg_download_particles": [P, P],
        "nsg_device_state": [P, P, P, P, P, P],
        "nsg_sort_particles": [P, P, I64],
        "nsg_gather": [P, P, C.c_int, P, P, P, P],
        "nsg_energy": [P, C.POINTER(D), C.POINTER(D)],
        "nsg_level_hist": [P, P, C.c_int],
        "nsg_levels": [P, P],
        "nsg_sync": [P, C.c_int],
        "nsg_status": [P, C.POINTER(C.c_uint32)],
        "nsg_clear_status": [P],
        "nsg_profile": [P, C.c_int],
        "nsg_counters": [P, C.POINTER(I64), C.POINTER(I64)],
        "nsg_selftest_division": [C.c_uint64, I64, C.POINTER(I64), C.POINTER(I64), P],
        "nsg_probe_fp64": [C.POINTER(D)] * 5,
        "nsg_upload_ensemble": [P, P, P, P, P, P, P, C.c_int],
        "nsg_num_halos": [P],
        "nsg_energy_halos": [P, P, P],
        "nsg_mlp_init": [P, C.c_uint64],
        "nsg_mlp_set_weights": [P, P, I64],
        "nsg_mlp_get_weights": [P, P, I64],
        "nsg_mlp_collect": [P, C.c_int, D, I64],
        "nsg_mlp_dataset": [P, C.POINTER(I64), P, P, I64],
        "nsg_mlp_train": [P, C.c_int, C.c_int, C.c_float, C.c_uint64, C.POINTER(D)],
        "nsg_mlp_grad": [P, P, P, I64, P, P, C.POINTER(D)],
        "nsg_mlp_predict": [P, P, I64, P, P],
        "nsg_profile_read": [P, C.POINTER(KernelStat), C.c_int, C.POINTER(C.c_int)],
        "nsg_tune_get": [P, P, C.c_int],
        "nsg_tune_set": [P, P, C.c_int],
        "nsg_autotune": [P, C.c_int, C.c_char_p, C.c_int],
        "nsg_sort_device_noalloc": [P, P, P, P, P, I64, P],
        "nsg_probe_latency": [P, C.c_int],
        "nsg_write_init": [P, C.c_char_p],
        "nsg_generate": [P, C.c_int, I64, C.c_uint64, D],
        "nsg_potential": [P, P, P, C.POINTER(D)],
        "nsg_read_init": [P, C.c_char_p, I64],
        "nsg_snapshot_open": [P, C.c_char_p, C.c_int],
        "nsg_snapshot": [P],
        "nsg_snapshot_close": [P],
        "nsg_track_open": [P, P, C.c_int, C.c_int, C.POINTER(Psi), I64],
        "nsg_track_read": [P, P, C.POINTER(I64), C.POINTER(I64)],
        "nsg_track_close": [P],
        "nsg_post_snapshot": [P, P, I64, P, P, C.POINTER(D)],
        "nsg_step_download": [P, C.c_int, P, P, P, P, P],
        "nsg_generate_om": [P, I64, C.c_uint64, D, D],
    }
    for name, args in sig.items():
        fn = getattr(L, name)
        fn.argtypes = args
        fn.restype = C.c_int
    L.nsg_destroy.argtypes = [P]
    L.nsg_destroy.restype = None
    L.nsg_last_error.argtypes = [P]
    L.nsg_last_error.restype = C.c_char_p
    L.nsg_mlp_num_params.argtypes = []
    L.nsg_mlp_num_params.restype = C.c_int
    _lib = L
    return L


class NsgError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__("nsg error %d: %s" % (code, msg))
        self.code = code


def default_params(**kw) -> Params:
    p = Params()
    lib().nsg_params_default(C.byref(p))
    for k, v in kw.items():
        if not hasattr(p, k):
            raise AttributeError("nsg_params has no field %r" % k)
        setattr(p, k, v)
    return p


def _ptr(a):
    return C.c_void_p(a.ctypes.data) if a is not None else None


class Context:
    """One libnsg context: device-resident state and its stream."""

    def __init__(self, params: Params | None = None, stream: int | None = None):
        self._L = lib()
        self.params = params if params is not None else default_params()
        h = C.c_void_p()
        rc = self._L.nsg_create(C.byref(h), C.byref(self.params), C.c_void_p(stream) if stream else None)
        if rc != NSG_OK:
            raise NsgError(rc, self._L.nsg_last_error(None).decode())
        self._h = h
        self.n = 0

    def _check(self, rc):
        if rc != NSG_OK:
            raise NsgError(rc, self._L.nsg_last_error(self._h).decode())

    def close(self):
        if getattr(self, "_h", None):
            self._L.nsg_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    @property
    def handle(self):
        return self._h

    def set_params(self, params: Params):
        self._check(self._L.nsg_set_params(self._h, C.byref(params)))
        self.params = params

    def upload(self, r, vr, ell, ids, aux=None):
        r, vr, ell = (np.ascontiguousarray(x, dtype=np.float64) for x in (r, vr, ell))
        idd = np.ascontiguousarray(ids, dtype=np.float64)
        aux = None if aux is None else np.ascontiguousarray(aux, dtype=np.float64)
        n = r.shape[0]
        if not (vr.shape[0] == ell.shape[0] == idd.shape[0] == n):
            raise ValueError("columns must have equal length")
        self._check(self._L.nsg_upload(self._h, _ptr(r), _ptr(vr), _ptr(ell), _ptr(idd), _ptr(aux), n))
        self.n = n

    def upload_ensemble(self, r, vr, ell, ids, halo_n, aux=None):
        """Independent halos in one state: halo h is the next halo_n[h] rows."""
        r, vr, ell = (np.ascontiguousarray(x, dtype=np.float64) for x in (r, vr, ell))
        idd = np.ascontiguousarray(ids, dtype=np.float64)
        hn = np.ascontiguousarray(halo_n, dtype=np.int64)
        aux = None if aux is None else np.ascontiguousarray(aux, dtype=np.float64)
        if int(hn.sum()) != r.shape[0]:
            raise ValueError("halo sizes must add up to the number of rows")
        self._check(self._L.nsg_upload_ensemble(self._h, _ptr(r), _ptr(vr), _ptr(ell), _ptr(idd), _ptr(aux),
                                                _ptr(hn), int(hn.size)))
        self.n = r.shape[0]

    def energy_halos(self):
        nh = self._L.nsg_num_halos(self._h)
        K, W = np.zeros(nh), np.zeros(nh)
        self._check(self._L.nsg_energy_halos(self._h, _ptr(K), _ptr(W)))
        return K, W

    def step(self, nsteps: int = 1):
        self._check(self._L.nsg_step(self._h, int(nsteps)))

    def sort(self):
        self._check(self._L.nsg_sort(self._h))

    def download(self, with_aux: bool = False):
        # the library's own count sizes the arrays it fills
        n = self.n = self._n_from_ctx()
        r, vr, ell, idd = (np.empty(n) for _ in range(4))
        aux = np.empty(n) if with_aux else None
        self._check(self._L.nsg_download(self._h, _ptr(r), _ptr(vr), _ptr(ell), _ptr(idd), _ptr(aux)))
        out = (r, vr, ell, idd.astype(np.int32))
        return out + ((aux,) if with_aux else ())

    def step_download(self, nsteps: int = 1, with_aux: bool = False):
        """nsteps steps, then the state as download() returns it (the copy overlaps the
        last step's Levi-Civita chains)."""
        n = self.n = self._n_from_ctx()
        r, vr, ell, idd = (np.empty(n) for _ in range(4))
        aux = np.empty(n) if with_aux else None
        self._check(self._L.nsg_step_download(self._h, int(nsteps), _ptr(r), _ptr(vr), _ptr(ell), _ptr(idd),
                                              _ptr(aux)))
        out = (r, vr, ell, idd.astype(np.int32))
        return out + ((aux,) if with_aux else ())

    def gather(self, ids):
        ids = np.ascontiguousarray(ids, dtype=np.int32)
        k = ids.shape[0]
        r, vr, ell = np.empty(k), np.empty(k), np.empty(k)
        rank = np.empty(k, dtype=np.int32)
        self._check(self._L.nsg_gather(self._h, _ptr(ids), k, _ptr(r), _ptr(vr), _ptr(ell), _ptr(rank)))
        return r, vr, ell, rank

    def energy(self):
        K, W = C.c_double(), C.c_double()
        self._check(self._L.nsg_energy(self._h, C.byref(K), C.byref(W)))
        return K.value, W.value

    def level_hist(self, nbins: int = 66):
        h = np.zeros(nbins, dtype=np.int64)
        self._check(self._L.nsg_level_hist(self._h, _ptr(h), nbins))
        return h

    def levels(self):
        lv = np.empty(self._n_from_ctx(), dtype=np.int8)
        self._check(self._L.nsg_levels(self._h, _ptr(lv)))
        return lv

    def sync(self, timeout_ms: int = -1):
        self._check(self._L.nsg_sync(self._h, timeout_ms))

    def status(self) -> int:
        s = C.c_uint32()
        self._check(self._L.nsg_status(self._h, C.byref(s)))
        return s.value

    def clear_status(self):
        self._check(self._L.nsg_clear_status(self._h))

    # ---- learned level scheduler
    def mlp_init(self, seed: int = 1):
        self._check(self._L.nsg_mlp_init(self._h, seed))

    def mlp_weights(self):
        w = np.zeros(self._L.nsg_mlp_num_params(), dtype=np.float32)
        self._check(self._L.nsg_mlp_get_weights(self._h, _ptr(w), w.size))
        return w

    def mlp_set_weights(self, w):
        w = np.ascontiguousarray(w, dtype=np.float32)
        self._check(self._L.nsg_mlp_set_weights(self._h, _ptr(w), w.size))

    def mlp_collect(self, nsteps: int, keep_level0: float = 0.01, capacity: int = 1 << 20):
        self._check(self._L.nsg_mlp_collect(self._h, int(nsteps), float(keep_level0), int(capacity)))

    def mlp_dataset(self, max_samples: int | None = None):
        cnt = C.c_int64()
        self._check(self._L.nsg_mlp_dataset(self._h, C.byref(cnt), None, None, 0))
        k = cnt.value if max_samples is None else min(cnt.value, max_samples)
        X = np.zeros((k, 4), dtype=np.float32)
        y = np.zeros(k, dtype=np.int8)
        self._check(self._L.nsg_mlp_dataset(self._h, C.byref(cnt), _ptr(X), _ptr(y), k))
        return X, y

    def mlp_train(self, epochs: int, batch: int = 1024, lr: float = 3e-3, seed: int = 1) -> float:
        loss = C.c_double()
        self._check(self._L.nsg_mlp_train(self._h, int(epochs), int(batch), C.c_float(lr), seed, C.byref(loss)))
        return loss.value

    def mlp_grad(self, X, y, cls_w):
        X = np.ascontiguousarray(X, dtype=np.float32)
        y = np.ascontiguousarray(y, dtype=np.int8)
        cw = np.ascontiguousarray(cls_w, dtype=np.float32)
        g = np.zeros(self._L.nsg_mlp_num_params(), dtype=np.float32)
        loss = C.c_double()
        self._check(self._L.nsg_mlp_grad(self._h, _ptr(X), _ptr(y), X.shape[0], _ptr(cw), _ptr(g), C.byref(loss)))
        return loss.value, g

    def mlp_predict(self, X):
        X = np.ascontiguousarray(X, dtype=np.float32)
        cls = np.zeros(X.shape[0], dtype=np.int8)
        lg = np.zeros((X.shape[0], 8), dtype=np.float32)
        self._check(self._L.nsg_mlp_predict(self._h, _ptr(X), X.shape[0], _ptr(cls), _ptr(lg)))
        return cls, lg

    def counters(self):
        a, b = C.c_int64(), C.c_int64()
        self._check(self._L.nsg_counters(self._h, C.byref(a), C.byref(b)))
        return a.value, b.value

    def profile(self, enable: bool = True):
        self._check(self._L.nsg_profile(self._h, 1 if enable else 0))

    def _n_from_ctx(self) -> int:
        n = C.c_int64()
        self._check(self._L.nsg_device_state(self._h, None, None, None, None, C.byref(n)))
        return n.value

    def generate(self, model: int, n: int, seed: int, r_max: float = 100.0):
        """Seeded initial conditions generated on the GPU into the resident state."""
        self._check(self._L.nsg_generate(self._h, int(model), int(n), int(seed), float(r_max)))
        self.n = int(n)

    def generate_om(self, n: int, seed: int, r_max: float = 100.0, r_a: float = 1.0):
        """Hernquist with Osipkov-Merritt anisotropy radius r_a, generated on the GPU."""
        self._check(self._L.nsg_generate_om(self._h, int(n), int(seed), float(r_max), float(r_a)))
        self.n = int(n)

    def potential(self):
        """(psi, E, psi0) of the sorted resident state (see nsg_potential)."""
        n = self._n_from_ctx()
        psi = np.empty(n)
        E = np.empty(n)
        p0 = C.c_double()
        self._check(self._L.nsg_potential(self._h, _ptr(psi), _ptr(E), C.byref(p0)))
        return psi, E, p0.value

    # ---- files of the reference
    def write_init(self, path: str):
        """Writes the reference's initial-conditions file from the resident state."""
        self._check(self._L.nsg_write_init(self._h, os.fsencode(path)))

    def read_init(self, path: str, expected_n: int = -1):
        """Uploads the state of a reference initial-conditions file."""
        self._check(self._L.nsg_read_init(self._h, os.fsencode(path), int(expected_n)))
        self.n = self._n_from_ctx()

    def snapshot_open(self, path: str, append: bool = False):
        self._check(self._L.nsg_snapshot_open(self._h, os.fsencode(path), int(append)))

    def snapshot(self):
        """Appends an all_particle_data snapshot of the resident state (asynchronous)."""
        self._check(self._L.nsg_snapshot(self._h))

    def snapshot_close(self):
        self._check(self._L.nsg_snapshot_close(self._h))

    def track_open(self, ids, psi: Psi, capacity: int, k_clamped: int = 0):
        """Records r, v_r, ell, E_rel, mu of the particles `ids` after every step on
        the GPU (the reference's tracking, nsphere.c:6384-6450)."""
        ids = np.ascontiguousarray(ids, dtype=np.int32)
        self._track_k, self._track_cap = len(ids), int(capacity)
        self._check(self._L.nsg_track_open(self._h, _ptr(ids), len(ids), int(k_clamped), C.byref(psi),
                                           int(capacity)))

    def track_read(self):
        """(records[5, k, recorded], steps_seen): r, v_r, ell, E_rel, mu per step."""
        out = np.empty((5, self._track_k, self._track_cap))
        rec, seen = C.c_int64(), C.c_int64()
        self._check(self._L.nsg_track_read(self._h, _ptr(out), C.byref(rec), C.byref(seen)))
        return out[:, :, :rec.value], seen.value

    def track_close(self):
        self._check(self._L.nsg_track_close(self._h))

    def post_snapshot(self, records):
        """The reference's per-snapshot post-processing (nsphere.c:7060-7990) of one
        block of 16-byte snapshot records: (sorted RANK_SORTED records, RANK_UNSORTED
        records in record order, Psi_A(0)).  The records become the resident state."""
        rec = np.ascontiguousarray(records)
        if rec.dtype.itemsize != 16:
            raise ValueError("snapshot records are 16 bytes")
        n = len(rec)
        srt = np.empty(n, dtype=RANK_SORTED)
        uns = np.empty(n, dtype=RANK_UNSORTED)
        psi0 = C.c_double()
        self._check(self._L.nsg_post_snapshot(self._h, _ptr(rec), n, _ptr(srt), _ptr(uns), C.byref(psi0)))
        self.n = n
        return srt, uns, psi0.value

    def tune_get(self):
        """Launch shapes: (gather_level0 threads, its blocks/SM, log2 bucket, level blocks/SM)."""
        v = (C.c_int32 * 4)()
        self._check(self._L.nsg_tune_get(self._h, v, 4))
        return tuple(v)

    def tune_set(self, vals):
        v = (C.c_int32 * 4)(*[int(x) for x in vals])
        self._check(self._L.nsg_tune_set(self._h, v, 4))

    def autotune(self, steps=2):
        """Times candidate launch shapes on the resident state (which it restores) and
        keeps the fastest; returns the timing report as a dict."""
        import json
        buf = C.create_string_buffer(4096)
        self._check(self._L.nsg_autotune(self._h, int(steps), buf, 4096))
        return json.loads(buf.value.decode())

    def profile_read(self):
        arr = (KernelStat * 64)()
        cnt = C.c_int()
        self._check(self._L.nsg_profile_read(self._h, arr, 64, C.byref(cnt)))
        return [dict(name=arr[i].name.decode(), launches=arr[i].launches,
                     total_ms=arr[i].total_ms, bytes=arr[i].bytes) for i in range(min(cnt.value, 64))]


def selftest_division(count: int, seed: int = 1):
    """(mismatches, fast_path_count, first_bad_pair) of the integer-pipe division
    against the hardware IEEE division on the current GPU."""
    mism, fast = C.c_int64(), C.c_int64()
    first = np.zeros(2)
    rc = lib().nsg_selftest_division(seed, count, C.byref(mism), C.byref(fast), _ptr(first))
    if rc != NSG_OK:
        raise NsgError(rc, lib().nsg_last_error(None).decode())
    return mism.value, fast.value, tuple(first)


def probe_fp64() -> dict:
    """FP64 throughput and latency of the current GPU (see nsg_probe_fp64)."""
    vals = [C.c_double() for _ in range(5)]
    rc = lib().nsg_probe_fp64(*[C.byref(v) for v in vals])
    if rc != NSG_OK:
        raise NsgError(rc, lib().nsg_last_error(None).decode())
    keys = ["dfma_tflops", "div_hw_gps", "div_int_gps", "fma_latency_cycles", "div_latency_cycles"]
    return {k: v.value for k, v in zip(keys, vals)}


LATENCY_PROBES = ["fp64_fma", "fp64_fma_two_chains_one_warp", "fp64_fma_one_chain_two_warps",
                  "div_fp64_pipe", "div_int_throughput_form", "div_latency_form", "imad32", "mulhi64",
                  "i2f_fmul_f2i", "levi_civita_substep", "levi_civita_substep_zero_gravity",
                  "levi_civita_substep_both_quotients", "dadd_shuffle_half_warp", "dadd_select_f64"]


def probe_latency() -> dict:
    """Dependent latencies in cycles per iteration (see nsg_probe_latency)."""
    v = np.zeros(len(LATENCY_PROBES))
    rc = lib().nsg_probe_latency(_ptr(v), len(v))
    if rc != NSG_OK:
        raise NsgError(rc, lib().nsg_last_error(None).decode())
    return dict(zip(LATENCY_PROBES, v.tolist()))


def sort_particles(ctx: Context, particles: np.ndarray):
    """Drop-in for the reference's ``sort_particles(double **particles, int npts)``
    on a (4 or 5, n) float64 table, sorted in place on the GPU."""
    if particles.dtype != np.float64 or not particles.flags.c_contiguous:
        raise ValueError("particles must be a C-contiguous float64 (k, n) array")
    n = particles.shape[1]
    rows = (C.c_void_p * 5)(*[particles[min(i, particles.shape[0] - 1)].ctypes.data for i in range(5)])
    ctx._check(ctx._L.nsg_sort_particles(ctx._h, rows, n))
