"""ctypes access to the CPU checkers (TEST INFRASTRUCTURE ONLY).

``Oracle`` wraps ``liborc.so`` (the C restatement in nsg_oracle.c); ``Reference``
wraps ``_ref/libnsref.so`` (the reference's own functions, see build_oracle.py).
Only tests/, the smoke check and bench.py's CPU-baseline leg import this module.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))


class OrcParams(C.Structure):
    _fields_ = [
        ("G", C.c_double), ("M", C.c_double), ("dt", C.c_double), ("tol_r", C.c_double),
        ("tol_v", C.c_double), ("max_subdiv", C.c_int64), ("out_type", C.c_int),
        ("N_taumin", C.c_int), ("lc_rule", C.c_int), ("lc_alpha", C.c_double),
        ("lc_radius", C.c_double), ("max_tau_steps", C.c_int64), ("point_mass", C.c_double),
        ("nonfinite_stop", C.c_int), ("lc_fixed", C.c_int),
    ]


def _p(a):
    return C.c_void_p(a.ctypes.data) if a is not None else None


class Oracle:
    def __init__(self, path: str | None = None):
        path = path or os.path.join(HERE, "liborc.so")
        if not os.path.exists(path):
            from . import build_oracle  # noqa: F401  (package import when available)
        self.L = C.CDLL(path)
        L = self.L
        D, I64, I = C.c_double, C.c_int64, C.c_int
        L.orc_params_default.argtypes = [C.POINTER(OrcParams)]
        L.orc_gnum.argtypes = [I64, I64, D, D]
        L.orc_gnum.restype = D
        L.orc_adaptive_leap.argtypes = [D, D, D, D, D, D, D, I64, I, C.POINTER(D), C.POINTER(D), C.POINTER(I)]
        L.orc_adaptive_lc.argtypes = [D, D, D, D, D, I, D, D, I64, I, I64, C.POINTER(D), C.POINTER(D),
                                      C.POINTER(I), C.POINTER(I64)]
        L.orc_adaptive_lc.restype = I
        L.orc_micro_leap.argtypes = [D, D, D, D, D, I64, I, C.POINTER(D), C.POINTER(D)]
        L.orc_sort.argtypes = [I64, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]
        L.orc_sort.restype = I
        L.orc_step_adaptive.argtypes = [C.POINTER(OrcParams), I64, C.c_void_p, C.c_void_p, C.c_void_p,
                                        C.c_void_p, C.c_void_p]
        L.orc_step_adaptive.restype = I64
        L.orc_step_kdk.argtypes = [C.POINTER(OrcParams), I64, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]
        L.orc_lc_fixed.argtypes = [D, D, D, D, D, I, I64, C.POINTER(D), C.POINTER(D)]
        L.orc_psi.argtypes = [I, D, D, D, D, D, D, D]
        L.orc_psi.restype = D
        L.orc_track.argtypes = [I, D, D, D, D, D, D, I, I, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]
        L.orc_density.argtypes = [I64, C.c_void_p, D, C.c_void_p]
        L.orc_psi_knots.argtypes = [I64, C.c_void_p, C.c_void_p]
        L.orc_psi_knots.restype = None
        L.orc_post_snapshot.argtypes = [I64, C.c_void_p, C.c_void_p, C.c_void_p, D, D] + [C.c_void_p] * 10
        L.orc_energy.argtypes = [C.POINTER(OrcParams), I64, C.c_void_p, C.c_void_p, C.c_void_p,
                                 C.POINTER(D), C.POINTER(D)]
        L.orc_num_threads.restype = I

    def params(self, **kw) -> OrcParams:
        p = OrcParams()
        self.L.orc_params_default(C.byref(p))
        for k, v in kw.items():
            setattr(p, k, v)
        return p

    def gnum(self, i, n, G=1.0, M=1.0):
        return self.L.orc_gnum(i, n, G, M)

    def adaptive_leap(self, r, v, ell, gnum, h, tol_r=1e-7, tol_v=1e-7, max_subdiv=128, out_type=2):
        ro, vo, lv = C.c_double(), C.c_double(), C.c_int()
        self.L.orc_adaptive_leap(r, v, ell, gnum, h, tol_r, tol_v, max_subdiv, out_type,
                                 C.byref(ro), C.byref(vo), C.byref(lv))
        return ro.value, vo.value, lv.value

    def adaptive_lc(self, r, v, ell, gnum, dt, N_taumin=10, tol_r=1e-7, tol_v=1e-7, max_subdiv=128,
                    out_type=2, max_tau_steps=100000000):
        ro, vo, lv, nt = C.c_double(), C.c_double(), C.c_int(), C.c_int64()
        cap = self.L.orc_adaptive_lc(r, v, ell, gnum, dt, N_taumin, tol_r, tol_v, max_subdiv, out_type,
                                     max_tau_steps, C.byref(ro), C.byref(vo), C.byref(lv), C.byref(nt))
        return ro.value, vo.value, lv.value, nt.value, cap

    def sort(self, r, vr, ell, ids, aux=None):
        r, vr, ell = (np.array(x, dtype=np.float64) for x in (r, vr, ell))
        ids = np.array(ids, dtype=np.int32)
        aux = None if aux is None else np.array(aux, dtype=np.float64)
        rc = self.L.orc_sort(r.shape[0], _p(r), _p(vr), _p(ell), _p(ids), _p(aux))
        assert rc == 0
        return (r, vr, ell, ids) + ((aux,) if aux is not None else ())

    def step_adaptive(self, params: OrcParams, r, vr, ell, ids):
        r, vr, ell = (np.array(x, dtype=np.float64) for x in (r, vr, ell))
        ids = np.array(ids, dtype=np.int32)
        lv = np.zeros(r.shape[0], dtype=np.int8)
        capped = self.L.orc_step_adaptive(C.byref(params), r.shape[0], _p(r), _p(vr), _p(ell), _p(ids), _p(lv))
        return r, vr, ell, ids, lv, capped

    def step_kdk(self, params: OrcParams, r, vr, ell, ids):
        r, vr, ell = (np.array(x, dtype=np.float64) for x in (r, vr, ell))
        ids = np.array(ids, dtype=np.int32)
        self.L.orc_step_kdk(C.byref(params), r.shape[0], _p(r), _p(vr), _p(ell), _p(ids))
        return r, vr, ell, ids

    def energy(self, params: OrcParams, r, vr, ell):
        K, W = C.c_double(), C.c_double()
        r, vr, ell = (np.ascontiguousarray(x, dtype=np.float64) for x in (r, vr, ell))
        self.L.orc_energy(C.byref(params), r.shape[0], _p(r), _p(vr), _p(ell), C.byref(K), C.byref(W))
        return K.value, W.value

    def num_threads(self):
        return self.L.orc_num_threads()

    def density(self, R, M=1.0):
        """Smoothed density of the reference's post-processing at sorted radii R."""
        R = np.ascontiguousarray(R, dtype=np.float64)
        rho = np.empty(len(R))
        rc = self.L.orc_density(len(R), _p(R), M, _p(rho))
        if rc:
            raise ValueError("density undefined for these radii")
        return rho

    def psi_knots(self, R):
        R = np.ascontiguousarray(R, dtype=np.float64)
        k = np.empty(len(R) + 1)
        self.L.orc_psi_knots(len(R), _p(R), _p(k))
        return k

    def post_snapshot(self, r, v, l, G=1.0, M=1.0):
        """Rank-file quantities of float32 records (doubles before the float output)."""
        r, v, l = (np.ascontiguousarray(x, dtype=np.float32) for x in (r, v, l))
        n = len(r)
        out = {k: np.empty(n) for k in ("s_r", "s_v", "s_l", "s_psi", "s_E", "s_rho", "u_psi", "u_E")}
        idx = np.empty(n, dtype=np.int64)
        psi0 = C.c_double()
        rc = self.L.orc_post_snapshot(n, _p(r), _p(v), _p(l), G, M, _p(idx), _p(out["s_r"]), _p(out["s_v"]),
                                      _p(out["s_l"]), _p(out["s_psi"]), _p(out["s_E"]), _p(out["s_rho"]),
                                      _p(out["u_psi"]), _p(out["u_E"]), C.byref(psi0))
        out["s_idx"] = idx
        out["psi0"] = psi0.value
        out["density_ok"] = rc == 0
        return out

    def lc_fixed(self, r, v, ell, gnum, dt, N_taumin=1000, max_steps=200_000_000):
        ro, vo = C.c_double(), C.c_double()
        capped = self.L.orc_lc_fixed(r, v, ell, gnum, dt, N_taumin, max_steps, C.byref(ro), C.byref(vo))
        return ro.value, vo.value, capped

    def psi(self, model, a, r_trunc, r_lo, r_hi, r, G=1.0, M=1.0):
        return self.L.orc_psi(model, a, r_trunc, r_lo, r_hi, G, M, float(r))

    def track(self, model, a, r_trunc, r_lo, r_hi, r, vr, ell, k_clamped=0, G=1.0, M=1.0):
        """(5, k) records r, v_r, ell, E_rel, mu of one step."""
        r, vr, ell = (np.ascontiguousarray(x, dtype=np.float64) for x in (r, vr, ell))
        k = len(r)
        out = np.empty((5, k))
        self.L.orc_track(model, a, r_trunc, r_lo, r_hi, G, M, k, k_clamped, _p(r), _p(vr), _p(ell), _p(out))
        return out


class Reference:
    """The reference's own hot-path functions, built by build_oracle.build_reference()."""

    def __init__(self, fast: bool = False):
        path = os.path.join(HERE, "_ref", "libnsref_fast.so" if fast else "libnsref.so")
        if not os.path.exists(path):
            raise FileNotFoundError(path)
        self.L = C.CDLL(path)
        L = self.L
        D, I = C.c_double, C.c_int
        L.ref_set_units.argtypes = [D, D]
        L.ref_set_sort.argtypes = [I]
        L.ref_adaptive_leap.argtypes = [I, I, D, D, D, D, D, D, I, I, C.POINTER(D), C.POINTER(D)]
        L.ref_adaptive_lc.argtypes = [I, I, D, D, D, D, I, D, D, I, I, C.POINTER(D), C.POINTER(D)]
        L.ref_micro_leap.argtypes = [I, I, D, D, D, D, I, I, C.POINTER(D), C.POINTER(D)]
        L.ref_sort_particles.argtypes = [C.c_void_p, I]
        L.ref_step_method5.argtypes = [C.c_void_p, I, D, I, I, D, C.c_void_p]
        L.ref_step_kdk.argtypes = [C.c_void_p, I, D, C.c_void_p]
        L.ref_lc_fixed.argtypes = [I, I, D, D, D, D, I, C.POINTER(D), C.POINTER(D)]
        L.ref_step_method4.argtypes = [C.c_void_p, I, D, I, D, I, C.c_void_p]
        L.ref_num_threads.restype = I
        L.ref_set_units(1.0, 1.0)
        L.ref_set_sort(0)

    def adaptive_leap(self, i, n, r, v, ell, h, tol_r=1e-7, tol_v=1e-7, max_subdiv=128, out_type=2):
        ro, vo = C.c_double(), C.c_double()
        self.L.ref_adaptive_leap(i, n, r, v, ell, h, tol_r, tol_v, max_subdiv, out_type, C.byref(ro), C.byref(vo))
        return ro.value, vo.value

    def adaptive_lc(self, i, n, r, v, ell, dt, N_taumin=10, tol_r=1e-7, tol_v=1e-7, max_subdiv=128, out_type=2):
        ro, vo = C.c_double(), C.c_double()
        self.L.ref_adaptive_lc(i, n, r, v, ell, dt, N_taumin, tol_r, tol_v, max_subdiv, out_type,
                               C.byref(ro), C.byref(vo))
        return ro.value, vo.value

    @staticmethod
    def _table(cols):
        tab = np.ascontiguousarray(np.array(cols, dtype=np.float64))
        rows = (C.c_void_p * tab.shape[0])(*[tab[i].ctypes.data for i in range(tab.shape[0])])
        return tab, rows

    def sort_particles(self, r, vr, ell, ids, mu=None, parallel=False):
        n = len(r)
        mu = np.zeros(n) if mu is None else mu
        tab, rows = self._table([r, vr, ell, np.asarray(ids, dtype=np.float64), mu])
        self.L.ref_set_sort(1 if parallel else 0)
        self.L.ref_sort_particles(rows, n)
        self.L.ref_set_sort(0)
        return tab

    def step_method5(self, r, vr, ell, ids, dt, max_subdiv=128, lc_rule=0, lc_radius=1e-3, parallel_sort=False):
        n = len(r)
        tab, rows = self._table([r, vr, ell, np.asarray(ids, dtype=np.float64), np.zeros(n)])
        inv = np.zeros(n, dtype=np.int32)
        self.L.ref_set_sort(1 if parallel_sort else 0)
        self.L.ref_step_method5(rows, n, dt, max_subdiv, lc_rule, lc_radius, _p(inv))
        self.L.ref_set_sort(0)
        return tab, inv

    def lc_fixed(self, i, n, r, v, ell, dt, N_taumin=1000):
        ro, vo = C.c_double(), C.c_double()
        self.L.ref_lc_fixed(i, n, r, v, ell, dt, N_taumin, C.byref(ro), C.byref(vo))
        return ro.value, vo.value

    def step_method4(self, r, vr, ell, ids, dt, max_subdiv=128, tol=1e-8, N_taumin=1000):
        n = len(r)
        tab, rows = self._table([r, vr, ell, np.asarray(ids, dtype=np.float64), np.zeros(n)])
        inv = np.zeros(n, dtype=np.int32)
        self.L.ref_step_method4(rows, n, dt, max_subdiv, tol, N_taumin, _p(inv))
        return tab, inv

    def step_kdk(self, r, vr, ell, ids, dt, parallel_sort=False):
        n = len(r)
        tab, rows = self._table([r, vr, ell, np.asarray(ids, dtype=np.float64), np.zeros(n)])
        inv = np.zeros(n, dtype=np.int32)
        self.L.ref_set_sort(1 if parallel_sort else 0)
        self.L.ref_step_kdk(rows, n, dt, _p(inv))
        self.L.ref_set_sort(0)
        return tab, inv

    def num_threads(self):
        return self.L.ref_num_threads()


def potential_energy(r, vr, ell, G=1.0, M=1.0):
    """The reference's post-processing potential and energies (nsphere.c:7697-7846) on a
    state in sorted order, in its sequential summation order: (psi, E, psi0)."""
    import numpy as np
    n = len(r)
    dM = M / n
    inv = 1.0 / r
    suffix = np.empty(n)
    acc = 0.0
    for j in range(n - 1, -1, -1):
        acc = acc + inv[j]
        suffix[j] = acc
    after = np.concatenate([suffix[1:], [0.0]])
    Mr = (np.arange(n) + 1.0) * dM
    psi = G * ((Mr / r) + dM * after)
    E = psi - (ell * ell / (2.0 * r * r)) - 0.5 * vr * vr
    s = 0.0
    for j in range(n):
        s += inv[j]
    return psi, E, G * dM * s
