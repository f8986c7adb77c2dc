"""C-ABI checks that need no GPU: the library loads, exports every entry point that
include/nsg.h declares, reports defaults, rejects bad arguments, and refuses to
run without a GPU (there is no CPU fallback)."""
import ctypes as C
import os
import re
import subprocess

import pytest

from conftest import ROOT


def _declared():
    names = set()
    for h in os.listdir(os.path.join(ROOT, "include")):
        if h.endswith(".h"):
            txt = open(os.path.join(ROOT, "include", h)).read()
            txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
            names |= set(re.findall(r"\b(nsg_[a-z0-9_]+)\s*\(", txt))
    return names


def test_exports_every_declared_symbol(nsg):
    out = subprocess.run(["nm", "-D", "--defined-only", nsg.LIB_PATH], capture_output=True, text=True).stdout
    exported = set(re.findall(r"\bT (nsg_[a-z0-9_]+)", out))
    declared = _declared()
    assert declared, "no declarations parsed"
    missing = declared - exported
    assert not missing, "declared but not exported: %s" % sorted(missing)
    assert set(nsg.EXPORTS) <= exported


def test_params_layout_and_defaults(nsg):
    p = nsg.default_params()
    assert p.G == 1.0 and p.M_total == 1.0
    assert p.tol_r == 1e-7 and p.tol_v == 1e-7
    assert p.max_subdiv == 4096 * 4096 * 16
    assert p.out_type == 2 and p.N_taumin == 10 and p.lc_alpha == 0.05
    assert p.method == nsg.METHOD_ADAPTIVE_LC and p.lc_rule == nsg.LC_RCRIT
    assert p.max_tau_steps == 100000000
    # struct size as compiled in C (checked against a tiny C program)
    src = '#include "nsg.h"\n#include <stdio.h>\nint main(){printf("%zu",sizeof(nsg_params));return 0;}\n'
    exe = os.path.join(ROOT, "nsphere_gb300", "_build", "sizeof_params")
    os.makedirs(os.path.dirname(exe), exist_ok=True)
    cfile = exe + ".c"
    open(cfile, "w").write(src)
    subprocess.run(["gcc", "-I", os.path.join(ROOT, "include"), cfile, "-o", exe], check=True)
    size = int(subprocess.run([exe], capture_output=True, text=True).stdout)
    assert size == C.sizeof(nsg.Params)


def test_null_and_bad_arguments(nsg):
    L = nsg.lib()
    assert L.nsg_params_default(None) == nsg.NSG_EINVAL
    assert L.nsg_create(None, None, None) == nsg.NSG_EINVAL
    h = C.c_void_p()
    bad = nsg.default_params(dt=-1.0)
    assert L.nsg_create(C.byref(h), C.byref(bad), None) == nsg.NSG_EINVAL
    assert b"dt" in L.nsg_last_error(None)
    bad = nsg.default_params(method=7)
    assert L.nsg_create(C.byref(h), C.byref(bad), None) == nsg.NSG_EINVAL
    assert L.nsg_step(None, 1) == nsg.NSG_EINVAL
    assert L.nsg_upload(None, None, None, None, None, None, 0) == nsg.NSG_EINVAL


def test_no_gpu_means_error_not_fallback(nsg):
    """Without a CUDA device nsg_create must fail with NSG_ECUDA (no CPU path)."""
    try:
        import torch
        if torch.cuda.is_available():
            pytest.skip("a GPU is present")
    except ImportError:
        pass
    L = nsg.lib()
    h = C.c_void_p()
    p = nsg.default_params()
    rc = L.nsg_create(C.byref(h), C.byref(p), None)
    assert rc == nsg.NSG_ECUDA
    assert len(L.nsg_last_error(None)) > 0


def test_header_constants_match_python_mirror(nsg):
    """Every NSG_* integer constant of include/nsg.h has the same value in the Python
    mirror (status codes, status bits, methods, rules, schedules, IC models)."""
    txt = open(os.path.join(ROOT, "include", "nsg.h")).read()
    consts = dict(re.findall(r"#define\s+NSG_([A-Z0-9_]+)\s+\(?(-?(?:0x[0-9a-fA-F]+|\d+))u?\)?", txt))
    assert len(consts) > 15
    checked = 0
    for name, val in consts.items():
        for py in (name, "NSG_" + name):
            if hasattr(nsg, py):
                assert getattr(nsg, py) == int(val, 0), (name, val, getattr(nsg, py))
                checked += 1
                break
    assert checked >= 15
    assert nsg.ST_DEVICE_WAIT == 0x40
