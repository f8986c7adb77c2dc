"""Build recipe of the CPU checkers (test infrastructure only).

* ``liborc.so``: the C restatement ``oracle/nsg_oracle.c``.
* ``_ref/libnsref.so`` and ``_ref/libnsref_fast.so``: the reference's own hot-path
  functions.  The reference (kris-sigurdson/NSphere, ``src/c/nsphere.c``) is one
  C file that needs GSL and FFTW, which this machine does not have; its step-path
  functions do not.  ``extract_reference()`` therefore copies the line ranges
  below -- forces, integrators, sort subsystem -- and the vendored quadsort headers
  into ``oracle/_ref/`` (git-ignored build output), and ``ref_harness.c`` wraps
  them.  The copy travels with the working tree, so the reference compiles on a
  machine without the reference checkout too.

Flags: ``-O2 -fno-fast-math -ffp-contract=off`` for parity (IEEE rounding of every
operation, no fused multiply-add); the timing build uses the reference's release
flags (Makefile.Linux:13-20, 63-74): ``-march=native -DQUAD_CACHE=<half the L3
cache that /proc/cpuinfo reports, 6 MiB when it reports none, at least 256 KiB>
-fopenmp -funroll-loops -ffast-math -fno-math-errno -ffp-contract=fast``, with gcc
for the absent clang and ``-O2`` for ``-Ofast`` (gcc at -O3 miscompiles the
reference's parallel quadsort into a double free).

The reference checkout is read from ``NSG_REFERENCE_DIR``, else from a directory
named ``reference`` beside the repository.
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
REF_OUT = os.path.join(HERE, "_ref")
# a checkout beside the repository, when NSG_REFERENCE_DIR does not name one
SIBLING_REFERENCE = os.path.join(os.path.dirname(os.path.dirname(HERE)), "reference")

# (first, last) line ranges of src/c/nsphere.c, inclusive
REF_RANGES = [
    (476, 599),    # use_identity_gravity, gravitational_force, effective_angular_force, LC forces
    (1550, 2334),  # doMicroLeapfrog .. doAdaptiveFullLeviCivita
    (8280, 8665),  # sort subsystem: compare_particles .. sort_particles
]
REF_SORT_FILES = ["nsphere_sort.h", "quadsort.h", "quadsort.c"]

PARITY_FLAGS = ["-O2", "-fno-fast-math", "-ffp-contract=off", "-fopenmp", "-fPIC", "-shared"]


def quad_cache_bytes() -> int:
    """QUAD_CACHE as Makefile.Linux:13-20 computes it: half the 'cache size' line of
    /proc/cpuinfo (KiB), 6144 KiB when there is none, at least 256 KiB."""
    kb = 6144
    try:
        with open("/proc/cpuinfo") as f:
            for line in f:
                if line.startswith("cache size"):
                    kb = int(line.split(":")[1].split()[0])
                    break
    except (OSError, ValueError, IndexError):
        pass
    return max(kb * 1024 // 2, 262144)


def _native_flag() -> list:
    """-march=native where gcc accepts it for this host (the reference's flag)."""
    r = subprocess.run(["gcc", "-march=native", "-x", "c", "-c", "-o", os.devnull, "-"],
                       input="int x;\n", capture_output=True, text=True)
    return ["-march=native"] if r.returncode == 0 else []


FAST_BASE = ["-O2", "-fopenmp", "-funroll-loops", "-ffast-math", "-fno-math-errno", "-ffp-contract=fast",
             "-fPIC", "-shared"]


def fast_flags() -> list:
    return ["-O2", *_native_flag(), "-DQUAD_CACHE=%d" % quad_cache_bytes(), *FAST_BASE[1:]]


def _run(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("command failed: %s\n%s%s" % (" ".join(cmd), r.stdout, r.stderr))


def build_oracle(verbose: bool = False) -> str:
    out = os.path.join(HERE, "liborc.so")
    src = os.path.join(HERE, "nsg_oracle.c")
    if not os.path.exists(out) or os.path.getmtime(out) < max(
            os.path.getmtime(src), os.path.getmtime(os.path.join(HERE, "nsg_oracle.h"))):
        _run(["gcc", *PARITY_FLAGS, "-I", HERE, src, "-o", out, "-lm"])
        if verbose:
            print("built", out)
    return out


def extract_reference(reference_dir: str | None = None) -> bool:
    """Writes oracle/_ref/ref_hotpath.c from the reference checkout, if present."""
    ref = reference_dir or os.environ.get("NSG_REFERENCE_DIR") or SIBLING_REFERENCE
    src = os.path.join(ref, "src", "c", "nsphere.c")
    if not os.path.exists(src):
        return False
    os.makedirs(REF_OUT, exist_ok=True)
    with open(src, encoding="utf-8", errors="replace") as f:
        lines = f.read().split("\n")
    parts = ['#include "ref_prelude.h"\n', '#include "nsphere_sort.h"\n']
    for a, b in REF_RANGES:
        parts.append("#line %d \"nsphere.c\"\n" % a)
        parts.append("\n".join(lines[a - 1:b]) + "\n")
    with open(os.path.join(REF_OUT, "ref_hotpath.c"), "w") as f:
        f.write("".join(parts))
    for name in REF_SORT_FILES:
        shutil.copyfile(os.path.join(ref, "src", "c", name), os.path.join(REF_OUT, name))
    return True


def build_reference(verbose: bool = False) -> bool:
    """Builds oracle/_ref/libnsref{,_fast}.so when the extracted sources exist."""
    extract_reference()
    hot = os.path.join(REF_OUT, "ref_hotpath.c")
    if not os.path.exists(hot):
        return False
    harness = os.path.join(HERE, "ref_harness.c")
    newest = max(os.path.getmtime(hot), os.path.getmtime(harness),
                 os.path.getmtime(os.path.join(HERE, "ref_prelude.h")))
    for name, flags in (("libnsref.so", PARITY_FLAGS), ("libnsref_fast.so", None)):
        out = os.path.join(REF_OUT, name)
        if os.path.exists(out) and os.path.getmtime(out) >= newest:
            continue
        flags = flags or fast_flags()
        _run(["gcc", *flags, "-w", "-I", REF_OUT, "-I", HERE, harness, "-o", out, "-lm"])
        if name == "libnsref_fast.so":
            with open(os.path.join(REF_OUT, "fast_flags.txt"), "w") as f:
                f.write("gcc " + " ".join(flags) + "\n")
        if verbose:
            print("built", out)
    return True


def fast_flags_used() -> str:
    """The command-line flags of the last timing build of the reference."""
    try:
        with open(os.path.join(REF_OUT, "fast_flags.txt")) as f:
            return f.read().strip()
    except OSError:
        return "gcc " + " ".join(FAST_BASE)


if __name__ == "__main__":
    build_oracle(verbose=True)
    ok = build_reference(verbose=True)
    print("reference build:", "ok" if ok else "skipped (no reference sources)")
    sys.exit(0)
