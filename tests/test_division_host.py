"""The integer/FP32 division routines of nsg_div.cuh, compiled for the host, give
the CPU's IEEE quotient bit for bit on every operand pair they claim, also when
the reciprocal estimate they start from is perturbed within its error bound; the
integer-pipe multiplication of nsg_mul.cuh gives the CPU's IEEE product bit for bit
on every pair it claims and claims every product in the normal range."""
import os
import subprocess

import pytest

from conftest import ROOT


@pytest.fixture(scope="module")
def checker(tmp_path_factory):
    exe = str(tmp_path_factory.mktemp("div") / "div_host_check")
    subprocess.run(["g++", "-O2", "-std=c++17", "-fno-fast-math", "-ffp-contract=off",
                    "-I", os.path.join(ROOT, "nsphere_gb300", "csrc"),
                    os.path.join(ROOT, "tests", "div_host_check.cpp"), "-o", exe], check=True)
    return exe


@pytest.mark.parametrize("ulps", [0, 2, -2, 4, -4, 8, -8, 16])
def test_division_matches_ieee(checker, ulps):
    out = subprocess.run([checker, str(ulps), "1500000"], capture_output=True, text=True)
    assert out.returncode == 0, out.stdout + out.stderr
    claimed = int(out.stdout.split("lat claimed")[1].split(",")[0])
    assert claimed > 1_400_000


def test_multiplication_matches_ieee(tmp_path):
    exe = str(tmp_path / "mul_host_check")
    subprocess.run(["g++", "-O2", "-std=c++17", "-fno-fast-math", "-ffp-contract=off",
                    "-I", os.path.join(ROOT, "nsphere_gb300", "csrc"),
                    os.path.join(ROOT, "tests", "mul_host_check.cpp"), "-o", exe], check=True)
    out = subprocess.run([exe, "3000000"], capture_output=True, text=True)
    assert out.returncode == 0, out.stdout + out.stderr
    claimed = int(out.stdout.split("claimed ")[1].split(" ")[0])
    assert claimed > 2_000_000
