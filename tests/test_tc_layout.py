"""The tensor-core operand layout of nsg_tc.cuh, compiled for the host, against an
independent restatement of the canonical no-swizzle K-major layout of tcgen05
shared-memory operands: core matrices of 8 rows x 16 bytes, 128 contiguous bytes each,
cores adjacent along K one leading byte offset apart and cores adjacent along the rows
one stride byte offset (128 bytes) apart.  Checks that every element of each tile
shape the MLP inference uses has its own 2-byte slot inside the tile, that an MMA's
K = 16 slice is the two column groups the descriptor's offsets reach, and the bit
fields of the shared-memory and instruction descriptors (start address, leading and
stride offsets >> 4 at bits 0, 16, 32; version 1 at bit 46; no-swizzle layout 0 at
bits 61-63; FP32 accumulator at bit 4, BF16 A and B at bits 7 and 10, K-major, N >> 3
at bit 17, M >> 4 at bit 24)."""
import os
import subprocess

import pytest

from conftest import ROOT


@pytest.fixture(scope="module")
def dump(tmp_path_factory):
    exe = str(tmp_path_factory.mktemp("tc") / "tc_layout_check")
    subprocess.run(["g++", "-O1", "-std=c++17", "-I", os.path.join(ROOT, "nsphere_gb300", "csrc"),
                    os.path.join(ROOT, "tests", "tc_layout_check.cpp"), "-o", exe], check=True)
    return subprocess.run([exe], capture_output=True, text=True, check=True).stdout.split("\n")


def _tiles(lines):
    tiles, i = {}, 0
    while i < len(lines) and lines[i].startswith("tile"):
        _, R, K, _, lbo = lines[i].split()
        R, K, lbo = int(R), int(K), int(lbo)
        offs = [int(x) for x in lines[i + 1:i + 1 + R * K]]
        tiles[(R, K)] = (lbo, offs)
        i += 1 + R * K
    return tiles, lines[i:]


def test_operand_layout(dump):
    tiles, _ = _tiles(dump)
    assert set(tiles) == {(128, 16), (128, 64), (64, 16), (64, 64), (16, 64)}
    for (R, K), (lbo, offs) in tiles.items():
        assert lbo == (R // 8) * 128
        # a bijection onto the tile's 2-byte slots
        assert sorted(offs) == list(range(0, R * K * 2, 2))
        for row in range(R):
            for k in range(K):
                o = offs[row * K + k]
                core = (k // 8) * lbo + (row // 8) * 128      # leading (K) and stride (row) offsets
                assert o == core + (row % 8) * 16 + (k % 8) * 2
        # the MMA of K slice s starts at column group 2 s, i.e. 2 s leading offsets in
        for s in range(K // 16):
            assert offs[16 * s] == 2 * s * lbo


def test_descriptors(dump):
    _, rest = _tiles(dump)
    descs = [l.split() for l in rest if l.startswith("desc")]
    idescs = [l.split() for l in rest if l.startswith("idesc")]
    assert len(descs) == 18 and len(idescs) == 3
    for _, a, lbo, d in descs:
        a, lbo, d = int(a), int(lbo), int(d)
        assert d & 0x3FFF == (a >> 4) & 0x3FFF
        assert (d >> 16) & 0x3FFF == lbo >> 4
        assert (d >> 32) & 0x3FFF == 128 >> 4
        assert (d >> 46) & 0x3 == 1          # descriptor version
        assert (d >> 49) & 0x7 == 0          # base offset
        assert (d >> 52) & 0x1 == 0          # leading offset mode
        assert (d >> 61) & 0x7 == 0          # no swizzle
        assert d & ~((0x3FFF) | (0x3FFF << 16) | (0x3FFF << 32) | (1 << 46)) == 0
    for _, n, w in idescs:
        n, w = int(n), int(w)
        assert (w >> 4) & 0x3 == 1           # FP32 accumulator
        assert (w >> 7) & 0x7 == 1 and (w >> 10) & 0x7 == 1   # BF16 A and B
        assert (w >> 13) & 0x3 == 0          # no negation
        assert (w >> 15) & 0x3 == 0          # both K-major
        assert (w >> 17) & 0x3F == n >> 3
        assert (w >> 24) & 0x1F == 128 >> 4
        assert w & 0x3 == 0 and (w >> 2) & 0x3 == 0 and (w >> 30) == 0
