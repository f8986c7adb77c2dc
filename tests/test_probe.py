"""The latency probes the Levi-Civita design rests on: a warp does not overlap its
own FP64 instructions, two warps do, and the latency-oriented division is shorter
than the FP64 pipe's."""
import pytest

pytestmark = pytest.mark.gpu


def test_latency_probe(nsg):
    c = nsg.probe_latency()
    assert all(v > 0 for v in c.values()), c
    # two independent chains in one warp take about twice one chain ...
    assert c["fp64_fma_two_chains_one_warp"] > 1.6 * c["fp64_fma"]
    # ... while one chain in each of two warps does not
    assert c["fp64_fma_one_chain_two_warps"] < 1.3 * c["fp64_fma"]
    assert c["div_latency_form"] < c["div_fp64_pipe"]
    assert c["levi_civita_substep_zero_gravity"] < c["levi_civita_substep"]
