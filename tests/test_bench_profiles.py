"""The bench line's measured figures come from the committed ncu summaries
(profiles/): every kernel the default line reports has its per-launch DRAM
traffic there and the flux kernel its warp-instruction count; a flux
variant gets a figure only from a capture of the same kernel code (another
launch shape at most), else none (the line then reports null)."""
import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)
bench = pytest.importorskip("bench")


@pytest.mark.parametrize("precision,kernel,key,value", [
    ("mixed", "k_q_inner", "traffic", 247258368.0),
    ("mixed", "k_q_derivatives", "traffic", 154323200.0),
    ("mixed", "k_flux_update_rps<128,7>", "traffic", 435747328.0),
    ("mixed", "k_flux_update_rps<128,7>", "inst", 138046147.0),
    ("fp64", "k_flux_update<128>", "traffic", 979463424.0),
])
def test_profiles_carry_the_bench_figures(precision, kernel, key, value):
    v, captured = bench.measured_profile("transonic", precision, kernel, key)
    assert v == value and captured == kernel


@pytest.mark.parametrize("variant", range(19))
def test_flux_variant_figures_come_from_the_same_code(variant):
    form = bench.flux_kernel_form(variant)
    v, captured = bench.measured_profile("transonic", "mixed", form + "<128,4>")
    if v is None:
        assert captured is None
    else:
        assert captured.split("<")[0] == form
    if variant in (5, 10, 17):   # the staged, register-prefetch and owner-in-shared-memory forms
        assert v is not None


def test_profiles_name_their_commands():
    pdir = os.path.join(ROOT, "profiles")
    for name in os.listdir(pdir):
        text = open(os.path.join(pdir, name)).read()
        assert "ncu " in text and "--clock-control none" in text, name
