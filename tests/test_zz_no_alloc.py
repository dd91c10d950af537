"""alisgpu_farfield_sums_static, the scratch-free far-field entry point,
against alisgpu_farfield_sums through the device C ABI: two calls in a
row of each on the same phaser and direction batch must agree within
1e-12 of the largest sum (both are the same FP64 kernel), and a batch
larger than the static array must be refused without a launch.
Collected last so that it also runs after every other GPU test."""
import os
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.mark.gpu
def test_static_far_field_matches_allocating_entry():
    from alis_gb300 import build
    build.build_engine()
    exe = build.link_program(os.path.join(ROOT, "tests", "drivers", "no_alloc.c"),
                             os.path.join(ROOT, "tests", "drivers", "bin", "no_alloc"), "engine")
    r = subprocess.run([exe], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "refused_oversize 1" in r.stdout, r.stdout
