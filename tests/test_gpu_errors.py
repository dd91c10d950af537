"""Error paths of the device C ABI, exercised without a GPU fault: the
far-field entry points (alisgpu_farfield_sums and its scratch-free
variant) refuse a frequency outside the phaser's and test fields shorter
than the phaser box with ALISGPU_EINVAL, and an allocation failure --
injected on the host by alisgpu_inject_alloc_failures -- returns
ALISGPU_ENOMEM; none of them launches a kernel, and a call after them
gives the same sums as before.  alisgpu_world_set_storage refuses a world
already written (ALISGPU_EINVAL), a bad kind (ALISGPU_EINVAL) and complex
fields (ALISGPU_ENOTSUP); a half world refuses field uploads
(ALISGPU_ENOTSUP), downloads zeros before its first step, holds fewer
bytes, and may go back to float storage before it is stepped."""
import os
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.mark.gpu
def test_far_field_error_paths_launch_nothing():
    from alis_gb300 import build
    build.build_engine()
    exe = build.link_program(os.path.join(ROOT, "tests", "drivers", "no_alloc.c"),
                             os.path.join(ROOT, "tests", "drivers", "bin", "no_alloc"), "engine")
    r = subprocess.run([exe, "errors"], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "launched 0 same_after 1" in r.stdout, r.stdout
    assert "storage 1 " in r.stdout, r.stdout
