"""The device voxelizer against the host loops: the same object list
(seeded balls and rods, a rotation, lattices, a set difference, plain
and dispersive matter) put into a world by the engine (device
voxelizer) and by the oracle build (the same host layer's loops, on the
host cores) must give byte-identical eps^-1 and fill maps (hash over all
of them), with voxelizer launches in the engine run.  A list holding a
height-map object stays with the engine's host loops.  Supersampled,
point-sampled and edge-rule filling.  The parity scenes cover the same
path at their own sizes."""
import os
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _run(exe, args):
    r = subprocess.run([exe] + [str(a) for a in args], capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stdout + r.stderr
    out = {}
    for line in r.stdout.splitlines():
        parts = line.split()
        if len(parts) == 2 and parts[0] in ("cells", "dispersive", "launches", "seconds", "hash"):
            out[parts[0]] = parts[1]
    assert "hash" in out, r.stdout + r.stderr
    return out


@pytest.fixture(scope="module")
def exe():
    from alis_gb300 import build
    build.build_engine()
    build.build_oracle()
    src = os.path.join(ROOT, "tests", "drivers", "vox_device.c")
    out = os.path.join(ROOT, "tests", "drivers", "bin", "vox_")
    return {a: build.link_program(src, out + a, a) for a in ("engine", "oracle")}


@pytest.mark.gpu
@pytest.mark.parametrize("size,subN", [(300, 6), (300, 1), (300, -1), (600, 12)],
                         ids=["sub6", "point", "edge", "sub12-large"])
def test_device_voxelizer_matches_host_loops(exe, size, subN):
    dev = _run(exe["engine"], [size, subN])
    host = _run(exe["oracle"], [size, subN])
    assert int(dev["dispersive"]) > 0
    assert dev["hash"] == host["hash"]
    assert int(dev["launches"]) > 0 and int(host["launches"]) == 0
    print("voxelize %s cells subN %d: device %.3f s, host loops %.3f s" %
          (dev["cells"], subN, float(dev["seconds"]), float(host["seconds"])))


@pytest.mark.gpu
def test_height_map_list_stays_on_host(exe):
    """A list with a height map runs the engine's host loops: no voxelizer
    launches, the oracle's maps."""
    dev = _run(exe["engine"], [300, 4, "contour"])
    host = _run(exe["oracle"], [300, 4, "contour"])
    assert dev["hash"] == host["hash"]
    assert int(dev["launches"]) == 0
