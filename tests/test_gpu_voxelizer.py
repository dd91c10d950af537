"""The device voxelizer against the engine's own host loops: the same
object list (seeded balls and rods, a rotation, lattices, a set
difference, plain and dispersive matter) put into a world by two
processes, one with ALISGPU_VOXELIZE=host, must give byte-identical
eps^-1 and fill maps (hash over all of them), with voxelizer launches
only in the device run.  A list holding a height-map object stays with
the host loops in both.  Supersampled, point-sampled and edge-rule
filling.  The parity scenes cover the same path against the oracle."""
import os
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _run(exe, args, host):
    env = dict(os.environ)
    if host:
        env["ALISGPU_VOXELIZE"] = "host"
    else:
        env.pop("ALISGPU_VOXELIZE", None)
    r = subprocess.run([exe] + [str(a) for a in args], capture_output=True, text=True, timeout=600, env=env)
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
    return build.link_program(os.path.join(ROOT, "tests", "drivers", "vox_device.c"),
                              os.path.join(ROOT, "tests", "drivers", "bin", "vox_device"), "engine")


@pytest.mark.gpu
@pytest.mark.parametrize("size,subN", [(300, 6), (300, 1), (300, -1), (600, 12)],
                         ids=["sub6", "point", "edge", "sub12-large"])
def test_device_voxelizer_matches_host_loops(exe, size, subN):
    dev = _run(exe, [size, subN], host=False)
    host = _run(exe, [size, subN], host=True)
    assert int(dev["dispersive"]) > 0
    assert dev["hash"] == host["hash"]
    assert int(dev["launches"]) > int(host["launches"])
    print("voxelize %s cells subN %d: device %.3f s, host loops %.3f s" %
          (dev["cells"], subN, float(dev["seconds"]), float(host["seconds"])))


@pytest.mark.gpu
def test_height_map_list_stays_on_host(exe):
    dev = _run(exe, [300, 4, "contour"], host=False)
    host = _run(exe, [300, 4, "contour"], host=True)
    assert dev["hash"] == host["hash"]
    assert dev["launches"] == host["launches"]
