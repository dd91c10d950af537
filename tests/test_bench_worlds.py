"""The CPU program behind bench.py's host-core baseline builds the vacuum
plane-wave world at 128^3 cells (periodic x/y, the 16-cell z CPML counted
in) with its 16 phaser wavelengths, and reports the outgoing flux of each;
two runs of the same steps report the same spectrum."""
import json
import os
import subprocess

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def run(steps, warm):
    import sys
    sys.path.insert(0, ROOT)
    import bench
    exe = bench.build_cpu_baseline()
    env = dict(os.environ, OMP_NUM_THREADS="4")
    r = subprocess.run([exe, "c1", str(steps), str(warm)], capture_output=True, text=True, env=env, timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    return json.loads([l for l in r.stdout.splitlines() if l.startswith("{")][-1])


def test_plane_wave_world_and_spectrum():
    a = run(300, 3)
    assert a["cells"] == 128 ** 3
    assert a["steps"] == 300
    assert len(a["flux"]) == 16
    assert any(v != 0 for v in a["flux"])
    b = run(300, 3)
    assert a["flux"] == b["flux"]
