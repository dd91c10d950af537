"""The CPU program behind bench.py's host-core baseline builds the vacuum
plane-wave world at 128^3 cells (periodic x/y, the 16-cell z CPML counted
in) with its 16 phaser wavelengths, and reports the outgoing flux of each;
two runs of the same steps report the same spectrum.  On the GPU, the
whole 2000-step job of that world through the engine reproduces the host
cores' spectrum within 1e-5 of the largest flux.  The large-domain
workload's 200 seeded balls lie inside the domain, meet no other ball and
come out the same on every draw."""
import json
import os
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def run(steps, warm):
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


@pytest.mark.gpu
def test_plane_wave_job_spectrum_matches_host_cores():
    r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--workload", "c1", "--steps", "2000",
                        "--warmup", "16", "--cpu-steps", "2000", "--forms", "0"],
                       capture_output=True, text=True, timeout=900, cwd=ROOT)
    assert r.returncode == 0, r.stderr[-2000:]
    line = json.loads([l for l in r.stdout.splitlines() if l.startswith("{")][-1])
    assert line["config"]["cells"] == 128 ** 3
    check = line["spectrum_vs_cpu"]
    assert check["frequencies"] == 16 and check["steps"] == line["warmup"] + 2000
    assert check["within"] and check["max_rel_diff"] <= 1e-5, check


def test_large_domain_balls_inside_and_apart(tmp_path):
    import numpy as np
    exe = str(tmp_path / "c5_balls_check")
    src = os.path.join(ROOT, "tests", "drivers", "c5_balls_check.c")
    subprocess.run(["gcc", "-std=gnu99", "-O2", src, "-o", exe], check=True)
    args = [exe, "99", "200", "1024", "1024", "512", "5"]
    out = subprocess.run(args, capture_output=True, text=True, check=True).stdout
    assert out == subprocess.run(args, capture_output=True, text=True, check=True).stdout
    lines = out.strip().splitlines()
    dom = [float(v) for v in lines[-1].split()[1:]]
    B = np.array([[float(v) for v in l.split()] for l in lines[:-1]])
    assert B.shape == (200, 4)
    x, r = B[:, :3], B[:, 3]
    assert ((r >= 5 * 20) & (r <= 5 * 80)).all()
    for a in range(3):
        assert (x[:, a] - r >= dom[2 * a] - 1e-3).all() and (x[:, a] + r <= dom[2 * a + 1] + 1e-3).all()
    d = np.sqrt(((x[:, None, :] - x[None, :, :]) ** 2).sum(-1))
    np.fill_diagonal(d, np.inf)
    assert (d >= r[:, None] + r[None, :] - 1e-3).all()
