"""The request loop of the served form (alis_gb300/bench/serve.c) on the
host: built against the oracle, a few small requests of the mixed stream
and of the unit-cell sweep run one after another and alone, and each
request's result must be the same both ways.  (The GPU tests run the
served, concurrent form.)"""
import os
import subprocess

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _results(exe, args, env):
    r = subprocess.run([exe] + [str(a) for a in args], capture_output=True, text=True, timeout=600, env=env)
    assert r.returncode == 0, r.stdout[-2000:] + r.stderr[-2000:]
    out = {}
    for line in r.stdout.splitlines():
        p = line.split()
        if p and p[0] == "R":
            out[int(p[1])] = p[6]
    assert any(l.startswith("{") for l in r.stdout.splitlines())
    return out


def test_request_loop_alone_equals_sequential_on_the_oracle(tmp_path):
    from alis_gb300 import build
    build.build_oracle()
    exe = build.link_program(os.path.join(ROOT, "alis_gb300", "bench", "serve.c"), str(tmp_path / "serve_oracle"), "oracle")
    env = dict(os.environ, OMP_NUM_THREADS="4", SERVE_STEPS="30")
    seq = _results(exe, ["sequential", 3, 100, 7, "small"], env)
    assert len(seq) == 3
    alone = _results(exe, ["alone", 3, 100, 7, "small", 2], env)
    assert alone == {2: seq[2]}
    sweep = _results(exe, ["sequential", 2, 100, 7, "sweep"], env)
    assert len(sweep) == 2
