"""The served form (alis_gb300/bench/serve.c): a Poisson stream of mixed
requests -- vacuum with a dielectric ball, Drude bowtie antennas,
photonic-crystal k-point runs with complex fields -- admitted by device
footprint and stepped in turn, each world on streams of its own so that
their work overlaps on the device.  Every request's result (its outgoing
phaser flux summed over frequencies and k-points) must be bit-identical
in the mix, run one after another on the default streams, and run alone,
and the same as the oracle's result for that request: the request loop
built against the oracle runs the same seeded stream one request after
another on the host cores.  Prints the throughput of the served and the sequential runs and the
served latency percentiles."""
import json
import os
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _oracle_serve():
    from alis_gb300 import build
    build.build_oracle()
    return build.link_program(os.path.join(ROOT, "alis_gb300", "bench", "serve.c"),
                              os.path.join(ROOT, "tests", "drivers", "bin", "serve_oracle"), "oracle", extra=["-lm"])


def _run(exe, args, env=None):
    r = subprocess.run([exe] + [str(a) for a in args], capture_output=True, text=True, timeout=900, env=env)
    assert r.returncode == 0, r.stdout[-2000:] + r.stderr[-2000:]
    res, summary = {}, None
    for line in r.stdout.splitlines():
        p = line.split()
        if p and p[0] == "R":
            res[int(p[1])] = (int(p[2]), p[6])
        elif line.startswith("{"):
            summary = json.loads(line)
    assert summary is not None, r.stdout[-2000:]
    return res, summary


@pytest.mark.gpu
def test_served_results_equal_alone_and_sequential():
    from alis_gb300 import build
    build.build_engine()
    exe = build.link_program(os.path.join(ROOT, "alis_gb300", "bench", "serve.c"),
                             os.path.join(ROOT, "tests", "drivers", "bin", "serve"), "engine", extra=["-lm"])
    n, seed = 24, 7
    served, s1 = _run(exe, ["served", n, 2000, seed, "small", 8])
    seq, s2 = _run(exe, ["sequential", n, 2000, seed, "small"])
    assert len(served) == n and len(seq) == n
    for q in range(n):
        assert served[q] == seq[q], (q, served[q], seq[q])
    # alone: one request of each kind
    kinds = {}
    for q in range(n):
        kinds.setdefault(served[q][0], q)
    assert set(kinds) == {0, 1, 2}
    for kind, q in sorted(kinds.items()):
        alone, _ = _run(exe, ["alone", n, 2000, seed, "small", q])
        assert alone[q] == served[q], (q, alone[q], served[q])
    # the oracle, the same stream one request after another
    oracle, _ = _run(_oracle_serve(), ["sequential", n, 2000, seed, "small"])
    assert len(oracle) == n
    for q in range(n):
        assert oracle[q] == served[q], (q, oracle[q], served[q])
    print("served %.2f Gcell/s (p50 %.1f ms, p99 %.1f ms), sequential %.2f Gcell/s" %
          (s1["gcell_per_s"], s1["latency_ms"]["p50"], s1["latency_ms"]["p99"], s2["gcell_per_s"]))


@pytest.mark.gpu
def test_served_unit_cell_sweep_equals_sequential():
    """The metasurface sweep mix (periodic unit cells with a TFSF pulse and
    a transmission plane), shortened to 400 steps per cell: served,
    sequential and the oracle's results identical per request."""
    from alis_gb300 import build
    build.build_engine()
    exe = build.link_program(os.path.join(ROOT, "alis_gb300", "bench", "serve.c"),
                             os.path.join(ROOT, "tests", "drivers", "bin", "serve"), "engine", extra=["-lm"])
    env = dict(os.environ, SERVE_STEPS="400")
    served, s1 = _run(exe, ["served", 12, 2000, 7, "sweep", 8], env)
    seq, s2 = _run(exe, ["sequential", 12, 2000, 7, "sweep"], env)
    assert len(served) == 12 and served == seq
    assert any(int(v[1], 16) for v in served.values())
    oracle, _ = _run(_oracle_serve(), ["sequential", 12, 2000, 7, "sweep"], env)
    assert oracle == served
    print("sweep: served %.2f Gcell/s, sequential %.2f Gcell/s" % (s1["gcell_per_s"], s2["gcell_per_s"]))


@pytest.mark.gpu
@pytest.mark.parametrize("mix,n,env", [("small", 24, {}), ("sweep", 12, {"SERVE_STEPS": "400"})], ids=["small", "sweep"])
def test_batched_results_equal_sequential(mix, n, env):
    """The batched form (alisBatchBegin/End: every step of a wave of
    requests as a few launches over all their worlds, recorded by several
    host threads) gives every request the bytes it gets one request after
    another."""
    from alis_gb300 import build
    build.build_engine()
    exe = build.link_program(os.path.join(ROOT, "alis_gb300", "bench", "serve.c"),
                             os.path.join(ROOT, "tests", "drivers", "bin", "serve"), "engine", extra=["-lm"])
    e = dict(os.environ, **env)
    batched, s1 = _run(exe, ["batched", n, 2000, 7, mix, 8], e)
    seq, s2 = _run(exe, ["sequential", n, 2000, 7, mix], e)
    assert len(batched) == n and batched == seq
    print("%s: batched %.2f Gcell/s, sequential %.2f Gcell/s" % (mix, s1["gcell_per_s"], s2["gcell_per_s"]))
