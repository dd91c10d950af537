"""The multi-process (replica) path of bench.py on CPU: two gloo ranks
launched by torch.distributed.run on 127.0.0.1.  The reference arm runs
on rank 0 only and prints one JSON line; rank 1 exits 0 without work.
The rank helpers take the maximum over ranks."""
import json
import os
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _torchrun(args, nproc=2, timeout=600):
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node", str(nproc),
           "--master-addr", "127.0.0.1", "--master-port", "29533"] + args
    env = dict(os.environ, OMP_NUM_THREADS="2")
    return subprocess.run(cmd, cwd=ROOT, capture_output=True, text=True, timeout=timeout, env=env)


def test_reference_arm_two_ranks():
    pytest.importorskip("torch")
    r = _torchrun(["bench.py", "--impl", "reference", "--gpus", "2", "--steps", "2", "--warmup", "3", "--half", "60"])
    assert r.returncode == 0, r.stdout[-2000:] + r.stderr[-2000:]
    lines = [l for l in r.stdout.splitlines() if l.startswith("{")]
    assert len(lines) == 1, r.stdout
    line = json.loads(lines[0])
    assert line["impl"] == "reference" and line["n_gpus"] == 2
    assert line["value"] > 0 and line["e2e"]["value"] == line["value"]
    assert line["cpu_baseline"]["kind"] == "port"


RANKS = r'''
import os, sys
sys.path.insert(0, %r)
import torch.distributed as dist
dist.init_process_group("gloo")
import bench
rank, world, _ = bench.env_rank()
got = bench.reduce_max(float(rank + 1) * 0.5, world)
bench.barrier(world)
assert got == world * 0.5, got
if rank == 0:
    print("rank", rank, "max", got, flush=True)
dist.destroy_process_group()
'''


def test_reduce_max_two_ranks(tmp_path):
    pytest.importorskip("torch")
    script = tmp_path / "ranks.py"
    script.write_text(RANKS % ROOT)
    r = _torchrun([str(script)])
    assert r.returncode == 0, r.stdout[-2000:] + r.stderr[-2000:]
    assert "max 1.0" in r.stdout


def test_form_processes_leave_the_torchrun_group(monkeypatch):
    """The forms that run bench.py again in a process of their own do so
    as a single process on the rank's device: without the torchrun
    group's variables, with ALISGPU_DEVICE."""
    import bench
    seen = {}

    class Failed:
        returncode, stdout, stderr = 1, "", "not run"

    def fake_run(cmd, **kw):
        seen.update(kw.get("env") or {})
        return Failed()

    for k, v in (("RANK", "1"), ("WORLD_SIZE", "2"), ("LOCAL_RANK", "1"), ("MASTER_ADDR", "127.0.0.1"),
                 ("MASTER_PORT", "29500"), ("ALISGPU_DEVICE", "1")):
        monkeypatch.setenv(k, v)
    monkeypatch.setattr(bench.subprocess, "run", fake_run)
    line, err = bench.bench_line(["--workload", "c1"])
    assert line is None and err
    assert not {"RANK", "WORLD_SIZE", "LOCAL_RANK", "MASTER_ADDR", "MASTER_PORT"} & set(seen)
    assert seen.get("ALISGPU_DEVICE") == "1"
