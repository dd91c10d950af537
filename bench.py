"""Benchmark of the GB300 ALiS engine on the dispersive-scatterer workload.

One step = updateE + updateH + updatePhaser of the 256^3-cell world of
alis_gb300/bench/c2.c (gold block with Drude + 2 critical-point poles,
TFSF plane wave, CPML on all faces, 64-frequency box phasers), driven
through the public ALiS C API exactly as a user program does.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl engine|reference]

value     cells x steps / device time (CUDA events on the engine stream;
          fields resident in HBM; the 1.5 GB per step of field traffic
          exceeds the 129 MB L2, so no L2 flush is needed).  The K-step
          window is timed R times back to back, R chosen so that the R K
          steps are a whole number of phaser ring periods (64 steps) and
          last about a second: every window's time counts, so the phaser
          DFT flush, which runs once per ring period, is charged at its
          own rate whatever K is
e2e       the same through the public API timed on the host: R windows of
          K steps, each followed by the flux result (face fluxes reduced
          on the device, read back)
roofline  the fused half-step kernel: algorithmic bytes per step (84 B per
          cell, +32 B per CPML slab, ADE terms) over the mean E + H launch
          time, against the measured HBM copy bandwidth (frac) and the
          nominal 8 TB/s (frac_nominal)
cpu_baseline  the oracle restatement of the reference loops on the host
          cores (OpenMP), bounded sample of the same world
--impl reference  times that CPU implementation alone as the reference arm.
forms     the batched unit-cell sweep (64 cells) and the served request
          stream, each against its per-request path; the same workload
          with half field storage; the vacuum plane-wave job (128^3, 2000
          steps) timed whole on the device and on the host cores, with its
          phaser spectrum against theirs; and the large domain (1024 x 1024
          x 512, 200 balls) with float and half storage (--forms 0 skips
          them)
--workload c1 | c5  one of those two worlds as the main line instead
--storage half  E and H stored as IEEE half values with a power-of-two
          exponent per component and x plane, float arithmetic; the
          roofline then counts 2-byte field values (48 B per cell)
--sweep   the batched metasurface unit-cell sweep instead: N periodic unit
          cells (32-96 x 32-96 x 64-256 cells, Lorentz pillar, TFSF pulse,
          32-wavelength transmission plane, 3000 steps each) stepped
          together by batched launches, against the same cells one after
          another; both throughputs, the ratio, and whether every cell's
          result is byte-identical both ways (alis_gb300/bench/serve.c).

Multi-GPU: replicas only (each rank runs its own world on its own GPU);
value is the sum of all ranks' cell updates over the slowest rank's time.
"""
import argparse
import ctypes
import json
import os
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

HALF = 230          # domain half size in nm: 256^3 cells with the CPML
NFREQ = 64
STORAGE = {"float": "float E and H",
           "half": "E and H as IEEE half values times a power of two per component and x plane, float arithmetic"}
TUNE_STEPS = 16     # the engine times its launch shapes over a world's first 10 half steps of each field
C5 = (1024, 1024, 512, 200, 128)   # cells per axis with the CPML, balls, phaser frequencies
C1 = 128                           # cells per axis with the CPML of the vacuum plane-wave workload
C1_STEPS = 2000                    # its whole job
SPECTRUM_TOL = 1e-5                # phaser spectra against the host cores' run, relative to the largest value


def workload_c5(cells):
    return ("large domain %dx%dx%d (%d seeded Drude-Lorentz balls of radius 20-80 cells in an n=1.5 host, CPML 16, "
            "2 pulsed dipoles, %d-f transmission plane)" % C5)


def workload_c1(cells):
    return ("vacuum plane wave %d^3 (periodic x/y, CPML 16 on z, x-polarized 600 nm pulse, "
            "16-wavelength phaser plane)" % C1)


def workload(cells):
    n = round(cells ** (1 / 3))
    return "dispersive scatterer %d^3 (gold Drude+2CP, TFSF, CPML 12, 64-f box phasers)" % n


def env_rank():
    return int(os.environ.get("RANK", 0)), int(os.environ.get("WORLD_SIZE", 1)), int(os.environ.get("LOCAL_RANK", 0))


def build_bench_lib():
    from alis_gb300 import build
    so = build.build_engine()
    src = os.path.join(ROOT, "alis_gb300", "bench", "c2.c")
    out = os.path.join(ROOT, "alis_gb300", "lib", "libalis_c2bench.so")
    if not os.path.exists(out) or os.path.getmtime(out) < max(os.path.getmtime(src), os.path.getmtime(so)):
        cuda = build._cuda_home()
        build._run(["gcc", "-std=gnu99", "-O2", "-fPIC", "-shared", "-ffp-contract=off", "-w",
                    "-I" + os.path.join(ROOT, "include"), src, "-o", out,
                    "-L" + os.path.dirname(so), "-lalis_gb300", "-Wl,-rpath," + os.path.dirname(so),
                    "-L" + os.path.join(cuda, "lib64"), "-lcudart", "-lm"])
    return out


def build_cpu_baseline():
    from alis_gb300 import build
    build.build_oracle()
    out = os.path.join(ROOT, "oracle", "build", "c2_cpu")
    src = os.path.join(ROOT, "oracle", "c2_cpu.c")
    deps = [src, os.path.join(ROOT, "alis_gb300", "bench", "c2.c"), os.path.join(ROOT, "oracle", "build", "liboracle_alis.a")]
    if not os.path.exists(out) or os.path.getmtime(out) < max(os.path.getmtime(d) for d in deps):
        build._run(["gcc", "-std=gnu99", "-O3", "-fopenmp", "-ffp-contract=off", "-w",
                    "-I" + os.path.join(ROOT, "include"), src, "-o", out,
                    os.path.join(ROOT, "oracle", "build", "liboracle_alis.a"), "-lm"])
    return out


def run_cpu(half, steps, warmup):
    """The CPU program on the host cores: `half` the domain half size of the
    scatterer world, or "c1" for the vacuum plane-wave world."""
    exe = build_cpu_baseline()
    env = dict(os.environ)
    env.setdefault("OMP_PROC_BIND", "close")
    cores = os.cpu_count() or 1
    env.setdefault("OMP_NUM_THREADS", str(cores))
    r = subprocess.run([exe, str(half), str(steps), str(warmup)], capture_output=True, text=True, env=env, timeout=1800)
    if r.returncode:
        raise RuntimeError("CPU baseline failed: %s" % r.stderr[-2000:])
    line = [l for l in r.stdout.splitlines() if l.startswith("{")][-1]
    return json.loads(line)


def cpu_split(cpu):
    """Seconds of the timed steps in updateE + updateH and in updatePhaser."""
    return {"update": cpu.get("update_seconds"), "phaser": cpu.get("phaser_seconds")}


class Clocks:
    """nvidia-smi samples of SM clock and throttle reasons while running."""

    FIELDS = "clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown," \
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap"

    def __init__(self, index):
        self.index, self.rows, self.proc = index, [], None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), "--query-gpu=" + self.FIELDS,
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except OSError:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            parts = [p.strip() for p in line.split(",")]
            if len(parts) == 7:
                self.rows.append(parts)

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        if not self.rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        sm = [float(r[0]) for r in self.rows if r[0].replace(".", "").isdigit()]
        mx = [float(r[1]) for r in self.rows if r[1].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[q] for r in self.rows for q in range(4) if r[3 + q].lower() == "active"})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(self.rows)}


def cpu_model():
    """The host CPU's model name (lscpu, else /proc/cpuinfo)."""
    try:
        out = subprocess.run(["lscpu"], capture_output=True, text=True, timeout=10).stdout
        for line in out.splitlines():
            if line.startswith("Model name:"):
                return line.split(":", 1)[1].strip()
    except (OSError, subprocess.SubprocessError):
        pass
    try:
        for line in open("/proc/cpuinfo"):
            if line.lower().startswith(("model name", "cpu model")):
                return line.split(":", 1)[1].strip()
    except OSError:
        pass
    import platform
    return platform.processor() or platform.machine()


def windows(K, ring, target_steps):
    """Back-to-back timed windows of K steps: the fewest whose total is a
    whole number of ring periods and at least target_steps."""
    import math
    r0 = ring // math.gcd(K, ring)
    return r0 * max(1, -(-target_steps // (r0 * K)))


def peaks():
    try:
        return json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json"))), "measured"
    except (OSError, ValueError):
        return {"hbm_gbs": 6800.0}, "fallback"


def traffic_per_launch_pair():
    """DRAM bytes of one E + one H half-step launch from the committed ncu
    summary of this workload."""
    p = os.path.join(ROOT, "profiles", "k_half_step_c2.txt")
    try:
        for line in open(p):
            if line.startswith("dram_bytes_per_launch_pair:"):
                return float(line.split(":")[1])
    except OSError:
        pass
    return None


def reduce_max(x, world):
    if world == 1:
        return x
    import torch
    import torch.distributed as dist
    t = torch.tensor([x], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def barrier(world):
    if world > 1:
        import torch.distributed as dist
        dist.barrier()


def reference_arm(args, rank, world):
    if rank != 0:
        return
    # bounded sample: at most 256 timed steps (about 10 s on 16 cores) and 3
    # warm-up steps of the full world
    cpu = run_cpu(args.half, min(max(args.steps, 1), 256), min(args.warmup, 3))
    rate = cpu["cells"] * cpu["steps"] / cpu["seconds"] / 1e9
    sample = "%d timed steps (after %d warm-up) of the full %d^3-cell world" % (cpu["steps"], min(args.warmup, 3), round(cpu["cells"] ** (1 / 3)))
    model = cpu_model()
    line = {
        "impl": "reference", "metric": "Gcell-updates/s", "value": rate, "unit": "Gcell/s", "n_gpus": args.gpus,
        "steps": cpu["steps"], "warmup": args.warmup, "ms_per_step": 1e3 * cpu["seconds"] / cpu["steps"],
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": workload(cpu["cells"]), "cells": cpu["cells"], "parallelism": "host cores (OpenMP)"},
        "cpu_baseline": {"value": rate, "unit": "Gcell/s", "cores": cpu["threads"], "kind": "port",
                         "cpu_model": model, "split_s": cpu_split(cpu), "sample": sample},
        "e2e": {"value": rate, "unit": "Gcell/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def engine_arm(args, rank, world, local):
    os.environ.setdefault("ALISGPU_DEVICE", str(local))
    # the workload's phasers accumulate with compensated (Kahan) sums
    os.environ.setdefault("ALISGPU_PHASER_KAHAN", "1")
    half_storage = args.storage == "half"
    if half_storage:
        os.environ["ALIS_FIELD_STORAGE"] = "half"
    so = build_bench_lib()
    import alis_gb300
    eng = alis_gb300.library()
    lib = ctypes.CDLL(so)
    lib.c2_build.restype = ctypes.c_long
    lib.c5_build.restype = ctypes.c_long
    lib.c2_result.restype = ctypes.c_double
    lib.c2_step_bytes.restype = ctypes.c_double
    lib.c2_step_bytes_half.restype = ctypes.c_double
    lib.c2_step_h2d_bytes.restype = ctypes.c_double
    lib.c2_result_d2h_bytes.restype = ctypes.c_double
    lib.c2_phaser_face_cells.restype = ctypes.c_double
    lib.c2_nfreq.restype = ctypes.c_int
    eng.alisgpu_stream.restype = ctypes.c_void_p
    eng.alisgpu_launch_count.restype = ctypes.c_ulonglong
    cudart = ctypes.CDLL("libcudart.so.13" if os.path.exists("/usr/local/cuda/lib64/libcudart.so.13") else "libcudart.so")

    lib.c2_flux.restype = ctypes.c_double
    c5, c1 = args.workload == "c5", args.workload == "c1"
    cells = lib.c5_build(*C5) if c5 else lib.c1_build(C1) if c1 else lib.c2_build(args.half, NFREQ)
    # the one-world calls, or the batched form (--batched) of the same steps
    steps_fn = lib.c2_steps_batched if args.batched else lib.c2_steps
    stream = ctypes.c_void_p(eng.alisgpu_stream())
    K, W = args.steps, args.warmup
    ring = int(os.environ.get("ALISGPU_PHASER_RING", "64"))
    # the vacuum plane-wave job is timed whole: one window of its K steps
    R = 1 if c1 else windows(K, ring, args.timed_steps)
    ev = [ctypes.c_void_p() for _ in range(R + 1)]
    for e in ev:
        cudart.cudaEventCreate(ctypes.byref(e))

    # the warm-up covers the launch-shape tuner's first half steps and one
    # phaser ring period (the DFT flush), and reads one result (the face
    # fluxes): every kernel of the timed region has run once before it
    W = max(W, TUNE_STEPS, ring)
    steps_fn(W)
    lib.c2_result()
    eng.alisgpu_synchronize()
    with Clocks(local) as clk:
        # kernel-only throughput: device time of R back-to-back windows of
        # K steps, an event between windows
        barrier(world)
        eng.alisgpu_synchronize()
        l0 = eng.alisgpu_launch_count()
        cudart.cudaEventRecord(ev[0], stream)
        for r in range(R):
            steps_fn(K)
            cudart.cudaEventRecord(ev[r + 1], stream)
        cudart.cudaEventSynchronize(ev[R])
        launches = eng.alisgpu_launch_count() - l0
        win_ms = []
        for r in range(R):
            ms = ctypes.c_float()
            cudart.cudaEventElapsedTime(ctypes.byref(ms), ev[r], ev[r + 1])
            win_ms.append(ms.value)
        dev_s = reduce_max(sum(win_ms) / 1e3, world)
        # the job's spectrum after the timed window (W + K steps)
        spectrum = [lib.c2_flux(f) for f in range(lib.c2_nfreq())] if c1 else None
        # end to end through the public API, host timed: R windows of K
        # steps, each read back as the flux result
        barrier(world)
        eng.alisgpu_synchronize()
        t0 = time.perf_counter()
        for r in range(R):
            steps_fn(K)
            flux = lib.c2_result()
        e2e_s = reduce_max(time.perf_counter() - t0, world)
        # per-kernel device times for the roofline and the shares, over a
        # whole number of ring periods
        eng.alisgpu_profile(1)
        steps_fn(windows(K, ring, 1) * K)
        lib.c2_result()                        # the pass's last ring flush (its face fluxes are not a listed kind)
        kinds = {}
        for kind, name in enumerate(["step_E", "step_H", "ghost", "source", "gather", "flush", "farfield", "step_aux"]):
            t, n = ctypes.c_double(), ctypes.c_ulonglong()
            eng.alisgpu_profile_read(kind, ctypes.byref(t), ctypes.byref(n))
            kinds[name] = (t.value, n.value)
        eng.alisgpu_profile(0)
    clocks = clk.summary()
    if rank != 0:
        return
    step_bytes = lib.c2_step_bytes_half() if half_storage else lib.c2_step_bytes()
    tE, nE = kinds["step_E"]
    tH, nH = kinds["step_H"]
    pair_ms = tE / max(nE, 1) + tH / max(nH, 1)
    achieved = step_bytes / (pair_ms / 1e3) / 1e9
    pk, pk_kind = peaks()
    peak = pk.get("hbm_gbs", 6800.0)
    # ncu traffic of the committed capture, taken on the scatterer world
    traffic = None if half_storage or c1 or c5 else traffic_per_launch_pair()
    total_ms = sum(t for t, _ in kinds.values())
    cpu_baseline = spectrum_check = None
    if c1 and args.cpu_steps > 0:
        # the same job on the host cores: W warm-up and K timed steps, and
        # its spectrum against the engine's at the same step
        cpu = run_cpu("c1", K, W)
        cpu_rate = cpu["cells"] * cpu["steps"] / cpu["seconds"] / 1e9
        cpu_baseline = {"value": cpu_rate, "unit": "Gcell/s", "cores": cpu["threads"], "kind": "port",
                        "cpu_model": cpu_model(), "split_s": cpu_split(cpu),
                        "sample": "the whole %d-step job after %d warm-up steps (oracle restatement, OpenMP)" % (K, W)}
        top = max(abs(v) for v in cpu["flux"]) or 1.0
        diff = max(abs(a - b) for a, b in zip(spectrum, cpu["flux"])) / top
        spectrum_check = {"frequencies": len(spectrum), "steps": W + K, "max_rel_diff": diff,
                          "tolerance": SPECTRUM_TOL, "within": diff <= SPECTRUM_TOL and len(spectrum) == len(cpu["flux"]),
                          "how": "max |engine - host cores| over the phaser frequencies' outgoing flux, over the "
                                 "largest |flux|"}
    elif args.cpu_steps > 0 and not c5:
        cpu = run_cpu(args.half, args.cpu_steps, 1)
        cpu_rate = cpu["cells"] * cpu["steps"] / cpu["seconds"] / 1e9
        cpu_baseline = {"value": cpu_rate, "unit": "Gcell/s", "cores": cpu["threads"], "kind": "port",
                        "cpu_model": cpu_model(), "split_s": cpu_split(cpu),
                        "sample": "%d steps of the full world after 1 warm-up step (oracle restatement, OpenMP)" % cpu["steps"]}
    value = cells * K * R * world / dev_s / 1e9
    win_sorted = sorted(win_ms)
    line = {
        "metric": "Gcell-updates/s", "value": value, "unit": "Gcell/s", "n_gpus": world, "steps": K, "warmup": W,
        "ms_per_step": dev_s * 1e3 / (K * R), "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32", "data": "synthetic",
        "config": {"workload": workload_c5(cells) if c5 else workload_c1(cells) if c1 else workload(cells), "cells": cells,
                   "parallelism": "replicas" if world > 1 else "single GPU",
                   "storage": STORAGE[args.storage],
                   "l2": "inputs larger than L2 (%.0f MB of fields per step)" % (step_bytes / 1e6),
                   "phaser": "%d frequencies, %s, time-blocked ring of %s steps" % (
                       lib.c2_nfreq(),
                       "Kahan-compensated" if os.environ.get("ALISGPU_PHASER_KAHAN") == "1" else "plain float sums",
                       os.environ.get("ALISGPU_PHASER_RING", "64")),
                   "path": "batched launches (alisBatchBegin/End)" if args.batched else "one launch per half step",
                   "timing": ("the whole %d-step job as one window after %d warm-up steps; value from its device "
                              "time" % (K, W)) if c1 else
                             "%d back-to-back windows of %d steps (%d steps, a whole number of %d-step phaser "
                             "ring periods, so the DFT flush is charged at its own rate); value from their total "
                             "device time" % (R, K, R * K, ring),
                   "window_ms": {"median": win_sorted[len(win_sorted) // 2], "min": win_sorted[0],
                                 "max": win_sorted[-1]}},
        "e2e": {"value": cells * K * R * world / e2e_s / 1e9, "unit": "Gcell/s",
                "h2d_bytes_per_step": lib.c2_step_h2d_bytes(),
                "d2h_bytes_per_step": lib.c2_result_d2h_bytes() / K},
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                     "frac_nominal": achieved / 8000.0,
                     "peak_source": pk_kind, "traffic": traffic,
                     "kernel": "k_half_step (E + H launches, mean per launch pair)",
                     "algorithmic_bytes_per_step": step_bytes, "launch_pair_ms": pair_ms},
        "kernel_share": {k: round(t / total_ms, 4) for k, (t, n) in kinds.items() if n},
        "phaser": phaser_rate(lib, kinds, K, windows(K, ring, 1) * K),
        "cpu_baseline": cpu_baseline,
        "gpu_launches": int(launches),
        "clocks": clocks,
        "result_flux": flux,
    }
    if spectrum_check:
        line["spectrum_vs_cpu"] = spectrum_check
    if args.forms and not c5 and not c1:
        # the batched and served forms, each against its per-request path,
        # the same workload with half field storage, the vacuum plane-wave
        # job and the large domain
        line["forms"] = {"sweep": sweep_form(args.forms, threads=8), "served": served_form(),
                         "half_storage": half_form(args, line), "plane_wave": plane_wave_form(),
                         "large_domain": large_domain_form()}
    print(json.dumps(line), flush=True)


def phaser_rate(lib, kinds, K, profiled_steps):
    """The phaser DFT against the reference formulation, reported apart
    from the half-step roofline: per face cell per step the reference reads
    24 B of fields and read-modify-writes 4 complex accumulators per
    frequency, 64 B (128 B with the Kahan compensation terms); effective
    GB/s = those bytes / the gather and flush kernels' time per step (the
    engine's time-blocked DFT moves far fewer)."""
    cells, nf = lib.c2_phaser_face_cells(), lib.c2_nfreq()
    kahan = os.environ.get("ALISGPU_PHASER_KAHAN") == "1"
    ref = cells * (24 + (128 if kahan else 64) * nf)
    ms = (kinds["gather"][0] + kinds["flush"][0]) / max(profiled_steps, 1)
    return {"face_cells": cells, "frequencies": nf, "reference_bytes_per_step": ref,
            "ms_per_step": ms, "effective_GBps": ref / (ms / 1e3) / 1e9 if ms > 0 else None}


def half_form(args, line):
    """The workload with E and H stored as half values (--storage half, its
    own process): throughput, the roofline of its half steps over its own
    algorithmic bytes, and its speed against the float line."""
    h, err = bench_line(["--storage", "half", "--steps", str(args.steps), "--warmup", str(args.warmup),
                         "--cpu-steps", "0", "--forms", "0", "--half", str(args.half),
                         "--timed-steps", str(args.timed_steps)])
    if err:
        return err
    return {"storage": STORAGE["half"], "value": h["value"], "unit": h["unit"], "ms_per_step": h["ms_per_step"],
            "e2e": h["e2e"]["value"], "speedup": h["value"] / line["value"],
            "roofline": {k: h["roofline"][k] for k in ("achieved", "peak", "frac", "frac_nominal",
                                                        "algorithmic_bytes_per_step", "launch_pair_ms")},
            "clocks": h["clocks"], "result_flux": h["result_flux"]}


def bench_line(extra):
    """One run of this bench in its own process (its own world and
    device memory, on this rank's device, as a single process outside any
    torchrun group): its JSON line, or the error."""
    env = {k: v for k, v in os.environ.items()
           if k not in ("RANK", "WORLD_SIZE", "LOCAL_RANK", "LOCAL_WORLD_SIZE", "GROUP_RANK", "MASTER_ADDR", "MASTER_PORT")}
    r = subprocess.run([sys.executable, os.path.abspath(__file__)] + extra, capture_output=True, text=True,
                       timeout=1800, env=env)
    if r.returncode:
        return None, {"error": (r.stdout + r.stderr)[-500:]}
    return json.loads([l for l in r.stdout.splitlines() if l.startswith("{")][-1]), None


def plane_wave_form():
    """The vacuum plane-wave job (128^3, 2000 steps) timed whole on the
    device and on the host cores, and its phaser spectrum against the host
    cores' at the same step."""
    h, err = bench_line(["--workload", "c1", "--steps", str(C1_STEPS), "--warmup", str(TUNE_STEPS),
                         "--cpu-steps", str(C1_STEPS), "--forms", "0"])
    if err:
        return err
    return {"workload": h["config"]["workload"], "steps": h["steps"], "value": h["value"], "unit": h["unit"],
            "job_ms": h["ms_per_step"] * h["steps"], "e2e": h["e2e"]["value"],
            "roofline": {k: h["roofline"][k] for k in ("achieved", "peak", "frac", "algorithmic_bytes_per_step",
                                                        "launch_pair_ms")},
            "cpu_baseline": h["cpu_baseline"], "spectrum_vs_cpu": h.get("spectrum_vs_cpu"), "clocks": h["clocks"]}


def large_domain_form():
    """The large domain (1024 x 1024 x 512, 200 balls) with float and with
    half field storage: 256 timed steps each (four 64-step windows)."""
    out = {}
    for storage in ("float", "half"):
        h, err = bench_line(["--workload", "c5", "--storage", storage, "--steps", "64", "--warmup", str(TUNE_STEPS),
                             "--timed-steps", "256", "--cpu-steps", "0", "--forms", "0"])
        out[storage] = err or {
            "value": h["value"], "unit": h["unit"], "ms_per_step": h["ms_per_step"], "e2e": h["e2e"]["value"],
            "roofline": {k: h["roofline"][k] for k in ("achieved", "peak", "frac", "algorithmic_bytes_per_step",
                                                        "launch_pair_ms")},
            "clocks": h["clocks"]}
        if not err:
            out["workload"] = h["config"]["workload"]
    return out


def serve_exe():
    from alis_gb300 import build
    build.build_engine()
    return build.link_program(os.path.join(ROOT, "alis_gb300", "bench", "serve.c"),
                              os.path.join(ROOT, "alis_gb300", "lib", "serve"), "engine", extra=["-lm"])


def run_serve(exe, args, env):
    """One run of the request loop: per-request results and its summary."""
    r = subprocess.run([exe] + [str(a) for a in args], capture_output=True, text=True, env=env, timeout=3600)
    if r.returncode:
        raise RuntimeError("serve %s failed: %s" % (args[0], r.stderr[-2000:]))
    res = {l.split()[1]: l.split()[6] for l in r.stdout.splitlines() if l.startswith("R ")}
    return res, json.loads([l for l in r.stdout.splitlines() if l.startswith("{")][-1])


def sweep_form(n, steps=0, threads=8):
    """The batched metasurface sweep of n unit cells against the same cells
    one after another, and whether every cell's result is the same bytes."""
    exe = serve_exe()
    env = dict(os.environ, SERVE_THREADS=str(threads))
    if steps:
        env["SERVE_STEPS"] = str(steps)
    batched, b = run_serve(exe, ["batched", n, 2000, 7, "sweep", n, 200], env)
    seq, q = run_serve(exe, ["sequential", n, 2000, 7, "sweep"], env)
    return {"workload": "metasurface unit-cell sweep: %d periodic cells 32-96 x 32-96 x 64-256, TiO2-like Lorentz "
                        "pillar, TFSF pulse, 32-wavelength transmission plane, %d steps each" % (n, steps or 3000),
            "batched": {"value": b["gcell_per_s"], "unit": "Gcell/s", "wall_s": b["wall_s"],
                        "how": "alisBatchBegin/End, %d host threads recording" % threads},
            "per_instance": {"value": q["gcell_per_s"], "unit": "Gcell/s", "wall_s": q["wall_s"],
                             "how": "the same cells one after another through the same API"},
            "ratio": b["gcell_per_s"] / q["gcell_per_s"],
            "identical_results": batched == seq and len(batched) == n}


def served_form(n=48):
    """The served request stream in miniature: Poisson arrivals of mixed
    small requests, admitted by footprint, against the same requests one
    after another; latency percentiles of the served run."""
    exe = serve_exe()
    env = dict(os.environ)
    served, s = run_serve(exe, ["served", n, 200, 42, "small", 16], env)
    seq, q = run_serve(exe, ["sequential", n, 200, 42, "small"], env)
    return {"workload": "%d mixed small requests (vacuum and dielectric, Drude bowtie, photonic-crystal k-point "
                        "runs; 28^3-48^3 cells, 120-240 steps), Poisson arrivals offered at 200/s" % n,
            "served": {"value": s["gcell_per_s"], "unit": "Gcell/s", "latency_ms": s["latency_ms"],
                       "slots": 16, "host_threads": s["threads"]},
            "sequential": {"value": q["gcell_per_s"], "unit": "Gcell/s"},
            "ratio": s["gcell_per_s"] / q["gcell_per_s"],
            "identical_results": served == seq and len(served) == n}


def sweep_arm(args):
    """The batched unit-cell sweep against the per-instance path, one line."""
    f = sweep_form(args.sweep, args.sweep_steps)
    line = {"metric": "sweep Gcell-updates/s", "value": f["batched"]["value"], "unit": "Gcell/s", "n_gpus": 1,
            "higher_is_better": True, "dtype": "f32", "data": "synthetic", "config": {"workload": f["workload"]},
            "per_instance": f["per_instance"], "ratio": f["ratio"], "identical_results": f["identical_results"]}
    print(json.dumps(line), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=1024)
    ap.add_argument("--warmup", type=int, default=64)
    ap.add_argument("--impl", default="engine", choices=["engine", "reference"])
    ap.add_argument("--cpu-steps", type=int, default=256, help="steps of the CPU baseline sample, about 10 s on 16 cores (0: skip it)")
    ap.add_argument("--half", type=int, default=HALF, help="domain half size in nm (230: the 256^3 workload)")
    ap.add_argument("--timed-steps", type=int, default=3000,
                    help="least number of steps over all timed windows (about 1 s on the 256^3 workload)")
    ap.add_argument("--batched", action="store_true",
                    help="step the world through the batched launches (alisBatchBegin/End) instead")
    ap.add_argument("--sweep", type=int, default=0, metavar="N",
                    help="run the batched unit-cell sweep of N cells instead (512: the full sweep)")
    ap.add_argument("--sweep-steps", type=int, default=0, help="steps per unit cell (default 3000)")
    ap.add_argument("--workload", default="c2", choices=["c1", "c2", "c5"],
                    help="c2: the dispersive scatterer (256^3, the headline); c1: the vacuum plane wave (128^3, "
                         "timed as one window of --steps, its spectrum against the host cores' run); c5: the "
                         "large-domain precision workload (1024 x 1024 x 512, 200 balls), for its float and half "
                         "storage throughput")
    ap.add_argument("--storage", default="float", choices=sorted(STORAGE),
                    help="field storage of the world: float, or half values with a power-of-two exponent per "
                         "component and x plane (alisgpu_world_set_storage)")
    ap.add_argument("--forms", type=int, default=64, metavar="N",
                    help="after the main line's timing, the batched sweep of N unit cells and the served stream, "
                         "each against its per-request path, the half-storage run, the vacuum plane-wave job and "
                         "the large domain, as the line's 'forms' (0: skip)")
    args = ap.parse_args()
    if args.sweep:
        sweep_arm(args)
        return
    if args.warmup < 3:
        args.warmup = 3
    rank, world, local = env_rank()
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("gloo")
    if args.impl == "reference":
        reference_arm(args, rank, world)
    else:
        engine_arm(args, rank, world, local)
    if world > 1:
        import torch.distributed as dist
        dist.barrier()
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
