"""Build and run the parity scenes (tests/drivers/scenes.c) against the
GPU engine, the CPU oracle or the reference library, and compare dumps."""
import hashlib
import os
import subprocess
import tempfile

import numpy as np

from alis_dump import read_dump

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
DRIVER = os.path.join(ROOT, "tests", "drivers", "scenes.c")
BIN = os.path.join(ROOT, "tests", "drivers", "bin")

# (scene, scale, steps) run by the parity tests; small enough that the
# oracle finishes each in about a second
CASES = [
    ("c1", 1, 80),
    ("c2", 1, 80),
    ("dipole", 1, 80),
    ("bloch", 1, 80),
    ("sym", 1, 80),
    ("hbc", 1, 60),
    ("multi", 1, 80),
    # rows longer than one warp's 128 cells, with a ragged float4 at the end
    ("c2", 2, 30),
    ("c1", 3, 40),
    # the vacuum plane-wave workload at its lateral size (128 x 128 cells,
    # periodic), a longer run
    ("c1", 4, 400),
    ("nug", 1, 80),
    ("beam", 1, 80),
    ("beamtf", 1, 80),
    ("shg", 1, 80),
    # the other workloads in miniature: many dispersive objects (per-tile
    # object lists), a periodic unit cell, a Drude bowtie with symmetry
    # planes, a graded grid and edge-rule filling
    ("spheres", 1, 80),
    ("unitcell", 1, 120),
    ("bowtie", 1, 80),
    # the voxelizer: every shape of the object API with 4^3 supersampling,
    # point samples and the edge rule; a height map filled on the host
    ("shapes", 1, 40),
    ("shapespt", 1, 40),
    ("shapesedge", 1, 40),
    ("contour", 1, 40),
    # a PEC mirror under silver and a lossy (nk) film, symmetry planes,
    # a single-wavelength phaser; an anisotropic Drude-Lorentz ball with
    # the far-field intensities and ring fluxes; a dipole array whose
    # phasers replicate over three periods, with the far field's lattice
    # factor; the far-field images and angular cuts
    ("pec", 1, 120),
    ("aniso", 1, 120),
    ("lattice", 1, 120),
    ("farmaps", 1, 120),
    # a 128^3 window of the large-domain precision world: its seeded
    # Drude-Lorentz balls clipped to the window, 16-cell CPML, pulsed dipoles
    ("c5", 2, 80),
]
IDS = ["%s-x%d" % (c[0], c[1]) for c in CASES]

# every parity case is also pinned against the reference on the CPU
# (tests/test_oracle_pin.py)
PIN_CASES = list(CASES)
PIN_IDS = ["%s-x%d" % (c[0], c[1]) for c in PIN_CASES]


def binary(against):
    from alis_gb300 import build
    out = os.path.join(BIN, "scenes_" + against)
    if against == "engine":
        build.build_engine()
    elif against == "oracle":
        build.build_oracle()
    elif against == "oracle64":
        build.build_oracle(fp64=True)
    elif against == "reference":
        if build.build_reference() is None:
            return None
    deps = [DRIVER, os.path.join(ROOT, "tests", "drivers", "dump.h")]
    if against == "oracle64":
        deps.append(build.FP64_HEADER)
    lib = {"engine": os.path.join(build.LIB, "libalis_gb300.so"),
           "oracle": os.path.join(build.ORACLE_BUILD, "liboracle_alis.a"),
           "oracle64": os.path.join(build.ORACLE_BUILD, "liboracle_alis64.a"),
           "reference": os.path.join(build.ORACLE, "_ref", "libalis_ref.a")}[against]
    if os.path.exists(lib):
        deps.append(lib)
    if not os.path.exists(out) or os.path.getmtime(out) < max(os.path.getmtime(d) for d in deps):
        build.link_program(DRIVER, out, against)
    return out


def run(against, scene, scale, steps, env=None):
    exe = binary(against)
    if exe is None:
        return None
    e = dict(os.environ)
    if against == "reference":
        e["OMP_NUM_THREADS"] = "1"   # reductions in the order of a sequential run
    e.update(env or {})
    with tempfile.TemporaryDirectory() as d:
        out = os.path.join(d, "dump.bin")
        r = subprocess.run([exe, scene, out, str(scale), str(steps)], cwd=d, env=e,
                            capture_output=True, text=True, timeout=900)
        if r.returncode:
            raise RuntimeError("%s %s failed (%d):\n%s%s" % (against, scene, r.returncode, r.stdout[-2000:], r.stderr[-2000:]))
        return read_dump(out)


_CACHE = {}


def run_cached(against, scene, scale, steps):
    """run() of a case without extra environment, kept for the session."""
    key = (against, scene, scale, steps)
    if key not in _CACHE:
        _CACHE[key] = run(against, scene, scale, steps)
    return _CACHE[key]


def digest(arr):
    return hashlib.sha256(np.ascontiguousarray(arr).tobytes()).hexdigest()


def summary(arr):
    a = arr.astype(np.complex128)
    return {
        "shape": list(arr.shape),
        "dtype": str(arr.dtype),
        "sha256": digest(arr),
        "sum": [float(a.sum().real), float(a.sum().imag)],
        "l1": float(np.abs(a).sum()),
        "max": float(np.abs(a).max()) if a.size else 0.0,
    }


def compare_exact(a, b):
    """Names whose bytes differ between two dumps (and missing names)."""
    bad = sorted(set(a) ^ set(b))
    for k in set(a) & set(b):
        if a[k].shape != b[k].shape or a[k].dtype != b[k].dtype or \
                not np.array_equal(a[k].view(np.uint8), b[k].view(np.uint8)):
            bad.append(k)
    return sorted(bad)


def max_rel(a, b):
    """Largest |a-b| / max|b| over arrays (a dict of name -> value)."""
    out = {}
    for k in set(a) & set(b):
        x, y = a[k].astype(np.complex128), b[k].astype(np.complex128)
        scale = np.abs(y).max()
        out[k] = float(np.abs(x - y).max() / scale) if scale > 0 else float(np.abs(x).max())
    return out


def check_against_golden(dump, gold):
    """Names of the arrays of a dump that are not byte-identical to the
    golden digests (the reference's output); those must still agree in L1
    and in sum within 1e-5.  Shapes, types and the set of names must be
    the same."""
    assert sorted(dump) == sorted(gold), sorted(set(dump) ^ set(gold))
    inexact = []
    for name, g in gold.items():
        s = summary(dump[name])
        assert s["shape"] == g["shape"] and s["dtype"] == g["dtype"], name
        if s["sha256"] == g["sha256"]:
            continue
        inexact.append(name)
        scale = max(g["l1"], 1e-30)
        assert abs(s["l1"] - g["l1"]) <= 1e-5 * scale, (name, s["l1"], g["l1"])
        assert abs(complex(*s["sum"]) - complex(*g["sum"])) <= 1e-5 * scale, name
    return inexact
