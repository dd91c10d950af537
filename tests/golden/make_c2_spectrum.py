"""Generate tests/golden/c2_spectrum.json: the phaser spectrum of the
dispersive-scatterer benchmark world (alis_gb300/bench/c2.c, 256^3 cells,
64 frequencies) after 4000 steps, from the FP32 oracle and from the
oracle's FP64 build (oracle/fp64.h).  test_fp64_error holds the engine's
full-size spectrum, in both phaser modes, to the FP64 one.

    python tests/golden/make_c2_spectrum.py [steps]

About 20 minutes on 8 host cores.
"""
import json
import os
import platform
import subprocess
import sys
import tempfile

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)
from alis_gb300 import build  # noqa: E402

DRIVER = os.path.join(ROOT, "tests", "drivers", "c2_spectrum.c")
BIN = os.path.join(ROOT, "tests", "drivers", "bin")
OUT = os.path.join(os.path.dirname(os.path.abspath(__file__)), "c2_spectrum.json")


def spectrum(against, half, steps):
    if against == "oracle64":
        build.build_oracle(fp64=True)
    elif against == "oracle":
        build.build_oracle()
    else:
        build.build_engine()
    exe = build.link_program(DRIVER, os.path.join(BIN, "c2_spectrum_" + against), against)
    with tempfile.TemporaryDirectory() as d:
        r = subprocess.run([exe, str(half), str(steps)], cwd=d, capture_output=True, text=True, check=True)
    return json.loads(r.stdout.strip().splitlines()[-1])


def main():
    steps = int(sys.argv[1]) if len(sys.argv) > 1 else 4000
    out = {"world": "alis_gb300/bench/c2.c, half 230 (256^3 cells), 64 frequencies",
           "steps": steps, "host": platform.machine(), "threads": os.cpu_count()}
    for against in ("oracle", "oracle64"):
        s = spectrum(against, 230, steps)
        out[against] = {k: s[k] for k in ("f", "A", "flux")}
        out["cells"] = s["cells"]
    with open(OUT, "w") as f:
        json.dump(out, f, indent=1)
    print(OUT)


if __name__ == "__main__":
    main()
