"""Generate tests/golden/scenes.json from the reference itself.

Builds the ALiS reference library from its own sources (oracle/build_ref.sh,
which locates the read-only reference checkout: $ALIS_REFERENCE or the
build container's checkout), links tests/drivers/scenes.c against it, runs every
parity case with one OpenMP thread, and records per dumped array its
shape, dtype, SHA-256 of the bytes and a few sums.  The fixture pins the
oracle restatement (tests/test_oracle_pin.py) and the GPU engine
(tests/test_gpu_parity.py).

    python tests/golden/make_golden.py
"""
import json
import os
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(HERE))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

import scenes  # noqa: E402


def main():
    out = {}
    for scene, scale, steps in scenes.PIN_CASES:
        d = scenes.run("reference", scene, scale, steps)
        if d is None:
            sys.exit("reference sources not available")
        out["%s/%d/%d" % (scene, scale, steps)] = {k: scenes.summary(v) for k, v in sorted(d.items())}
        print(scene, len(d), "arrays")
    with open(os.path.join(HERE, "scenes.json"), "w") as f:
        json.dump(out, f, indent=0, sort_keys=True)


if __name__ == "__main__":
    main()
