"""The oracle restatement against the reference itself.

Every parity scene is run through the oracle (engine host setup + CPU
restatement of the stepping loops) and each dumped array -- eps^-1 maps,
fill factors, ADE coefficients, fields, ADE currents, phaser faces,
fluxes, far-field values -- is compared with the golden fixture made by
running the same scene through the reference build
(tests/golden/make_golden.py).  On the x86-64 host that generated the
fixture the match is byte for byte; on another host ISA the C library's
float transcendentals may round differently in the last bit, and the
check falls back to the recorded sums at 1e-5.
"""
import json
import os
import platform

import numpy as np
import pytest

import scenes

GOLDEN = json.load(open(os.path.join(os.path.dirname(__file__), "golden", "scenes.json")))
EXACT_HOST = platform.machine() == "x86_64"


@pytest.mark.parametrize("scene,scale,steps", scenes.PIN_CASES, ids=scenes.PIN_IDS)
def test_oracle_matches_reference(scene, scale, steps):
    dump = scenes.run("oracle", scene, scale, steps)
    inexact = scenes.check_against_golden(dump, GOLDEN["%s/%d/%d" % (scene, scale, steps)])
    if EXACT_HOST:
        assert not inexact, "not bit-identical: %s" % inexact[:10]


def test_reference_build_agrees_with_fixture():
    """Where the reference checkout exists, its build still reproduces the
    committed fixture (guards the fixture itself)."""
    if scenes.binary("reference") is None:
        pytest.skip("reference sources not present on this machine")
    scene, scale, steps = scenes.CASES[1]
    dump = scenes.run("reference", scene, scale, steps)
    inexact = scenes.check_against_golden(dump, GOLDEN["%s/%d/%d" % (scene, scale, steps)])
    if EXACT_HOST:
        assert not inexact


def test_planted_mistake_is_caught():
    """A one-ulp change in one oracle array must fail the golden check."""
    scene, scale, steps = scenes.CASES[0]
    dump = scenes.run("oracle", scene, scale, steps)
    name = "W.E0.x"
    a = dump[name].copy()
    flat = a.reshape(-1)
    idx = int(np.argmax(np.abs(flat)))
    flat[idx] = np.nextafter(flat[idx], np.float32(np.inf))
    dump[name] = a
    gold = GOLDEN["%s/%d/%d" % (scene, scale, steps)]
    assert scenes.summary(dump[name])["sha256"] != gold[name]["sha256"]
