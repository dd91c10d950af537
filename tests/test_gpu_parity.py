"""GPU engine against the oracle and the golden fixtures.

The engine (CUDA kernels built for sm_103a, reached through the ALiS C
API) runs every parity scene; the oracle runs the same scene on the
host cores of the same machine.  Both use the same C library for the
waveforms and phase factors, so every dumped array must be identical
byte for byte: fields, CPML-affected cells, ADE currents, TFSF boxes,
Bloch/HBC/symmetry ghosts, phaser accumulators and fluxes.  Far-field
values are FP64 sums on the GPU and are compared at 1e-5 relative to
the oracle's FP64 restatement.
"""
import json
import os

import numpy as np
import pytest

import scenes

GOLDEN = json.load(open(os.path.join(os.path.dirname(__file__), "golden", "scenes.json")))
FAR = ("F.ffP", "F.ffS")


@pytest.mark.gpu
@pytest.mark.parametrize("scene,scale,steps", scenes.CASES, ids=scenes.IDS)
def test_engine_bit_identical_to_oracle(scene, scale, steps):
    gpu = scenes.run("engine", scene, scale, steps)
    cpu = scenes.run("oracle", scene, scale, steps)
    near = {k: v for k, v in gpu.items() if not k.startswith(FAR)}
    bad = scenes.compare_exact(near, {k: v for k, v in cpu.items() if not k.startswith(FAR)})
    assert not bad, "differs from the oracle: %s" % bad[:10]
    far = [k for k in gpu if k.startswith(FAR)]
    if far:
        # 1e-5 relative to the value, or to 1e-6 of the scene's largest
        # far-field sample for directions whose exact value is near zero
        wide = scenes.run("oracle", scene, scale, steps, env={"ALIS_ORACLE_FF64": "1"})
        top = max(abs(complex(wide[k].reshape(-1)[0])) for k in far)
        for k in far:
            x, y = complex(gpu[k].reshape(-1)[0]), complex(wide[k].reshape(-1)[0])
            assert abs(x - y) <= 1e-5 * max(abs(y), 1e-6 * top, 1e-30), (k, x, y)


@pytest.mark.gpu
@pytest.mark.parametrize("scene,scale,steps", scenes.CASES[:2], ids=scenes.IDS[:2])
def test_engine_matches_reference_fixture(scene, scale, steps):
    gpu = scenes.run("engine", scene, scale, steps)
    gold = GOLDEN["%s/%d/%d" % (scene, scale, steps)]
    exact = 0
    for name, g in gold.items():
        if name.startswith(FAR):
            continue
        s = scenes.summary(gpu[name])
        if s["sha256"] == g["sha256"]:
            exact += 1
            continue
        scale_ = max(g["l1"], 1e-30)
        assert abs(s["l1"] - g["l1"]) <= 1e-5 * scale_, (name, s["l1"], g["l1"])
    assert exact > 0


def _rel_l1(a, b, keys):
    num = sum(np.abs(a[k].astype(np.complex128) - b[k].astype(np.complex128)).sum() for k in keys)
    den = sum(np.abs(b[k].astype(np.complex128)).sum() for k in keys)
    return num / den


@pytest.mark.gpu
@pytest.mark.parametrize("scene,scale,steps", [("c1", 1, 600), ("c2", 1, 200)], ids=["c1-600", "c2-200"])
def test_kahan_phasers_against_fp64_accumulation(scene, scale, steps):
    """Compensated phaser accumulation (ALISGPU_PHASER_KAHAN=1) against the
    oracle's FP64 accumulation of the same float fields and phase factors:
    at most 1e-6 relative (L1 over every face array), never further than
    the reference's plain float sums; fluxes within 1e-5 relative."""
    gpu = scenes.run("engine", scene, scale, steps, env={"ALISGPU_PHASER_KAHAN": "1"})
    plain = scenes.run("oracle", scene, scale, steps)
    wide = scenes.run("oracle", scene, scale, steps, env={"ALIS_ORACLE_DFT64": "1"})
    faces = [k for k in wide if k.startswith("P.") and k.count(".") == 3 and k.split(".")[3][0] in "EH"]
    assert faces
    err_k, err_p = _rel_l1(gpu, wide, faces), _rel_l1(plain, wide, faces)
    print("phaser error vs FP64: kahan %.3e plain %.3e" % (err_k, err_p))
    assert err_k <= 1e-6 and err_k <= err_p, (err_k, err_p)
    for k in wide:
        if k.endswith(".flux"):
            x, y = float(gpu[k].reshape(-1)[0]), float(wide[k].reshape(-1)[0])
            assert abs(x - y) <= 1e-5 * max(abs(y), 1e-30), (k, x, y)


# every TFSF scene with its auxiliary column inside the world's launches
# (the form large worlds and served worlds take)
ATTACH = [c for c in scenes.CASES if (c[0], c[1]) in (("c1", 1), ("c2", 1), ("bloch", 1), ("beamtf", 1), ("unitcell", 1))]


@pytest.mark.gpu
@pytest.mark.parametrize("scene,scale,steps", ATTACH, ids=["%s-x%d" % (c[0], c[1]) for c in ATTACH])
def test_attached_auxiliary_column_bit_identical(scene, scale, steps):
    gpu = scenes.run("engine", scene, scale, steps, env={"ALISGPU_AUX_ATTACH": "2"})
    cpu = scenes.run("oracle", scene, scale, steps)
    near = {k: v for k, v in gpu.items() if not k.startswith("F.")}
    bad = scenes.compare_exact(near, {k: v for k, v in cpu.items() if not k.startswith("F.")})
    assert not bad, "differs from the oracle: %s" % bad[:10]
