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
# far-field outputs: FP64 sums on the GPU, compared with the oracle's FP64
# restatement (amplitudes F.ff* / FL.ff*, intensities and ring fluxes FA.*,
# farFieldProfile images FP.*, farFieldTheta / farFieldPhi rows FT.*)
FAR = ("F.", "FA.", "FL.ff", "FP.", "FT.")


def _linear(key, a):
    """A log10 image back to intensities (log10 of 0 is -inf: 0)."""
    a = a.astype(np.complex128).reshape(-1)
    if key.startswith("FP.") and "Log" in key and not key.endswith(".max"):
        re = a.real
        a = np.where(np.isfinite(re), np.power(10.0, np.where(np.isfinite(re), re, 0.0)), 0.0).astype(np.complex128)
    return a


def check_far_field(gpu, wide):
    """Every far-field output within 1e-5 relative of the FP64 oracle, or of
    1e-6 x the largest sample of its group for values whose exact value is
    near zero.  A group is one image or one cut; the scalars of a scene
    form one group.  The cuts are printed with 6 significant digits
    (writeRow's %g), so they may differ by one unit in the last digit
    more: 2.1e-5."""
    far = sorted(k for k in gpu if k.startswith(FAR))
    assert sorted(k for k in wide if k.startswith(FAR)) == far
    scalars = [k for k in far if gpu[k].size == 1]
    top_scalar = max((abs(_linear(k, wide[k])[0]) for k in scalars), default=0.0)
    for k in far:
        x, y = _linear(k, gpu[k]), _linear(k, wide[k])
        finite = np.isfinite(y)
        assert np.array_equal(np.isfinite(x), finite), k
        top = top_scalar if y.size == 1 else float(np.abs(y[finite]).max(initial=0.0))
        rel = 2.1e-5 if k.startswith("FT.") else 1e-5
        tol = rel * np.maximum(np.maximum(np.abs(y[finite]), 1e-6 * top), 1e-30)
        err = np.abs(x[finite] - y[finite])
        assert (err <= tol).all(), (k, float((err / tol).max()))


@pytest.mark.gpu
@pytest.mark.parametrize("scene,scale,steps", scenes.CASES, ids=scenes.IDS)
def test_engine_bit_identical_to_oracle(scene, scale, steps):
    gpu = scenes.run("engine", scene, scale, steps)
    cpu = scenes.run("oracle", scene, scale, steps)
    near = {k: v for k, v in gpu.items() if not k.startswith(FAR)}
    bad = scenes.compare_exact(near, {k: v for k, v in cpu.items() if not k.startswith(FAR)})
    assert not bad, "differs from the oracle: %s" % bad[:10]
    if any(k.startswith(FAR) for k in gpu):
        check_far_field(gpu, scenes.run("oracle", scene, scale, steps, env={"ALIS_ORACLE_FF64": "1"}))


@pytest.mark.gpu
@pytest.mark.parametrize("scene,scale,steps", scenes.CASES, ids=scenes.IDS)
def test_engine_matches_reference_fixture(scene, scale, steps):
    """The engine against the reference's own output, recorded as golden
    digests on an x86-64 host: every near-field array identical byte for
    byte or, where the host C library's float transcendentals (waveforms,
    phase factors: computed on this host) round differently in the last
    bit, within 1e-5 in L1 and in sum.  The byte-identical share is
    printed; the eps^-1 maps, which no transcendental function touches,
    must all be identical."""
    gpu = scenes.run("engine", scene, scale, steps)
    gold = {k: v for k, v in GOLDEN["%s/%d/%d" % (scene, scale, steps)].items() if not k.startswith(FAR)}
    near = {k: v for k, v in gpu.items() if not k.startswith(FAR)}
    inexact = scenes.check_against_golden(near, gold)
    print("%s: %d of %d arrays byte-identical to the reference" % (scene, len(gold) - len(inexact), len(gold)))
    static = [k for k in inexact if k.split(".")[1].startswith("CE")]
    assert not static, static


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


# the launch shapes of the large-world half step (ALISGPU_STEP_SHAPE): one
# plane per block of 32 x 2, 32 x 4 or 32 x 8 threads.  Scenes with CPML on
# every face, TFSF boxes, many dispersive objects, complex fields, a graded
# grid, PEC walls, rows longer than one warp.
SHAPE_SCENES = [c for c in scenes.CASES if (c[0], c[1]) in
                (("c2", 1), ("c2", 2), ("bloch", 1), ("spheres", 1), ("unitcell", 1), ("nug", 1), ("pec", 1), ("multi", 1))]


@pytest.mark.gpu
@pytest.mark.parametrize("shape", [0, 1, 2])
@pytest.mark.parametrize("scene,scale,steps", SHAPE_SCENES, ids=["%s-x%d" % (c[0], c[1]) for c in SHAPE_SCENES])
def test_every_launch_shape_bit_identical(scene, scale, steps, shape):
    gpu = scenes.run("engine", scene, scale, steps, env={"ALISGPU_STEP_SHAPE": str(shape)})
    cpu = scenes.run_cached("oracle", scene, scale, steps)
    near = {k: v for k, v in gpu.items() if not k.startswith(FAR)}
    bad = scenes.compare_exact(near, {k: v for k, v in cpu.items() if not k.startswith(FAR)})
    assert not bad, "shape %d differs from the oracle: %s" % (shape, bad[:10])
