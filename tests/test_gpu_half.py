"""FP16 field storage against the oracle's restatement of the same form.

With ALIS_FIELD_STORAGE=half the engine holds the E and H components of
every world the user steps as IEEE half values times a power of two per
component and x plane (alisgpu_world_set_storage); with
ALIS_ORACLE_FP16_STORAGE=1 the oracle rounds its float arrays to the same
values at the same points: after each half step's cell updates with the
exponent taken from the previous step's plane maxima, and after the source
patches.  Arithmetic stays float in both, so every near-field array must
be identical byte for byte; far-field values are FP64 sums, held to 1e-5
of the oracle's FP64 restatement over the same rounded phasers.  The
observers (Poynting planes, probes, slice DFTs, object absorption) read
the half values on the device.  Complex (Bloch) and coupled (chi2)
worlds refuse half storage.
"""
import re

import numpy as np
import pytest

import scenes
from test_gpu_parity import FAR, check_far_field

ENGINE = {"ALIS_FIELD_STORAGE": "half"}
ORACLE = {"ALIS_ORACLE_FP16_STORAGE": "1"}

# real-field scenes: periodic, CPML, symmetry and PEC walls, TFSF columns,
# dipoles, Drude / Lorentz / critical-point matter, more than 8 objects,
# graded grids, far-field maps
HALF_CASES = [
    ("c1", 1, 120), ("c2", 1, 100), ("dipole", 1, 120), ("unitcell", 1, 120), ("sym", 1, 120),
    ("pec", 1, 120), ("spheres", 1, 80), ("nug", 1, 120), ("bowtie", 1, 120), ("multi", 1, 100),
    ("aniso", 1, 100), ("lattice", 1, 100), ("farmaps", 1, 100), ("beamtf", 1, 100), ("c5", 2, 80),
]
IDS = ["%s-%d-%d" % c for c in HALF_CASES]


@pytest.mark.gpu
@pytest.mark.parametrize("scene,scale,steps", HALF_CASES, ids=IDS)
def test_half_storage_bit_identical_to_oracle(scene, scale, steps):
    gpu = scenes.run("engine", scene, scale, steps, env=ENGINE)
    cpu = scenes.run("oracle", scene, scale, steps, env=ORACLE)
    near = {k: v for k, v in gpu.items() if not k.startswith(FAR)}
    bad = scenes.compare_exact(near, {k: v for k, v in cpu.items() if not k.startswith(FAR)})
    assert not bad, "differs from the oracle's half storage: %s" % bad[:10]
    if any(k.startswith(FAR) for k in gpu):
        check_far_field(gpu, scenes.run("oracle", scene, scale, steps, env=dict(ORACLE, ALIS_ORACLE_FF64="1")))


def half_fields(dump):
    return [k for k in dump if re.fullmatch(r"W\.[EH]0\.[xyz]", k)]


def assert_half_values(dump):
    """Every E and H value is a half value times a power of two: at most
    11 significant bits, so the low 13 of a float's 23 stored mantissa
    bits are zero (normal floats; the exponents keep every value normal)."""
    fields = half_fields(dump)
    assert fields
    for k in fields:
        v = np.ascontiguousarray(dump[k], dtype=np.float32).reshape(-1)
        u = v.view(np.uint32)
        assert not (u & 0x7F800000 == 0)[v != 0].any(), k
        assert not (u & 0x1FFF).any(), k


@pytest.mark.gpu
def test_half_storage_is_the_stored_form():
    """The half run differs from the float run (the rounding is in effect)
    and dumps only half values."""
    half = scenes.run("engine", "c2", 1, 60, env=ENGINE)
    full = scenes.run("engine", "c2", 1, 60)
    assert any(not np.array_equal(half[k], full[k]) for k in half_fields(half))
    assert_half_values(half)


@pytest.mark.gpu
@pytest.mark.parametrize("scene,scale,steps", [("c1", 1, 120), ("c2", 1, 100), ("unitcell", 1, 120)],
                         ids=["c1", "c2", "unitcell"])
@pytest.mark.parametrize("shape", [0, 2], ids=["32x2", "32x8"])
def test_half_storage_fused_column_and_shapes(scene, scale, steps, shape):
    """Half storage with the TFSF auxiliary column inside the world's own
    half-step launch (ALISGPU_AUX_ATTACH=2: the k_half_step_aux instances)
    and with each other block shape (ALISGPU_STEP_SHAPE), byte-identical to
    the oracle's half storage."""
    env = dict(ENGINE, ALISGPU_AUX_ATTACH="2", ALISGPU_STEP_SHAPE=str(shape))
    gpu = scenes.run("engine", scene, scale, steps, env=env)
    cpu = scenes.run("oracle", scene, scale, steps, env=ORACLE)
    near = {k: v for k, v in gpu.items() if not k.startswith(FAR)}
    bad = scenes.compare_exact(near, {k: v for k, v in cpu.items() if not k.startswith(FAR)})
    assert not bad, "differs from the oracle's half storage: %s" % bad[:10]


@pytest.mark.gpu
def test_complex_world_keeps_float_storage():
    """With ALIS_FIELD_STORAGE=half a world with complex (Bloch) fields
    stays in float storage (the device refuses half storage for it): the
    same bytes as the oracle's float run."""
    gpu = scenes.run("engine", "bloch", 1, 80, env=ENGINE)
    cpu = scenes.run("oracle", "bloch", 1, 80)
    near = {k: v for k, v in gpu.items() if not k.startswith(FAR)}
    bad = scenes.compare_exact(near, {k: v for k, v in cpu.items() if not k.startswith(FAR)})
    assert not bad, "differs from the oracle's float run: %s" % bad[:10]
