"""The oracle's FP16 storage form (ALIS_ORACLE_FP16_STORAGE=1), on the
host: the checker of the engine's half storage.  Its fields carry only
half values times a power of two, the rounding is in effect, the run is
deterministic, and the exponent rule matches the C-ABI's statement."""
import numpy as np

import scenes
from test_gpu_half import ORACLE, assert_half_values, half_fields


def test_oracle_half_fields_are_half_values():
    half = scenes.run("oracle", "c2", 1, 40, env=ORACLE)
    full = scenes.run("oracle", "c2", 1, 40)
    assert any(not np.array_equal(half[k], full[k]) for k in half_fields(half))
    assert_half_values(half)


def test_oracle_half_storage_deterministic():
    a = scenes.run("oracle", "dipole", 1, 40, env=ORACLE)
    b = scenes.run("oracle", "dipole", 1, 40, env=ORACLE)
    assert not scenes.compare_exact(a, b)

