"""The oracle's host generator of the seeded fBm volumes (oracle/scene_oracle.cpp) against the
independent numpy restatement in tests/_scenes.py: identical bits, for a single cloud and a
union of two (the device generator is compared with the oracle's on the GPU)."""
import numpy as np
import pytest

from oracle import orc
from rtc8_gb300.configs import VolumeSpec

from ._scenes import fbm_numpy


@pytest.mark.parametrize("spec", [VolumeSpec(n=24, seed=9, octaves=5, threshold=0.4),
                                  VolumeSpec(n=20, seed=3, octaves=6, threshold=0.0),
                                  VolumeSpec(n=16, seed=9, octaves=5, threshold=0.5, union_seed=11)])
def test_host_fbm_matches_numpy_restatement(spec):
    got = orc.fbm_volume(spec)
    ref = fbm_numpy(spec.n, spec.seed, spec.octaves, spec.lacunarity, spec.gain, spec.base_frequency, spec.threshold)
    if spec.union_seed is not None:
        ref = np.maximum(ref, fbm_numpy(spec.n, spec.union_seed, spec.octaves, spec.lacunarity, spec.gain,
                                        spec.base_frequency, spec.threshold))
    np.testing.assert_array_equal(got, ref)
    assert got.min() >= 0.0 and got.max() == 1.0
