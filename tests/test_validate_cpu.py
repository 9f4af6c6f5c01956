"""Host-side helpers of the validation and bench workloads (no GPU)."""
import numpy as np

from lbmcl_gb300.validate import smooth_lid


def test_smooth_lid_is_seeded_bounded_and_smooth():
    a = smooth_lid(64, np.random.default_rng(1234))
    b = smooth_lid(64, np.random.default_rng(1234))
    np.testing.assert_array_equal(a, b)                       # seeded
    assert a.shape == (64, 64)
    dev = a - 0.05
    assert abs(np.abs(dev).max() - 0.02) < 1e-15              # total amplitude 0.02 around 0.05
    # smooth: neighbouring columns differ by far less than the amplitude
    assert np.abs(np.diff(a, axis=1)).max() < 0.02 * 2 * np.pi * 3 * 4 / 64
    assert not np.array_equal(a, smooth_lid(64, np.random.default_rng(7)))
