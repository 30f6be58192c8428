"""CPU check of the float-estimated division that the multigrid sweeps, the
restrictions and the E kernel use for node coordinates (div_small in
csrc/espic_world.h): for n < 2^24, trunc(float(n) * RN(1/d)) is within one of
n // d, so one remainder test makes it exact.  Emulated with numpy float32,
whose products round to nearest like the device's float multiply."""
import numpy as np


def div_small(n, d):
    inv = np.float32(1.0) / np.float32(d)
    q = np.trunc(n.astype(np.float32) * inv).astype(np.int64)
    est = q.copy()
    r = n - q * d
    q = np.where(r < 0, q - 1, np.where(r >= d, q + 1, q))
    return est, q


def test_float_estimated_division_is_exact_below_2_pow_24():
    rng = np.random.default_rng(24)
    top = 1 << 24
    for d in range(1, 4097):
        # every remainder class near multiples of d across the range, plus
        # random samples and the last representable values
        k = rng.integers(0, top // d, 256)
        n = np.concatenate([k * d, k * d + d - 1, rng.integers(0, top, 256),
                            np.arange(top - 64, top)]).astype(np.int64)
        n = n[(n >= 0) & (n < top)]
        est, q = div_small(n, d)
        want = n // d
        assert np.all(np.abs(est - want) <= 1), d
        assert np.array_equal(q, want), d
