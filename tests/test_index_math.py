"""CPU checks of the integer arithmetic the fast kernels replace by FP32
operations (k_fast.cu): the oversampled region's floor division of a window
coordinate by the scale k is computed as floor((x + 1/2) * (1/k)) with the
correctly rounded FP32 reciprocal.  The claim in the kernel's comment -- exact
for |x| < 2^21 and every k in 1..128 -- is checked here exhaustively with
IEEE FP32 arithmetic (numpy float32: the same rounded add and multiply the
device performs; the add and the multiply cannot be fused into one FMA)."""
import numpy as np


def _floordiv_scale(x, k):
    inv = np.float32(1.0) / np.float32(k)
    return np.floor((x.astype(np.float32) + np.float32(0.5)) * inv).astype(np.int64)


def test_region_floor_division_is_exact():
    x = np.arange(-(1 << 21), 1 << 21, dtype=np.int64)
    for k in range(1, 129):
        q = _floordiv_scale(x, k)
        assert np.array_equal(q, x // k), k


def test_region_floor_division_fails_only_beyond_the_stated_range():
    """The bound is not slack for nothing: far beyond it the FP32 sum x + 1/2
    is no longer exact and the quotient can be off (here for k = 3)."""
    x = np.arange((1 << 25) - 4096, (1 << 25), dtype=np.int64)
    assert not np.array_equal(_floordiv_scale(x, 3), x // 3)
