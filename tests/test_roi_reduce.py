"""ROI reduction of sparse beamlet columns (ee_roi_*, host code) against the
loop-for-loop restatement of the reference's _reduce_by_roi
(CCCS/DoseCalcIO/sparse_io.cpp:62-158) in oracle/sparse_io.py: identical
keys, values and row-block sizes, bit for bit.  Runs without a GPU."""
import numpy as np
import pytest

from endtoend_gb300 import engine
from oracle.sparse_io import reduce_by_roi


def _case(seed):
    rng = np.random.default_rng(seed)
    size = (int(rng.integers(6, 14)), int(rng.integers(5, 12)), int(rng.integers(4, 10)))  # x, y, z
    nvox = size[0] * size[1] * size[2]
    n = int(rng.integers(1, nvox // 2))
    keys = np.sort(rng.choice(nvox, n, replace=False)).astype(np.int32)
    vals = rng.uniform(0.0, 1.0, n).astype(np.float32)
    vals[rng.random(n) < 0.05] = 0.0  # zero rows are dropped
    rois = []
    for _ in range(int(rng.integers(1, 4))):
        c0 = [int(rng.integers(0, s)) for s in size]
        cn = [int(rng.integers(1, s - c + 1)) for s, c in zip(size, c0)]
        mask = rng.random((cn[2], cn[1], cn[0])) < 0.6
        rois.append((c0, mask))
    return size, keys, vals, rois


@pytest.mark.parametrize("seed", range(8))
def test_reduce_matches_reference_restatement(seed):
    size, keys, vals, rois = _case(seed)
    rk, rv, rb = reduce_by_roi(keys, vals, size, rois)
    L = engine.RoiList(size, rois)
    try:
        k, v, b = L.reduce(keys, vals)
        caps = L.capacities()
    finally:
        L.close()
    np.testing.assert_array_equal(k, rk)
    np.testing.assert_array_equal(v, rv)
    np.testing.assert_array_equal(b, rb)
    np.testing.assert_array_equal(caps, [int(m.sum()) for _, m in rois])


def test_overlapping_rois_and_errors():
    size = (4, 3, 2)
    mask = np.ones((2, 3, 4), bool)
    keys = np.arange(24, dtype=np.int32)
    vals = np.arange(1, 25, dtype=np.float32)
    L = engine.RoiList(size, [((0, 0, 0), mask), ((0, 0, 0), mask)])
    try:
        k, v, b = L.reduce(keys, vals)
        # every voxel once per ROI; the second block starts after the first's 24 rows
        assert list(b) == [24, 24] and k[24] == 24 and len(k) == 48
        # x slowest, z fastest: position 1 is voxel (0, 0, 1) = key 12
        assert v[1] == vals[12]
        with pytest.raises(engine.EEError):
            L.reduce(np.array([24], np.int32), np.array([1.0], np.float32))
    finally:
        L.close()
    with pytest.raises(engine.EEError):
        engine.RoiList(size, [((3, 0, 0), np.ones((1, 1, 2), bool))])
