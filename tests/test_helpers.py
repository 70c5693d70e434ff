"""Small host-side helpers of the Python mirror: the Partitioner's unit conversions
(Partitioner.cs:127), Rectangle and the per-rank baseline slices of the distributed layout."""
import os

import numpy as np

from conftest import pkg
from conftest import entry

C_LIGHT = 299792458.0


def test_unit_conversions_follow_the_partitioner():
    # Partitioner.MetersToLambda / MetersToPixels: m * f / c and m * imageSize * f / c
    m, f, img = 1234.5, 1.4e9, 0.0223
    assert pkg.Partitioner.MetersToLambda(m, f) == m * (f / C_LIGHT)
    assert pkg.Partitioner.MetersToPixels(m, img, f) == m * img * (f / C_LIGHT)


def test_rectangle_extents():
    r = pkg.Rectangle(3, 5, 10, 21)
    assert (r.YExtent(), r.XExtent()) == (7, 16)


def test_local_block_slices_each_rank():
    dist_mod = entry._load_module(entry.PKG_NAME + ".distributed", os.path.join(entry.PKG_DIR, "distributed.py"))
    uvw = np.arange(10 * 4 * 3, dtype=np.float64).reshape(10, 4, 3)
    parts = [dist_mod.local_block([uvw, None], 10, 3, r) for r in range(3)]
    assert [p[0].shape[0] for p in parts] == [3, 3, 4] and all(p[1] is None for p in parts)
    assert np.array_equal(np.concatenate([p[0] for p in parts]), uvw)
