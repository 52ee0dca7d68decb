"""bench.py's host arrays for the C-ABI calls: anonymous mappings advised
onto huge pages, shaped like the state, writable, and readable back."""
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)


def test_host_array_matches_the_state():
    import bench
    like = np.arange(5 * 6 * 7, dtype=np.float64).reshape(5, 6, 7)
    a, huge = bench.host_array(like)
    assert a.shape == like.shape and a.dtype == like.dtype and isinstance(huge, bool)
    a[...] = like
    assert np.array_equal(a, like)
    assert a.flags.c_contiguous and a.flags.writeable
