"""The warp-cooperative direct fold (rust-sloth_gb300/csrc/direct.cuh, direct_raster_warp)
finds a sample's row as floor((i + 0.5) * rcp(cols)) in f32 instead of an integer
division.  A direct triangle has at most 256 samples in its range plus one probe column per
row, so i < 1024 and cols <= 257; this checks the f32 form against i // cols over a wider
range, with the same correctly rounded operations (an exact add, a correctly rounded
reciprocal and product)."""
import numpy as np


def test_reciprocal_row_division_is_exact():
    i = np.arange(0, 4096, dtype=np.int64)
    for cols in range(1, 600):
        r = np.float32(1.0) / np.float32(cols)
        q = ((i.astype(np.float32) + np.float32(0.5)) * r).astype(np.int64)
        assert np.array_equal(q, i // cols), cols
