"""The tensor-core transform packs of production height tables (M = 1001 modes: 680 live rows at D = 256) are cut
into calls of at most 256 rows and 512 columns that tile the table exactly once (no GPU work: packing only)."""
import numpy as np
import pytest


@pytest.mark.parametrize("shape", [(680, 256), (256, 680), (1320, 496), (496, 1320), (128, 64)])
def test_transform_slices_tile_the_table(shape):
    from ffnoml_gb300.executor import XFORM_TC_MAX_K, TcXform
    M, K = shape
    T = np.random.default_rng(0).normal(size=shape)
    tx = TcXform(T, "cpu")
    cover = np.zeros(shape, np.int64)
    for r0, rows, c0, cols, packed, res in tx.slices:
        assert 1 <= rows <= 256 and 1 <= cols <= XFORM_TC_MAX_K
        cover[r0:r0 + rows, c0:c0 + cols] += 1
        if res is not None:
            Mp, Kp = res[1], res[2]
            assert Mp >= rows and Kp >= cols and Mp % 16 == 0 and Kp % 16 == 0
    assert (cover == 1).all()
