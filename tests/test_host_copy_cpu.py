"""The runtime's chunked multi-threaded host copy (pinned staging in and out of GB300Backend and the streaming
forward): exact for small and large arrays, non-contiguous and float64 sources, and every chunk boundary."""
import numpy as np
import pytest

from ffnoml_gb300.runtime import _host_copy


@pytest.mark.parametrize("n", [1, 7, (1 << 22) - 1, (1 << 22) + 3, 3 * (1 << 22) + 17, 8 * (1 << 22) + 5])
def test_host_copy_exact(n):
    rng = np.random.default_rng(n)
    src = rng.standard_normal(n).astype(np.float32)
    dst = np.full(n, np.nan, np.float32)
    _host_copy(dst, src)
    assert np.array_equal(dst, src)


def test_host_copy_shapes_and_types():
    rng = np.random.default_rng(0)
    src = rng.standard_normal((6, 40, 30, 20))
    dst = np.empty((6, 40, 30, 20), np.float32)
    _host_copy(dst, src)                                  # float64 source: converted like np.asarray(.., float32)
    assert np.array_equal(dst, src.astype(np.float32))
    t = rng.standard_normal((20, 30, 40)).astype(np.float32).transpose(2, 1, 0)   # non-contiguous source
    d2 = np.empty((40, 30, 20), np.float32)
    _host_copy(d2, t)
    assert np.array_equal(d2, t)


def test_host_copy_refuses_a_destination_it_cannot_fill_in_place():
    src = np.ones((4, 5), np.float32)
    for dst in (np.empty((5, 4), np.float32).T, np.empty((4, 5), np.float64), np.empty((2, 9), np.float32)):
        with pytest.raises(ValueError):
            _host_copy(dst, src)


def test_host_copy_flattens_into_a_flat_buffer():
    src = np.arange(24, dtype=np.float32).reshape(2, 3, 4)
    dst = np.empty(24, np.float32)                        # the streaming forward's flat pinned buffers
    _host_copy(dst, src)
    assert np.array_equal(dst, src.reshape(-1))
