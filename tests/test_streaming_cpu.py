"""Host logic of the streaming backend's predict_si (ffno_batched_backend.py:291-308): request validation and the
report of populations limited to 10^+-37 (the device kernel clamps them; the reference's own test plants log10 values
of 44.9, 41.9 and -50). The device pass is replaced by a fake that returns clamped populations."""
import numpy as np
import pytest

from ffnoml_gb300.streaming import StreamingBackend


def _backend(pop):
    be = StreamingBackend.__new__(StreamingBackend)          # no device: the host logic alone
    be.messages = []
    be.log = be.messages.append
    be.forward = lambda *args, **kw: pop
    return be


def _request(shape=(24, 11, 9)):
    g = np.random.default_rng(0)
    features = g.normal(size=(6,) + shape).astype(np.float32)
    features[0] = 1e4
    z = np.linspace(14e6, -1e6, shape[0])[:, None, None] * np.ones(shape)
    return features, z


def test_limited_populations_are_reported():
    pop = np.full((24, 11, 9, 6), 1e10, np.float32)
    pop[3, 2, 1, 4] = pop[3, 2, 1, 5] = np.float32(10.0 ** 37)   # log10 44.9 and 41.9 clamped
    pop[4, 2, 1, 0] = np.float32(10.0 ** -37)                     # log10 -50 clamped
    be = _backend(pop)
    out = be.predict_si(*_request(), 48e3, 48e3)
    assert np.isfinite(out).all() and (out > 0).all()
    assert abs(np.log10(out[3, 2, 1, 4]) - 37.0) < 1e-4 and abs(np.log10(out[4, 2, 1, 0]) + 37.0) < 1e-4
    assert any("3 predicted populations" in m for m in be.messages)


def test_nothing_is_reported_within_the_limits():
    pop = np.full((24, 11, 9, 6), 1e36, np.float32)
    pop[0, 0, 0, 0] = np.float32(10.0 ** -36.9)
    be = _backend(pop)
    be.predict_si(*_request(), 48e3, 48e3)
    assert be.messages == []


def test_requests_are_validated_before_the_device():
    be = _backend(None)
    f, z = _request()
    bad = f.copy()
    bad[0, 0, 0, 0] = -1.0
    with pytest.raises(ValueError, match="temperature"):
        be.predict_si(bad, z, 48e3, 48e3)
    bad = f.copy()
    bad[2, 1, 1, 1] = np.nan
    with pytest.raises(ValueError, match="NaN"):
        be.predict_si(bad, z, 48e3, 48e3)
    with pytest.raises(ValueError):
        be.predict_si(f[:5], z, 48e3, 48e3)
