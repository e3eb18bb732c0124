"""GB300Backend's request checks (the reference's ValueError messages, ffno_fsdp_runtime.py) now that the request's
status is read once with the results: invalid inputs are reported as such whatever the model part did with them, and a
valid call after an invalid one is unaffected."""
import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu

from test_service_gpu import _model, _request  # noqa: E402


@pytest.fixture(scope="module")
def backend():
    from ffnoml_gb300.runtime import GB300Backend
    return GB300Backend(_model("bf16"), [f"l{i}" for i in range(12)])


@pytest.mark.parametrize("op", ["predict", "vjp", "jvp"])
@pytest.mark.parametrize("bad", ["nan_feature", "nan_height", "negative_temperature"])
def test_invalid_requests_raise(backend, op, bad):
    f, z = _request((16, 8, 8), 3)
    if bad == "nan_feature":
        f[4, 3, 2, 1] = np.nan
        msg = "FFNO request contains NaN or Inf"
    elif bad == "nan_height":
        z[5, 1, 1] = np.nan
        msg = "FFNO request contains NaN or Inf"
    else:
        f[0, 2, 2, 2] = -10.0
        msg = "FFNO request temperature must be positive"
    with pytest.raises(ValueError, match=msg):
        if op == "predict":
            backend.predict_local(f, z, 48e3, 48e3)
        elif op == "vjp":
            backend.vjp_local(f, z, 48e3, 48e3, np.ones((16, 8, 8, 12), np.float32))
        else:
            backend.jvp_local(f, z, 48e3, 48e3, np.ones_like(f))
    f, z = _request((16, 8, 8), 3)
    a = backend.predict_local(f, z, 48e3, 48e3)
    b = backend.predict_local(f, z, 48e3, 48e3)
    assert np.isfinite(a).all() and np.array_equal(a, b)


def test_vjp_cotangent_check(backend):
    f, z = _request((16, 8, 8), 4)
    cot = np.ones((16, 8, 8, 12), np.float32)
    cot[1, 1, 1, 1] = np.inf
    with pytest.raises(ValueError, match="FFNO VJP cotangent contains NaN or Inf"):
        backend.vjp_local(f, z, 48e3, 48e3, cot)
    out = backend.vjp_local(f, z, 48e3, 48e3, np.ones((16, 8, 8, 12), np.float32))
    assert np.isfinite(out["features"]).all() and np.isfinite(out["z_scale"]).all()
