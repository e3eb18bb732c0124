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


def _call(backend, op, f, z, extra, wire):
    """One call through the numpy interface (*_local) or the service's wire-layout one (*_wire)."""
    if not wire:
        if op == "predict":
            return backend.predict_local(f, z, 48e3, 48e3)
        return getattr(backend, op + "_local")(f, z, 48e3, 48e3, extra)
    arrays = [f, z] + ([] if op == "predict" else [extra])
    flat = np.concatenate([np.asarray(a, np.float32).reshape(-1, order="F") for a in arrays])
    out = torch.empty(13 * z.size).pin_memory()
    return getattr(backend, op + "_wire")(torch.from_numpy(flat).pin_memory(), z.shape, 48e3, 48e3, out)


@pytest.mark.parametrize("wire", [False, True], ids=["local", "wire"])
@pytest.mark.parametrize("op", ["predict", "vjp", "jvp"])
@pytest.mark.parametrize("bad", ["nan_feature", "nan_height", "negative_temperature"])
def test_invalid_requests_raise(backend, op, bad, wire):
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
    extra = np.ones((16, 8, 8, 12), np.float32) if op == "vjp" else np.ones_like(f)
    with pytest.raises(ValueError, match=msg):
        _call(backend, op, f, z, extra, wire)
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


@pytest.mark.parametrize("shape", [(7, 5, 3, 6), (40, 33, 17, 12), (1, 64, 48, 64), (12, 1, 70, 1)])
def test_reverse_axes4_matches_numpy(shape):
    from ffnoml_gb300 import _native as nat
    a = torch.randn(*shape, generator=torch.Generator().manual_seed(1))
    out = torch.full((a.numel(),), float("nan"), device="cuda")
    ad = a.cuda().contiguous()
    nat.call("ffno_reverse_axes4", ad.data_ptr(), *shape, out.data_ptr(), torch.cuda.current_stream().cuda_stream)
    torch.cuda.synchronize()
    assert torch.equal(out.cpu().reshape(shape[::-1]), a.permute(3, 2, 1, 0))


def test_wire_layout_calls_equal_the_numpy_calls():
    """predict_wire / vjp_wire / jvp_wire (the service's path: arrays as received, in Fortran order, reordered on the
    device) give the same bits as predict_local / vjp_local / jvp_local on the same request."""
    from ffnoml_gb300.runtime import GB300Backend
    be = GB300Backend(_model("bf16"), [f"l{i}" for i in range(12)])
    shape = (19, 12, 10)
    f, z = _request(shape, 5)
    g = np.random.default_rng(6)
    cot = (g.normal(size=shape + (12,)) * 1e-15).astype(np.float32)
    tan = g.normal(size=f.shape).astype(np.float32) * np.abs(f) * np.float32(1e-3)
    V = np.prod(shape)

    def wire(*arrays):
        flat = np.concatenate([np.asarray(a, np.float32).reshape(-1, order="F") for a in arrays])
        return torch.from_numpy(flat).pin_memory()

    out = torch.empty(13 * V).pin_memory()
    n = be.predict_wire(wire(f, z), shape, 48e3, 48e3, out)
    pop = out.numpy()[:n].reshape(shape + (12,), order="F")
    assert np.array_equal(pop, be.predict_local(f, z, 48e3, 48e3))
    n = be.vjp_wire(wire(f, z, cot), shape, 48e3, 48e3, out)
    ref = be.vjp_local(f, z, 48e3, 48e3, cot)
    assert np.array_equal(out.numpy()[:6 * V].reshape((6,) + shape, order="F"), ref["features"])
    assert np.array_equal(out.numpy()[6 * V:n].reshape(shape, order="F"), ref["z_scale"])
    n = be.jvp_wire(wire(f, z, tan), shape, 48e3, 48e3, out)
    assert np.array_equal(out.numpy()[:n].reshape(shape + (12,), order="F"), be.jvp_local(f, z, 48e3, 48e3, tan))
