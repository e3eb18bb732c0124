"""GPU parity of the hand-written input VJP against the reference's float64 autograd VJP (tests/golden/)."""
import pytest
import torch

from golden_io import CASES, load, model_config

pytestmark = pytest.mark.gpu


def _model(meta, state):
    from ffnoml_gb300 import FFNO3D
    m = FFNO3D(**model_config(meta))
    m.load_state_dict({k: v.float() for k, v in state.items()}, strict=True)
    return m.cuda().eval()


def _rel(a, b):
    return ((a - b).abs().max() / b.abs().max()).item()


@pytest.mark.parametrize("cache", [True, False], ids=["cached", "recomputed"])
@pytest.mark.parametrize("name", CASES)
def test_vjp_matches_reference_float64(name, cache):
    meta, state, a = load(name)
    model = _model(meta, state)
    model.executor().cache_states = cache
    x = a["x"].float().cuda().requires_grad_(True)
    z = a["z"].float().cuda().requires_grad_(True)
    y = model(x, z, meta["dx"], meta["dy"])
    y.backward(a["cot"].float().cuda())
    xb, zb = x.grad.double().cpu(), z.grad.double().cpu()
    ex = _rel(xb, a["xbar"])
    ez = _rel(zb, a["zbar"])
    print(f"{name}: x_bar rel {ex:.2e}  z_bar rel {ez:.2e}")
    # FP32 path: VJP relative error <= 1e-4 against the float64 reference gradient
    assert ex < 1e-4
    # z_bar (depth weights, z_proj and the height tables of the shared column or of every column) against float64
    assert ez < 1e-3


def _grads(model, a, meta, cache):
    model.executor().cache_states = cache
    x = a["x"].float().cuda().requires_grad_(True)
    z = a["z"].float().cuda().requires_grad_(True)
    y = model(x, z, meta["dx"], meta["dy"])
    y.backward(a["cot"].float().cuda())
    return y.detach(), x.grad, z.grad


@pytest.mark.parametrize("precision", ["fp32", "bf16"])
@pytest.mark.parametrize("name", CASES)
def test_cached_block_states_equal_recompute(name, precision):
    """Keeping every block's intermediates from the forward gives the same bits as recomputing each block in the
    backward (the same kernels on the same inputs)."""
    meta, state, a = load(name)
    model = _model(meta, state).set_precision(precision)
    y0, xb0, zb0 = _grads(model, a, meta, False)
    y1, xb1, zb1 = _grads(model, a, meta, True)
    assert torch.equal(y0, y1)
    assert torch.equal(xb0, xb1)
    assert torch.equal(zb0, zb1)
