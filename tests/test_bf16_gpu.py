"""The BF16 tensor-core path against the reference's float64 outputs: max |d log10 n| <= 2e-3 and input-VJP relative
error <= 1e-2."""
import pytest
import torch

from golden_io import CASES, load, model_config

pytestmark = pytest.mark.gpu


def _model(meta, state):
    from ffnoml_gb300 import FFNO3D
    m = FFNO3D(**model_config(meta))
    m.load_state_dict({k: v.float() for k, v in state.items()}, strict=True)
    return m.cuda().eval().set_precision("bf16")


@pytest.mark.parametrize("name", CASES)
def test_bf16_forward_and_vjp(name):
    meta, state, a = load(name)
    model = _model(meta, state)
    x = a["x"].float().cuda().requires_grad_(True)
    z = a["z"].float().cuda().requires_grad_(True)
    y = model(x, z, meta["dx"], meta["dy"])
    err = (y.detach().double().cpu() - a["y64"]).abs().max().item()
    y.backward(a["cot"].float().cuda())
    ex = ((x.grad.double().cpu() - a["xbar"]).abs().max() / a["xbar"].abs().max()).item()
    print(f"{name}: bf16 max |d log10 n| {err:.2e}, x_bar rel {ex:.2e}")
    assert err < 2e-3
    assert ex < 1e-2
