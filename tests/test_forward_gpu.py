"""GPU parity of the forward pass: the GB300 kernels (through the C ABI, driven by the drop-in module) against the
reference's float64 outputs in tests/golden/ and the float64 oracle."""
import pytest
import torch

from golden_io import CASES, load, model_config

pytestmark = pytest.mark.gpu


def _model(meta, state):
    from ffnoml_gb300 import FFNO3D
    cfg = model_config(meta)
    m = FFNO3D(**cfg)
    m.load_state_dict({k: v.float() for k, v in state.items()}, strict=True)
    return m.cuda().eval()


@pytest.mark.parametrize("name", CASES)
def test_forward_matches_reference_float64(name):
    meta, state, a = load(name)
    model = _model(meta, state)
    with torch.no_grad():
        y = model(a["x"].float().cuda(), a["z"].float().cuda(), meta["dx"], meta["dy"])
    torch.cuda.synchronize()
    err = (y.double().cpu() - a["y64"]).abs().max().item()
    ref_err = (a["y32"] - a["y64"]).abs().max().item()
    # FP32 path: max |d log10 n| <= 1e-5 (the reference's own FP32 rounding is ref_err)
    assert err < 1e-5, (err, ref_err)


def test_forward_is_deterministic():
    meta, state, a = load("w32_m16")
    model = _model(meta, state)
    x, z = a["x"].float().cuda(), a["z"].float().cuda()
    with torch.no_grad():
        y1 = model(x, z, meta["dx"], meta["dy"])
        y2 = model(x, z, meta["dx"], meta["dy"])
    assert torch.equal(y1, y2)
