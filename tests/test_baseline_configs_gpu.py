"""GPU parity at the benchmark configurations' architectures against the reference's own float64 run
(tests/golden/make_golden.py RECIPE_CASES): config 0 in full (width 32, 4 blocks, M = 16, [1,6,64,32,32]); the
width-64, 8-block, two-species model of configs 1-4 on a 64 x 32 x 32 sub-cube; the production model (width 96,
M = 1001) at D = 64 and D = 256; production M at D = 256 on width 64 (the tensor-core path's sliced 680-row height
transforms); and config 3's central-difference check at 64 pairs.

Bounds (from the specification of this path): max |d log10 n| <= 1e-5 for the FP32 path (or 1.5 x the reference's
own FP32 error where that exceeds 1e-5) and <= 2e-3 for the split-BF16 path; input-VJP relative error
max |d x_bar| / max |x_bar| <= 1e-4 (FP32) and <= 1e-2 (BF16)."""
import numpy as np
import pytest
import torch

from golden_io import RECIPE_CASES, load_recipe, recipe_fp32_bound, recipe_model

pytestmark = pytest.mark.gpu


def _rel(a, b):
    return ((a - b).abs().max() / b.abs().max()).item()


def _run(model, a, meta, grad=True):
    x = a["x"].float().cuda().requires_grad_(grad)
    z = a["z"].float().cuda().requires_grad_(grad)
    y = model(x, z, meta["dx"], meta["dy"])
    if not grad:
        return y.detach().double().cpu(), None, None
    y.backward(a["cot"].float().cuda())
    torch.cuda.synchronize()
    return y.detach().double().cpu(), x.grad.double().cpu(), z.grad.double().cpu()


@pytest.mark.parametrize("name", RECIPE_CASES)
def test_fp32_forward_and_vjp_against_reference_float64(name):
    meta, a = load_recipe(name)
    model = recipe_model(meta)
    y, xb, zb = _run(model, a, meta)
    err = (y - a["y64"]).abs().max().item()
    ex, ez = _rel(xb, a["xbar"]), _rel(zb, a["zbar"])
    bound = recipe_fp32_bound(meta)
    print(f"{name} fp32: max |d log10 n| {err:.2e} (bound {bound:.2e}; reference fp32 {meta['env32']:.2e}), "
          f"x_bar rel {ex:.2e} (reference fp32 {meta['env_xbar32']:.2e}), z_bar rel {ez:.2e}")
    assert err <= bound
    assert ex <= 1e-4
    assert ez <= 1e-3


@pytest.mark.parametrize("name", RECIPE_CASES)
def test_bf16_forward_and_vjp_against_reference_float64(name):
    meta, a = load_recipe(name)
    model = recipe_model(meta).set_precision("bf16")
    y, xb, zb = _run(model, a, meta)
    err = (y - a["y64"]).abs().max().item()
    ex = _rel(xb, a["xbar"])
    ex_ = model.executor()
    print(f"{name} bf16: max |d log10 n| {err:.2e}, x_bar rel {ex:.2e}, tensor cores: widths 16-64 kernels "
          f"{ex_._packed.tc}, width-96 kernels {ex_._tc_fuse96()}, transforms {ex_._tc_xf()}")
    assert err <= 2e-3
    assert ex <= 1e-2


@pytest.mark.parametrize("precision,bound", [("fp32", 1e-4), ("bf16", 1e-2)])
def test_vjp_against_reference_central_differences(precision, bound):
    """Config 3's check: the input VJP at 64 random (channel, voxel) pairs against the reference's float64 central
    differences, eps = 1e-3 on the normalised inputs, of <cotangent, output>; width-64, 8-block, two-species model."""
    meta, a = load_recipe("cfg3_fd")
    model = recipe_model(meta).set_precision(precision)
    _, xb, _ = _run(model, a, meta)
    idx, fd = a["fd_index"].numpy(), a["fd_value"].numpy()
    assert len(idx) == 64 and meta["fd_eps"] == 1e-3
    got = xb.reshape(-1)[torch.from_numpy(idx)].numpy()
    scale = float(xb.abs().max())
    worst = float(np.abs(got - fd).max() / scale)
    print(f"cfg3_fd {precision}: max |FD - VJP| / max |VJP| over 64 pairs = {worst:.2e}")
    assert worst <= bound
