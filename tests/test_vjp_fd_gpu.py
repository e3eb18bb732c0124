"""The FP32 input VJP against central finite differences of the float64 oracle: eps = 1e-3 on normalised inputs at
random (voxel, channel) pairs, the check the reference's inversion uses for its gradients (config 3's FD check, at a
size the float64 oracle runs in seconds)."""
import numpy as np
import pytest
import torch

from golden_io import load, model_config

pytestmark = pytest.mark.gpu

EPS = 1e-3
PAIRS = 24


@pytest.mark.parametrize("name", ["w64_m32", "hca_stretched"])
def test_vjp_matches_central_differences_of_the_float64_oracle(name):
    from ffnoml_gb300 import FFNO3D
    from oracle.ffno_oracle import OracleFFNO3D
    meta, state, a = load(name)
    cfg = model_config(meta)
    model = FFNO3D(**cfg)
    model.load_state_dict({k: v.float() for k, v in state.items()}, strict=True)
    model = model.cuda().eval()
    x = a["x"].float().cuda().requires_grad_(True)
    z = a["z"].float().cuda()
    cot = a["cot"].double()
    model(x, z, meta["dx"], meta["dy"]).backward(cot.float().cuda())
    xbar = x.grad.double().cpu()

    oracle = OracleFFNO3D({k: v.double() for k, v in state.items()}, cfg, torch.float64)
    x64, z64 = a["x"].double(), a["z"].double()

    def objective(xx):
        with torch.no_grad():
            return float((oracle.forward(xx, z64, meta["dx"], meta["dy"]) * cot).sum())

    g = np.random.default_rng(11)
    flat = x64.reshape(-1)
    idx = g.choice(flat.numel(), size=PAIRS, replace=False)
    scale = float(xbar.abs().max())
    worst = 0.0
    for i in idx:
        xp, xm = flat.clone(), flat.clone()
        xp[i] += EPS
        xm[i] -= EPS
        fd = (objective(xp.reshape(x64.shape)) - objective(xm.reshape(x64.shape))) / (2 * EPS)
        worst = max(worst, abs(fd - float(xbar.reshape(-1)[i])) / scale)
    print(f"{name}: max |FD - VJP| / max|VJP| over {PAIRS} pairs = {worst:.2e}")
    # central differences in float64 at eps = 1e-3 carry O(eps^2) truncation; the FP32 VJP is ~1e-7 relative
    assert worst < 1e-4
