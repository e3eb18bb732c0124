"""Generate the SI-level golden fixture tests/golden/si_hca.npz with the reference's own service conversions
(harshmathur1990/FFNOML ffno_fsdp_runtime.py: _model_inputs, linear_populations, and the composition of
_forward_linear / _canonical_populations, :265-292) around the reference's own FFNO3D, in float64 on CPU.

Run where the reference is checked out, naming its directory in FFNOML_REFERENCE or with --reference:
    FFNOML_REFERENCE=<reference checkout> python tests/golden/make_golden_si.py
The fixture is committed; the tests read it and never import the reference.

It holds the seeded model's state dict, its config (json), SI inputs (features (6, nz, nx, ny): T [K], vx, vy, vz
[m/s], log10 ne, log10 rho; z (nz, nx, ny) in metres), the float64 populations (nz, nx, ny, L) as predict_local
lays them out, a population cotangent with the float64 VJP (features_bar, z_bar) as vjp_local returns it, and a
feature tangent with the float64 population tangent as jvp_local returns it (heights fixed).
"""
import json
import os
import sys

import numpy as np
import torch
import torch.autograd.forward_ad as fwAD

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)
from make_golden import ATOM, MEAN_X, STD_X, build, synthetic  # noqa: E402  (puts the reference on sys.path)
from ffno_fsdp_runtime import _model_inputs, linear_populations  # noqa: E402

CONFIG = dict(width=16, n_layers=2, hidden_spectral=16, hidden_vertical=16, freq_mix_rank=4, z_min_wavelength=0.5,
              atoms=["H", "CA"])
SEED, SHAPE, DX, DY = 21, (1, 6, 12, 6, 8), 48e3, 48e3


def si_inputs():
    """The synthetic model-unit inputs of make_golden, turned into the SI quantities the service receives."""
    x, z_mm = synthetic(SHAPE, SEED + 100, "stretched")
    raw = x * torch.as_tensor(STD_X, dtype=torch.float64)[:, None, None, None] + \
        torch.as_tensor(MEAN_X, dtype=torch.float64)[:, None, None, None]
    feats = torch.cat((10.0 ** raw[:, 0:1], raw[:, 1:4] * 1.0e3, raw[:, 4:6]), dim=1)
    return feats[0].float().double(), (z_mm[0] * 1.0e6).float().double()


def main():
    model = build(CONFIG, SEED)
    state = {k: v.detach().clone().numpy() for k, v in model.state_dict().items()}
    torch.set_default_dtype(torch.float64)
    m64 = model.double()
    norm = {k: getattr(m64, k).detach()[None, :, None, None, None] for k in ("mean_X", "std_X", "mean_Y", "std_Y")}

    def populations(features, z_m):
        # _forward_linear (ffno_fsdp_runtime.py:265-281) and _canonical_populations (:283-292) in float64
        f, z_model = _model_inputs(features[None], z_m[None])
        pred = m64((f - norm["mean_X"]) / norm["std_X"], z_model, DX, DY)
        return linear_populations(pred * norm["std_Y"] + norm["mean_Y"])[0].permute(1, 2, 3, 0)

    features, z_m = si_inputs()
    L = sum(ATOM[a]["levels"] for a in CONFIG["atoms"])
    g = torch.Generator().manual_seed(SEED + 200)
    fr = features.clone().requires_grad_(True)
    zr = z_m.clone().requires_grad_(True)
    pops = populations(fr, zr)
    cot = torch.randn(pops.shape, generator=g, dtype=torch.float64) / pops.detach()
    fb, zb = torch.autograd.grad(pops, (fr, zr), cot)
    scale = torch.tensor([0.01, 100.0, 100.0, 100.0, 0.01, 0.01], dtype=torch.float64)[:, None, None, None]
    tangent = torch.randn(features.shape, generator=g, dtype=torch.float64) * scale
    tangent[0] *= features[0]                                    # relative temperature perturbations
    # as jvp_local (ffno_fsdp_runtime.py:350-372): dual tensors under no_grad, so the blocks run without checkpointing
    with torch.no_grad(), fwAD.dual_level():
        pdot = fwAD.unpack_dual(populations(fwAD.make_dual(features, tangent), z_m)).tangent
    torch.set_default_dtype(torch.float32)
    meta = dict(config=CONFIG, seed=SEED, shape=list(SHAPE), dx=DX, dy=DY)
    np.savez_compressed(os.path.join(HERE, "si_hca.npz"), meta=json.dumps(meta), features=features.numpy(),
                        z_m=z_m.numpy(), pops=pops.detach().numpy(), cot=cot.numpy(), features_bar=fb.numpy(),
                        z_bar=zb.numpy(), tangent=tangent.numpy(), pops_dot=pdot.detach().numpy(),
                        **{"state/" + k: v for k, v in state.items()})
    print(f"si_hca: populations {tuple(pops.shape)}, range {pops.min().item():.3e} .. {pops.max().item():.3e}")


if __name__ == "__main__":
    main()
