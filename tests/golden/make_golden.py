"""Generate the golden fixtures under tests/golden/ by running the reference's own FFNO3D (harshmathur1990/FFNOML,
models/ffno_model.py) in float64 on CPU.

Run in a container that has the reference checked out (default /root/reference, override with FFNOML_REFERENCE):
    python tests/golden/make_golden.py
The fixtures are committed; the tests read them and never import the reference.

Each fixture (.npz) holds: the seeded model's state dict (float32, as initialised), its constructor config (json), the
inputs (float64), the reference's float64 output, the reference's float32 output (its own rounding envelope), and the
float64 input VJP (x_bar, z_bar) along a seeded cotangent.
"""
import json
import math
import os
import sys

import numpy as np
import torch

REF = os.environ.get("FFNOML_REFERENCE", "/root/reference")
sys.path.insert(0, REF)
from config import ATOM_CONFIG  # noqa: E402
from models.ffno_model import FFNO3D  # noqa: E402

HERE = os.path.dirname(os.path.abspath(__file__))
ATOM = {a: {k: ATOM_CONFIG[a][k] for k in ("levels", "log10_particle_mass", "multi3d_lte")} for a in ("H", "CA")}
# normalisation: the analytic moments of the synthetic input distributions (log10 T ~ U(3.5, 6), v ~ N(0, 5 km/s),
# log10 ne ~ U(14, 21), log10 rho ~ U(-12, -4)), in model units
MEAN_X = np.array([4.75, 0.0, 0.0, 0.0, 17.5, -8.0], np.float32)
STD_X = np.array([2.5 / math.sqrt(12), 5.0, 5.0, 5.0, 7.0 / math.sqrt(12), 8.0 / math.sqrt(12)], np.float32)


def build(config, seed):
    torch.set_default_dtype(torch.float32)
    torch.manual_seed(seed)
    cfg = dict(config)
    cfg["species"] = [ATOM[a] for a in cfg.pop("atoms")]
    out = sum(s["levels"] for s in cfg["species"])
    model = FFNO3D(in_channels=6, out_channels=out, **cfg).eval()
    with torch.no_grad():
        # every branch live: the low-rank U (zero at init) and the species' total-correction rows
        for name, p in model.named_parameters():
            if ".freq_u." in name:
                p.normal_(0.0, 0.1)
        c = 0
        for s in cfg["species"]:
            model.proj2.weight[c + s["levels"]].normal_(0.0, 0.3)
            model.proj2.bias[c + s["levels"]].normal_(0.0, 0.3)
            c += s["levels"] + 1
    model.set_normalization(MEAN_X, STD_X, np.linspace(0.5, 1.5, out), np.linspace(1.0, 2.0, out))
    return model


def synthetic(shape, seed, z_kind):
    """Inputs of the synthetic distributions, z-scored; heights in Mm, top first."""
    B, _, D, H, W = shape
    g = torch.Generator().manual_seed(seed)
    raw = torch.empty(B, 6, D, H, W, dtype=torch.float64)
    raw[:, 0] = 3.5 + 2.5 * torch.rand(B, D, H, W, generator=g, dtype=torch.float64)
    raw[:, 1:4] = 5.0 * torch.randn(B, 3, D, H, W, generator=g, dtype=torch.float64)
    raw[:, 4] = 14 + 7 * torch.rand(B, D, H, W, generator=g, dtype=torch.float64)
    raw[:, 5] = -12 + 8 * torch.rand(B, D, H, W, generator=g, dtype=torch.float64)
    x = (raw - torch.as_tensor(MEAN_X, dtype=torch.float64)[:, None, None, None]) / \
        torch.as_tensor(STD_X, dtype=torch.float64)[:, None, None, None]
    if z_kind == "uniform":
        col = torch.linspace(14.0, -1.0, D, dtype=torch.float64)
    elif z_kind == "stretched":
        s = torch.linspace(0.0, 1.0, D, dtype=torch.float64)
        col = (-1.0 + 15.0 * (0.4 * s + 0.6 * s ** 2)).flip(0)
    elif z_kind == "tall":
        col = torch.linspace(15.0, 0.0, D, dtype=torch.float64)
    else:
        raise ValueError(z_kind)
    z = col[:, None, None].expand(D, H, W)[None].repeat(B, 1, 1, 1).contiguous()
    # round the grid to float32 values so that the float32 and float64 runs see the same heights
    return x.float().double(), z.float().double()


CASES = {
    # name: (constructor config, seed, input shape, z kind, per-column perturbation)
    "h_uniform": (dict(width=16, n_layers=2, hidden_spectral=16, hidden_vertical=16, z_min_wavelength=0.3,
                       atoms=["H"]), 3, (1, 6, 12, 10, 9), "uniform", False),
    "hca_stretched": (dict(width=16, n_layers=2, hidden_spectral=16, hidden_vertical=16, freq_mix_rank=4,
                           z_min_wavelength=0.5, atoms=["H", "CA"]), 4, (1, 6, 20, 8, 12), "stretched", False),
    "per_column": (dict(width=16, n_layers=1, hidden_spectral=16, hidden_vertical=16, z_min_wavelength=0.5,
                        atoms=["H"]), 5, (1, 6, 10, 5, 6), "uniform", True),
    "tall_box": (dict(width=16, n_layers=1, hidden_spectral=16, hidden_vertical=16, z_reference_length=20.0,
                      z_min_wavelength=0.5, atoms=["H"]), 6, (1, 6, 16, 6, 8), "tall", False),
    "batch2": (dict(width=16, n_layers=1, hidden_spectral=16, hidden_vertical=16, z_min_wavelength=0.5,
                    atoms=["H", "CA"]), 7, (2, 6, 9, 7, 5), "stretched", False),
    "w32_m16": (dict(width=32, n_layers=2, hidden_spectral=32, hidden_vertical=32, z_min_wavelength=40.0 / 15,
                     atoms=["H"]), 8, (1, 6, 16, 16, 16), "uniform", False),
    "w64_m32": (dict(width=64, n_layers=1, hidden_spectral=32, hidden_vertical=32, z_min_wavelength=40.0 / 31,
                     atoms=["H", "CA"]), 9, (1, 6, 16, 8, 8), "uniform", False),
}


def run_case(name, config, seed, shape, z_kind, per_column):
    model = build(config, seed)
    state = {k: v.detach().clone().numpy() for k, v in model.state_dict().items()}
    x, z = synthetic(shape, seed + 100, z_kind)
    if per_column:
        z = z.clone()
        z[0, :, 2, 3] += 0.05 * torch.linspace(0.0, 1.0, shape[2], dtype=torch.float64)     # one column apart
        z = z.float().double()
    L = sum(ATOM[a]["levels"] for a in config["atoms"])
    g = torch.Generator().manual_seed(seed + 200)
    cot = torch.randn(shape[0], L, *shape[2:], generator=g, dtype=torch.float64)
    dx, dy = 48e3, 48e3
    with torch.no_grad():
        y32 = model(x.float(), z.float(), dx, dy).double()
    torch.set_default_dtype(torch.float64)
    m64 = model.double()
    xr = x.clone().requires_grad_(True)
    zr = z.clone().requires_grad_(True)
    y64 = m64(xr, zr, dx, dy)
    xb, zb = torch.autograd.grad(y64, (xr, zr), cot)
    torch.set_default_dtype(torch.float32)
    meta = dict(config=config, seed=seed, shape=list(shape), z_kind=z_kind, per_column=per_column, dx=dx, dy=dy)
    np.savez_compressed(os.path.join(HERE, f"{name}.npz"), meta=json.dumps(meta), x=x.numpy(), z=z.numpy(),
                        y64=y64.detach().numpy(), y32=y32.numpy(), cot=cot.numpy(), xbar=xb.numpy(), zbar=zb.numpy(),
                        **{"state/" + k: v for k, v in state.items()})
    err32 = (y32 - y64.detach()).abs().max().item()
    print(f"{name}: out {tuple(y64.shape)}, reference fp32 vs fp64 max |d| = {err32:.2e}")


def head_case():
    """The head alone on random head channels, [H, CA] (FFNO3D.head_output, models/ffno_model.py:730-749)."""
    model = build(dict(width=16, n_layers=1, hidden_spectral=16, hidden_vertical=16, z_min_wavelength=0.5,
                       atoms=["H", "CA"]), 11)
    g = torch.Generator().manual_seed(12)
    head = torch.randn(1, 14, 5, 4, 3, generator=g, dtype=torch.float64) * 3
    x, _ = synthetic((1, 6, 5, 4, 3), 13, "uniform")
    torch.set_default_dtype(torch.float64)
    m64 = model.double()
    out = m64.head_output(head, x)
    torch.set_default_dtype(torch.float32)
    state = {k: v.detach().float().numpy() for k, v in model.state_dict().items()}
    np.savez_compressed(os.path.join(HERE, "head.npz"), meta=json.dumps(dict(atoms=["H", "CA"])), head=head.numpy(),
                        x=x.numpy(), y64=out.detach().numpy(), **{"state/" + k: v for k, v in state.items()})
    print("head: done")


if __name__ == "__main__":
    for name, case in CASES.items():
        run_case(name, *case)
    head_case()
