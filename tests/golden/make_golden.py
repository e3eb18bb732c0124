"""Generate the golden fixtures under tests/golden/ by running the reference's own FFNO3D (harshmathur1990/FFNOML,
models/ffno_model.py) in float64 on CPU.

Run where the reference is checked out, naming its directory in FFNOML_REFERENCE or with --reference:
    FFNOML_REFERENCE=<reference checkout> python tests/golden/make_golden.py [--only name ...]
The fixtures are committed; the tests read them and never import the reference.

Each fixture (.npz) holds: the seeded model's state dict (float32, as initialised), its constructor config (json), the
inputs (float64), the reference's float64 output, the reference's float32 output (its own rounding envelope), and the
float64 input VJP (x_bar, z_bar) along a seeded cotangent.
"""
import argparse
import json
import math
import os
import sys
import time

import numpy as np
import torch


def _reference_dir():
    ap = argparse.ArgumentParser(add_help=False)
    ap.add_argument("--reference", default=os.environ.get("FFNOML_REFERENCE"))
    args, _ = ap.parse_known_args()
    if not args.reference:
        sys.exit("name the reference checkout in FFNOML_REFERENCE or with --reference")
    return args.reference


sys.path.insert(0, _reference_dir())
from config import ATOM_CONFIG  # noqa: E402
from models.ffno_model import FFNO3D  # noqa: E402

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(HERE))
import golden_io as gio  # noqa: E402
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


# ------------------------------------------------------------------------------------------------ recipe fixtures
# The benchmark configurations (their architectures; sub-cubes where the whole cube would not run in float64 on a CPU
# in minutes), with weights and inputs from the recipe of tests/golden_io.py: name -> (constructor config, seed, input
# shape, central-difference pairs). Each stores the reference's float64 output and input VJP, the largest difference
# of the reference's own float32 run from them, and for fd > 0 the reference's float64 central differences
# (eps = 1e-3 on normalised inputs) of <cotangent, output> at fd random (channel, voxel) pairs.
PRODUCTION = dict(dropout=0.0, spec_dropout=0.08, vertical_dropout=0.08, spec_dropout_layers=[0, 1, 2, 3],
                  vertical_dropout_layers=[0, 1, 2, 3], hidden_spectral=128, hidden_vertical=128, checkpoint_blocks=True,
                  freq_mix_rank=8, z_reference_length=40.0, z_min_wavelength=0.04, z_feature_wavelength=0.3)
RECIPE_CASES = {
    # config 0 in full: width 32, 4 blocks, M = 16, H
    "cfg0": (dict(width=32, n_layers=4, z_min_wavelength=40.0 / 15, atoms=["H"]), 20, (1, 6, 64, 32, 32), 0),
    # configs 1-4's model (width 64, 8 blocks, hidden 128, M = 32, H + Ca II) on a 64 x 32 x 32 sub-cube
    "cfg1_sub": (dict(width=64, n_layers=8, z_min_wavelength=40.0 / 31, atoms=["H", "CA"]), 21, (1, 6, 64, 32, 32),
                 0),
    # config 3's finite-difference check: the same model, 64 pairs on a 32 x 16 x 16 sub-cube
    "cfg3_fd": (dict(width=64, n_layers=8, z_min_wavelength=40.0 / 31, atoms=["H", "CA"]), 25, (1, 6, 32, 16, 16),
                64),
    # the production model (config.MODEL_CONFIG: width 96, 4 blocks, M = 1001): 84 live modes at D = 64, 340 at
    # D = 256 (a 680-row height transform)
    "w96_p_d64": (dict(width=96, n_layers=4, atoms=["H", "CA"], **PRODUCTION), 22, (1, 6, 64, 16, 16), 0),
    "w96_p_d256": (dict(width=96, n_layers=4, atoms=["H", "CA"], **PRODUCTION), 23, (1, 6, 256, 8, 8), 0),
    # production M at D = 256 on a width the tensor-core kernels take (their sliced tall transforms)
    "w64_p_d256": (dict(width=64, n_layers=2, atoms=["H", "CA"], **PRODUCTION), 24, (1, 6, 256, 8, 8), 0),
}
FD_EPS = 1e-3


def run_recipe_case(name, config, seed, shape, fd_pairs):
    t0 = time.time()
    cfg = dict(config)
    species = [ATOM[a] for a in cfg.pop("atoms")]
    L = sum(s["levels"] for s in species)
    torch.set_default_dtype(torch.float32)
    model = FFNO3D(in_channels=6, out_channels=L, species=species, **cfg).eval()
    state = gio.recipe_state({k: tuple(p.shape) for k, p in model.named_parameters()}, seed)
    with torch.no_grad():
        for k, p in model.named_parameters():
            p.copy_(torch.from_numpy(state[k]))
    mean_y, std_y = gio.recipe_normalisation(L)
    model.set_normalization(gio.MEAN_X.astype(np.float32), gio.STD_X.astype(np.float32), mean_y, std_y)
    x, z = gio.recipe_inputs(shape, seed + 1)
    cot = gio.recipe_cotangent(shape, L, seed + 2)
    x, z, cot = torch.from_numpy(x), torch.from_numpy(z), torch.from_numpy(cot)
    dx = dy = 48e3
    # the reference's float32 run: forward and input VJP (its own rounding envelope)
    x32, z32 = x.float().requires_grad_(True), z.float().requires_grad_(True)
    y32 = model(x32, z32, dx, dy)
    xb32, zb32 = torch.autograd.grad(y32, (x32, z32), cot.float())
    torch.set_default_dtype(torch.float64)
    m64 = model.double()
    xr, zr = x.clone().requires_grad_(True), z.clone().requires_grad_(True)
    y64 = m64(xr, zr, dx, dy)
    xb, zb = torch.autograd.grad(y64, (xr, zr), cot)
    y64 = y64.detach()
    env32 = (y32.detach().double() - y64).abs().max().item()
    env_xbar32 = ((xb32.double() - xb).abs().max() / xb.abs().max()).item()
    fd_index, fd_value = np.zeros(0, np.int64), np.zeros(0)
    if fd_pairs:
        rng = np.random.default_rng(seed + 3)
        fd_index = rng.choice(x.numel(), size=fd_pairs, replace=False).astype(np.int64)
        flat = x.reshape(-1)
        vals = []
        with torch.no_grad():
            for i in fd_index:
                xp, xm = flat.clone(), flat.clone()
                xp[i] += FD_EPS
                xm[i] -= FD_EPS
                jp = float((m64(xp.reshape(x.shape), z, dx, dy) * cot).sum())
                jm = float((m64(xm.reshape(x.shape), z, dx, dy) * cot).sum())
                vals.append((jp - jm) / (2 * FD_EPS))
        fd_value = np.array(vals)
    torch.set_default_dtype(torch.float32)
    meta = dict(config=config, seed=seed, shape=list(shape), dx=dx, dy=dy, digest=gio.recipe_digest(state),
                env32=env32, env_xbar32=env_xbar32, fd_eps=FD_EPS)
    np.savez_compressed(os.path.join(HERE, f"{name}.npz"), meta=json.dumps(meta), y64=y64.numpy(),
                        xbar=xb.numpy(), zbar=zb.numpy(), fd_index=fd_index, fd_value=fd_value)
    print(f"{name}: out {tuple(y64.shape)}, reference fp32 vs fp64 max |d| = {env32:.2e}, x_bar rel {env_xbar32:.2e}"
          f", {fd_pairs} FD pairs, {time.time() - t0:.0f} s")


if __name__ == "__main__":
    ap = argparse.ArgumentParser()
    ap.add_argument("--reference")
    ap.add_argument("--only", nargs="*")
    args = ap.parse_args()
    for name, case in CASES.items():
        if not args.only or name in args.only:
            run_case(name, *case)
    if not args.only or "head" in args.only:
        head_case()
    for name, case in RECIPE_CASES.items():
        if not args.only or name in args.only:
            run_recipe_case(name, *case)
