"""The reference's own known answers for the level-fraction head (its tests/test_level_fraction_head.py), restated
against the oracle (oracle/ffno_oracle.py) on the reference's seeded initialisation (the drop-in module's, which
tests/test_module_cpu.py pins): any target within the total bound is reproduced exactly, a fresh model's total is
rho / mass, populations stay finite in float32 with the total at its bound, and only rho moves the total."""
import math

import numpy as np
import torch

from ffnoml_gb300 import FFNO3D
from golden_io import ATOMS
from oracle.ffno_oracle import OracleFFNO3D, lte_log_weights

BASE = dict(in_channels=6, width=16, n_layers=2, hidden_spectral=16, hidden_vertical=16)
MEAN_X = np.array([3.8, 0.0, 0.0, 0.0, 16.0, -7.0], np.float32)
STD_X = np.array([0.4, 5.0, 5.0, 5.0, 2.0, 2.5], np.float32)


def fraction_oracle(atoms, seed=3, dtype=torch.float64, total_bias=None):
    species = [ATOMS[a] for a in atoms]
    out = sum(s["levels"] for s in species)
    cfg = dict(out_channels=out, species=species, **BASE)
    torch.manual_seed(seed)
    module = FFNO3D(**cfg)
    module.set_normalization(MEAN_X, STD_X, np.linspace(10.0, 15.0, out), np.linspace(1.0, 2.0, out))
    state = {k: v.clone() for k, v in module.state_dict().items()}
    if total_bias is not None:
        state["proj2.bias"][species[0]["levels"]] = total_bias
    return OracleFFNO3D(state, cfg, dtype)


def inputs(shape=(1, 6, 24, 11, 9), seed=5):
    torch.manual_seed(seed)
    x = torch.randn(*shape)
    z = torch.linspace(14.0, -1.0, shape[2])[:, None, None].repeat(1, *shape[3:])[None].repeat(shape[0], 1, 1, 1)
    return x, z


def log10_populations(o, y):
    return y * o.p["std_Y"][None, :, None, None, None] + o.p["mean_Y"][None, :, None, None, None]


def log10_reference_total(o, x, s):
    return x[:, 5] * o.p["std_X"][5] + o.p["mean_X"][5] - o.p["log10_particle_mass"][s]


def test_any_target_within_the_bound_is_reproduced_exactly():
    # totals from -3.16 to +5.40 dex about rho / mass, level ratios over 30 dex
    o = fraction_oracle(["H", "CA"])
    torch.manual_seed(11)
    x = torch.randn(1, 6, 5, 4, 3, dtype=torch.float64)
    offsets = torch.tensor([-3.16, -0.5, -0.021, 0.0, 1.93, 5.40], dtype=torch.float64)
    lte = lte_log_weights(x[:, 0] * o.p["std_X"][0] + o.p["mean_X"][0], x[:, 4] * o.p["std_X"][4] + o.p["mean_X"][4],
                          o.tables)
    log10_n = torch.empty(1, 12, 5, 4, 3, dtype=torch.float64)
    head = torch.empty(1, 14, 5, 4, 3, dtype=torch.float64)
    for sp in (0, 1):
        ratios = torch.randn(1, 6, 5, 4, 3, dtype=torch.float64) * 6.0
        frac = ratios - torch.logsumexp(ratios * math.log(10.0), 1, keepdim=True) / math.log(10.0)
        s = offsets[torch.randint(0, 6, (1, 5, 4, 3))]
        log10_n[:, 6 * sp:6 * sp + 6] = log10_reference_total(o, x, sp)[:, None] + s[:, None] + frac
        head[:, 7 * sp:7 * sp + 6] = ratios * math.log(10.0) - lte[:, 6 * sp:6 * sp + 6]
        head[:, 7 * sp + 6] = o.total_bound * torch.atanh(s / o.total_bound)
    y = log10_populations(o, o.head(head, x))
    assert (y - log10_n).abs().max().item() < 1e-9


def test_total_starts_at_rho_over_mass():
    o = fraction_oracle(["H", "CA"])
    x, z = inputs()
    with torch.no_grad():
        log10_n = log10_populations(o, o.forward(x.double(), z.double(), 48e3, 48e3))
    for sp in (0, 1):
        total = torch.logsumexp(log10_n[:, 6 * sp:6 * sp + 6] * math.log(10.0), 1) / math.log(10.0)
        assert (total - log10_reference_total(o, x.double(), sp)).abs().max().item() < 1e-5
    assert o.p["proj2.weight"].shape[0] == 14


def test_populations_stay_finite_in_float32():
    o = fraction_oracle(["H"], dtype=torch.float32, total_bias=1e6)       # the total correction at its bound
    x, z = inputs()
    with torch.no_grad():
        y = log10_populations(o, o.forward(x, z, 48e3, 48e3))
    assert torch.isfinite(torch.pow(10.0, y)).all()
    assert (y.max() - (log10_reference_total(o, x, 0).max() + 6.0)).item() < 1e-3


def test_only_rho_moves_a_fresh_models_total():
    o = fraction_oracle(["H"])
    x, z = inputs((1, 6, 6, 5, 4))
    x = x.double().requires_grad_(True)
    y = log10_populations(o, o.forward(x, z.double(), 48e3, 48e3))
    total = torch.logsumexp(y * math.log(10.0), dim=1) / math.log(10.0)
    (g,) = torch.autograd.grad(total.sum(), x)
    assert (g[:, 5] - o.p["std_X"][5]).abs().max().item() < 1e-4
    assert g[:, :5].abs().max().item() < 1e-4
