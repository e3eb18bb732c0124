"""The reference's own known answers for the level-fraction head (its tests/test_level_fraction_head.py), restated
against the oracle (oracle/ffno_oracle.py) on the reference's seeded initialisation (the drop-in module's, which
tests/test_module_cpu.py pins): any target within the total bound is reproduced exactly, a fresh model's total is
rho / mass, populations stay finite in float32 with the total at its bound, and only rho moves the total; and from
its tests/test_departure_coefficients.py, zero departure gives MULTI3D's LTE level fractions (checked against an
independent float64 statement of calc_lte_populations) and level 2 follows Boltzmann in temperature."""
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


# ---------------------------------------------------------------------------------------------------------------------
# zero departure = MULTI3D's LTE (the reference's tests/test_departure_coefficients.py)
# ---------------------------------------------------------------------------------------------------------------------
def lte_fractions(t, ne_cm3, atom):
    """MULTI3D calc_lte_populations' n*_i / sum n*, in numpy float64 (an independent statement of the published
    algorithm: Saha-Boltzmann relative to the ground level with Debye lowering of the ionisation energies)."""
    q_e, h, m_e, k_b = 1.602189e-12, 6.626176e-27, 9.109534e-28, 1.380662e-16
    g, ev, ion = atom["g"], atom["ev"], atom["ion"]
    stage = [0] * 21                       # lowering multiple of each ionisation stage, shifted to the ground's
    for i in range(2, 21):
        stage[i] = stage[i - 1] + (i - 1)
    for i in range(1, 21):                 # the shift zeroes stage[ion_1] as it passes, as MULTI3D's loop does
        stage[i] -= stage[ion[0]]
    saha = np.log(0.5 * (h / math.sqrt(2.0 * 3.14159265359 * m_e) / math.sqrt(k_b)) ** 3 * ne_cm3) - 1.5 * np.log(t)
    lowering = 4.98e-4 * 5040.0 / t * np.sqrt(ne_cm3 * k_b * t)
    rel = [np.ones_like(t)]
    for i in range(1, len(g)):
        ln_rel = math.log(g[i] / g[0]) - (q_e / k_b) / t * (ev[i] - lowering * stage[ion[i]])
        rel.append(np.exp(ln_rel - (ion[i] - ion[0]) * saha))
    rel = np.stack(rel)
    return rel / rel.sum(0)


def solar_inputs(shape=(1, 6, 24, 11, 9), seed=5):
    """Normalised inputs whose T and ne span 2,000-60,000 K and 10^14-10^23 m^-3, independently."""
    g = torch.Generator().manual_seed(seed)
    x = torch.randn(*shape, generator=g)
    span = math.log10(6e4) - math.log10(2000.0)
    log10_t = math.log10(2000.0) + span * torch.rand(shape[0], *shape[2:], generator=g)
    log10_ne = 14.0 + 9.0 * torch.rand(shape[0], *shape[2:], generator=g)
    x[:, 0] = (log10_t - float(MEAN_X[0])) / float(STD_X[0])
    x[:, 4] = (log10_ne - float(MEAN_X[4])) / float(STD_X[4])
    z = torch.linspace(14.0, -1.0, shape[2])[:, None, None].repeat(1, *shape[3:])[None].repeat(shape[0], 1, 1, 1)
    return x, z


def zero_delta_oracle(atoms):
    o = fraction_oracle(atoms)
    c = 0
    for lv in o.levels:
        o.p["proj2.weight"][c:c + lv] = 0.0
        o.p["proj2.bias"][c:c + lv] = 0.0
        c += lv + 1
    return o


def test_zero_departure_gives_multi3d_lte_fractions():
    o = zero_delta_oracle(["H", "CA"])
    x, z = solar_inputs()
    with torch.no_grad():
        log10_n = log10_populations(o, o.forward(x.double(), z.double(), 48e3, 48e3))
    t = 10.0 ** (x[0, 0].double() * float(STD_X[0]) + float(MEAN_X[0])).numpy()
    ne_cm3 = 10.0 ** ((x[0, 4].double() * float(STD_X[4]) + float(MEAN_X[4])).numpy() - 6.0)
    for sp, atom in enumerate((ATOMS["H"]["multi3d_lte"], ATOMS["CA"]["multi3d_lte"])):
        n = log10_n[0, 6 * sp:6 * sp + 6]
        got = (n - torch.logsumexp(n * math.log(10.0), 0) / math.log(10.0)).numpy()
        expected = np.log10(np.maximum(lte_fractions(t, ne_cm3, atom), 1e-300))
        usable = expected > -37.0
        assert usable.mean() > 0.5
        assert np.abs(got - expected)[usable].max() < 2e-5


def test_level_2_follows_boltzmann_in_temperature():
    # at zero departure d log10(n2/n1) / d log10 T = (e/k) E_2 / T (times std_X[0] for the normalised input)
    o = zero_delta_oracle(["H"])
    x, z = solar_inputs((1, 6, 6, 5, 4))
    x = x.double().requires_grad_(True)
    y = log10_populations(o, o.forward(x, z.double(), 48e3, 48e3))
    (g,) = torch.autograd.grad((y[:, 1] - y[:, 0]).sum(), x)
    t = 10.0 ** (x.detach()[:, 0] * float(STD_X[0]) + float(MEAN_X[0])).numpy()
    expected = (1.602189e-12 / 1.380662e-16) * ATOMS["H"]["multi3d_lte"]["ev"][1] / t * float(STD_X[0])
    assert g[:, 1:].abs().max().item() < 1e-6 * np.abs(expected).max()
    assert np.abs(g[:, 0].numpy() - expected).max() / np.abs(expected).max() < 1e-4


def test_kernel_saha_constant_matches_its_formula():
    """The kernels carry MULTI3D's Saha constant as a literal; it is the formula's value (the oracle evaluates it
    with math.log and math.sqrt)."""
    import os
    import re
    from oracle.ffno_oracle import LN_CCON
    src = open(os.path.join(os.path.dirname(__file__), "..", "ffnoml_gb300", "csrc", "common.cuh")).read()
    m = re.search(r"kLN_CCON = (-?[0-9.eE+-]+);", src)
    assert m is not None
    assert abs(float(m.group(1)) - LN_CCON) <= 4e-16 * abs(LN_CCON)
