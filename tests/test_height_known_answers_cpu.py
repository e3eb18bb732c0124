"""The reference's own known answers for the height operator (its tests/test_height_operator.py), restated against
the oracle (oracle/ffno_oracle.py) and the host table builders the product uses (ffnoml_gb300/tables.py): Filon
weights exact for piecewise-linear columns and symmetric under flipping the grid, the taper following the column
spacing, frequency features independent of the band limit, the same populations on any vertical grid, the
depth-weighted GroupNorm with unit weights equal to GroupNorm, and the per-column path equal to the shared-grid one."""
import math

import numpy as np
import pytest
import torch

from ffnoml_gb300 import tables as tb
from golden_io import ATOMS
from oracle import ffno_oracle as orc

K = torch.tensor([0.0, 0.7, 5.0, 40.0], dtype=torch.float64)


def uniform(depth):
    return torch.linspace(14.0, -1.0, depth, dtype=torch.float64)


def stretched(depth):
    """Fine low down, coarse higher up, top first like the simulation grids."""
    s = torch.linspace(0.0, 1.0, depth, dtype=torch.float64)
    return (-1.0 + 15.0 * (0.4 * s + 0.6 * s ** 2)).flip(0)


def weights(impl, z, k):
    if impl == "oracle":
        return orc.filon_weights(z, k)
    re, im = tb.filon(z.numpy(), k.numpy())
    return torch.from_numpy(re), torch.from_numpy(im)


@pytest.mark.parametrize("impl", ["oracle", "tables"])
def test_filon_weights_are_exact_for_piecewise_linear_columns(impl):
    z = stretched(30)
    q_re, q_im = weights(impl, z, K)
    trap = orc.trapezoid(z[None, None, :, None, None])[0, 0, :, 0, 0]
    assert (q_re[:, 0] - trap).abs().max().item() < 1e-12
    assert q_im[:, 0].abs().max().item() < 1e-12
    x = 2.0 - 0.3 * z                                       # linear: the integral is exact at every k
    lo, hi = z.min().item(), z.max().item()
    for m, km in enumerate(K[1:].tolist(), start=1):
        f = lambda zz: np.exp(-1j * km * zz) * ((2.0 - 0.3 * zz) / (-1j * km) - (-0.3) / (-1j * km) ** 2)
        exact = f(hi) - f(lo)
        got = complex((x * q_re[:, m]).sum().item(), (x * q_im[:, m]).sum().item())
        assert abs(got - exact) < 1e-9 * max(1.0, abs(exact)), km
    f_re, f_im = weights(impl, z.flip(0), K)
    assert (f_re.flip(0) - q_re).abs().max().item() < 1e-12
    assert (f_im.flip(0) - q_im).abs().max().item() < 1e-12


@pytest.mark.parametrize("impl", ["oracle", "tables"])
@pytest.mark.parametrize("dz", [0.012, 0.02, 0.025, 0.164])
def test_taper_follows_the_column_spacing(impl, dz):
    k = orc.base_wavenumbers(int(math.floor(40.0 / 0.04)) + 1, 40.0).double()    # a 40 Mm box resolving 0.04 Mm
    column = torch.arange(0, 14.0, dz).double()
    taper = orc.column_taper(column, k) if impl == "oracle" else torch.from_numpy(tb.taper(column.numpy(), k))
    wavelength = 2 * math.pi / k[1:]
    assert torch.all(taper[1:][wavelength >= 3 * dz * 1.001] == 1)
    assert torch.all(taper[1:][wavelength <= 2 * dz] < 1e-6)
    assert float(taper[0]) == 1.0


@pytest.mark.parametrize("impl", ["oracle", "tables"])
def test_features_do_not_depend_on_the_band_limit(impl):
    coarse_m, fine_m = int(math.floor(40.0 / 0.3)) + 1, int(math.floor(40.0 / 0.04)) + 1
    if impl == "oracle":
        feats = lambda m: orc.height_features(orc.base_wavenumbers(m, 40.0).double(), 0.3)
    else:
        feats = lambda m: tb.height_features(tb.base_wavenumbers(m, 40.0), 0.3)
    assert torch.allclose(feats(coarse_m), feats(fine_m)[:coarse_m])


def _atmosphere(z, rows=6, columns=5):
    """Six smooth input channels on heights z [D], varying in x and y: [1, 6, D, H, W] and z_scale [1, D, H, W]."""
    y = torch.linspace(0, 2 * np.pi, rows + 1, dtype=torch.float64)[:-1]
    x = torch.linspace(0, 2 * np.pi, columns + 1, dtype=torch.float64)[:-1]
    zz, yy, xx = torch.meshgrid(z, y, x, indexing="ij")
    channels = [torch.tanh((zz - 2.0) / 1.5) + 0.3 * torch.sin(xx) * torch.cos(yy),
                0.5 * torch.sin(zz / 2.0 + xx), 0.5 * torch.cos(zz / 3.0 + yy),
                torch.exp(-((zz - 5.0) / 3.0) ** 2) * torch.cos(xx - yy),
                -zz / 7.0 + 0.2 * torch.sin(yy), -zz / 5.0 + 0.1 * torch.cos(xx)]
    return torch.stack(channels)[None].float().double(), zz[None].float().double()


def test_same_populations_on_any_vertical_grid():
    """The oracle on a 3001-level grid and on three others, compared at the same heights: within 5e-3 of the output
    range, the reference's own bound for its model."""
    from ffnoml_gb300 import FFNO3D
    cfg = dict(in_channels=6, out_channels=6, width=16, n_layers=2, hidden_spectral=16, hidden_vertical=16,
               species=[ATOMS["H"]], z_reference_length=40.0, z_min_wavelength=0.3, z_feature_wavelength=0.3,
               freq_mix_rank=4)
    torch.manual_seed(1)
    module = FFNO3D(**cfg)                                   # the reference's seeded initialisation
    module.set_normalization(np.array([3.8, 0.0, 0.0, 0.0, 16.0, -7.0], np.float32),
                             np.array([0.4, 5.0, 5.0, 5.0, 2.0, 2.5], np.float32), np.zeros(6), np.ones(6))
    oracle = orc.OracleFFNO3D(module.state_dict(), cfg, torch.float64)

    def populations(z):
        x, zs = _atmosphere(z)
        with torch.no_grad():
            return oracle.forward(x, zs, 48e3, 48e3).permute(0, 1, 3, 4, 2)          # depth last

    ref_z = uniform(3001)
    ref = populations(ref_z)
    scale = (ref.max() - ref.min()).item()
    order = torch.argsort(ref_z)
    flat = ref.reshape(-1, ref.shape[-1])[:, order].numpy()
    worst = 0.0
    for z in (uniform(400), stretched(250), stretched(497)):
        want = torch.from_numpy(np.stack([np.interp(z.numpy(), ref_z[order].numpy(), row) for row in flat]))
        got = populations(z).reshape(-1, len(z))
        worst = max(worst, (got - want).abs().max().item() / scale)
    assert worst < 5e-3


def _small_oracle(seed=0):
    from ffnoml_gb300 import FFNO3D
    cfg = dict(in_channels=6, out_channels=6, width=16, n_layers=1, hidden_spectral=16, hidden_vertical=16,
               species=[ATOMS["H"]], z_reference_length=40.0, z_min_wavelength=0.04, z_feature_wavelength=0.3,
               freq_mix_rank=2)
    torch.manual_seed(seed)
    module = FFNO3D(**cfg)
    state = {k: v.clone() for k, v in module.state_dict().items()}
    for k in state:                                           # the low-rank term live, as the reference's test has it
        if ".freq_u." in k:
            state[k] = torch.randn(state[k].shape, generator=torch.Generator().manual_seed(seed + 1)) * 0.1
    return orc.OracleFFNO3D(state, cfg, torch.float64)


def test_weighted_groupnorm_with_unit_weights_is_groupnorm():
    o = _small_oracle()
    x = torch.randn(2, 16, 7, 3, 4, generator=torch.Generator().manual_seed(2), dtype=torch.float64)
    got = o._wgn("lift.1", x, torch.ones(2, 1, 7, 3, 4, dtype=torch.float64))
    want = torch.nn.functional.group_norm(x, o.groups, o.p["lift.1.weight"], o.p["lift.1.bias"], eps=1e-5)
    assert (got - want).abs().max().item() < 1e-12


def test_shared_grid_equals_per_column_path():
    """The height operator on one shared column grid, and on the same grid with one column moved by 1e-9 Mm (which
    takes the per-column path): the same output."""
    o = _small_oracle()
    x = torch.randn(1, 16, 300, 2, 3, generator=torch.Generator().manual_seed(3), dtype=torch.float64)
    z = torch.linspace(6.0, 0.0, 300, dtype=torch.float64)[None, :, None, None].expand(1, 300, 2, 3).clone()
    prefix = "blocks.0.vertical"
    shared = o.vertical(prefix, x, z)
    z[0, 150, 1, 2] += 1e-9
    assert (o.vertical(prefix, x, z) - shared).abs().max().item() < 1e-6
