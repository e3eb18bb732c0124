"""tables.percolumn_prep, the host half of the per-column height tables: its live count and per-column f agree with
the float64 host tables, its taper derivative df with autograd of the taper in the median spacing, and its median
index with the spacing torch.median picks on the shifted heights."""
import math

import numpy as np
import torch

from ffnoml_gb300 import tables as tb


def _cols(ncol, D, seed):
    g = np.random.default_rng(seed)
    return np.ascontiguousarray(14.0 - np.cumsum(g.uniform(0.25, 0.7, (ncol, D)), axis=1))


def test_live_and_f_match_the_host_tables():
    length = 15.0
    k = torch.arange(0, 40, dtype=torch.float64) * math.pi / length
    cols = _cols(6, 50, 1)
    live, f, _, _ = tb.percolumn_prep(cols, length, k)
    live0, _, tzi = tb.percolumn_tables(cols, length, k)
    assert live == live0
    z = cols - cols.min(axis=1, keepdims=True)
    # tzi[c][j][m] = cos(z_j k_m) f[c][m]: node j = the column's minimum (z = 0) gives f itself
    jmin = np.argmin(cols, axis=1)
    np.testing.assert_allclose(tzi[np.arange(6), jmin, :live], f, rtol=0, atol=1e-15)
    assert z.min() == 0.0


def test_taper_derivative_matches_autograd():
    length = 15.0
    k = torch.arange(0, 40, dtype=torch.float64) * math.pi / length
    cols = _cols(5, 60, 2)
    live, f, df, med = tb.percolumn_prep(cols, length, k)
    assert np.any(df != 0.0) and np.any(df == 0.0)
    z = cols - cols.min(axis=1, keepdims=True)
    sp = np.abs(z[:, 1:] - z[:, :-1])
    dz = torch.tensor(sp[np.arange(5), med], dtype=torch.float64, requires_grad=True)
    kk = k[:live]
    kn = math.pi / dz[:, None]
    u = ((kk - 2 * kn / 3) / (kn / 3)).clamp(0, 1)
    factor = torch.full((live,), 2.0, dtype=torch.float64)
    factor[0] = 1.0
    ft = factor * 0.5 * (1 + torch.cos(math.pi * u)) / length
    np.testing.assert_allclose(ft.detach().numpy(), f, rtol=1e-14, atol=1e-15)
    for m in range(live):
        (g,) = torch.autograd.grad(ft[:, m].sum(), dz, retain_graph=True)
        np.testing.assert_allclose(g.numpy(), df[:, m], rtol=1e-12, atol=1e-14)


def test_median_index_is_torch_median_of_shifted_spacings():
    length = 15.0
    k = torch.arange(0, 10, dtype=torch.float64) * math.pi / length
    cols = np.tile(np.linspace(14.0, -1.0, 33), (3, 1))       # uniform grids: every spacing ties
    _, _, _, med = tb.percolumn_prep(cols, length, k)
    zt = torch.from_numpy(cols)
    zt = zt - zt.amin(dim=-1, keepdim=True)
    assert np.array_equal(med, (zt[:, 1:] - zt[:, :-1]).abs().median(dim=-1).indices.numpy())
