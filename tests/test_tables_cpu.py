"""Host-built tables of the spectral operators: the real DFT matrices reproduce rfft2/irfft2 (including the
non-Hermitian half spectra that the mixing produces), the height tables equal the oracle's Filon weights, taper and
phases, and the table adjoint matches finite differences."""
import math

import numpy as np
import pytest
import torch

from ffnoml_gb300 import tables as tb
from oracle import ffno_oracle as orc


@pytest.mark.parametrize("H,W", [(8, 12), (7, 9), (6, 2), (16, 16)])
def test_plane_dft_reproduces_rfft2_and_irfft2(H, W):
    Wf = W // 2 + 1
    twf, thf, thi, twi = tb.plane_dft(H, W)
    g = torch.Generator().manual_seed(H * 100 + W)
    x = torch.randn(H, W, dtype=torch.float64, generator=g)
    z = np.einsum("kw,hw->hk", twf, x.numpy())                      # [H][2Wf]
    zr = np.concatenate([z[:, :Wf], z[:, Wf:]], 0)                   # [2H][Wf]
    X = thf @ zr
    ref = torch.fft.rfft2(x).numpy()
    assert np.abs(X[:H] - ref.real).max() < 1e-10 and np.abs(X[H:] - ref.imag).max() < 1e-10
    Y = torch.randn(H, Wf, dtype=torch.complex128, generator=g)   # a non-Hermitian half spectrum, as mixing makes
    P = thi @ np.concatenate([Y.real.numpy(), Y.imag.numpy()], 0)
    y = np.einsum("wk,hk->hw", twi, np.concatenate([P[:H], P[H:]], 1))
    assert np.abs(y - torch.fft.irfft2(Y, s=(H, W)).numpy()).max() < 1e-10


@pytest.mark.parametrize("kind", ["uniform", "stretched"])
def test_height_tables_match_oracle(kind):
    D = 40
    if kind == "uniform":
        col = torch.linspace(14.0, -1.0, D, dtype=torch.float64)
    else:
        s = torch.linspace(0.0, 1.0, D, dtype=torch.float64)
        col = (-1.0 + 15.0 * (0.4 * s + 0.6 * s ** 2)).flip(0)
    col = col - col.min()
    k = orc.base_wavenumbers(1001, 40.0).double()
    live, tzf, tzi = tb.height_tables(col.numpy(), 40.0, k)
    taper = orc.column_taper(col, k)
    assert live == int((taper > 0).sum()) and bool((taper[live:] == 0).all())
    q_re, q_im = orc.filon_weights(col, k[:live])
    assert np.abs(tzf[:live].T - q_re.numpy()).max() < 1e-12
    assert np.abs(tzf[live:].T - q_im.numpy()).max() < 1e-12
    f = torch.cat([torch.ones(1), 2 * torch.ones(live - 1)]).double() * taper[:live] / 40.0
    ph = col[:, None] * k[None, :live]
    assert np.abs(tzi[:, :live] - (torch.cos(ph) * f).numpy()).max() < 1e-12
    assert np.abs(tzi[:, live:] + (torch.sin(ph) * f).numpy()).max() < 1e-12


def test_height_table_adjoint_matches_finite_differences():
    D = 12
    s = np.linspace(0.0, 1.0, D)
    col = (-1.0 + 15.0 * (0.4 * s + 0.6 * s ** 2))[::-1].copy()
    k = orc.base_wavenumbers(134, 40.0).double()
    live, tzf, tzi = tb.height_tables(col - col.min(), 40.0, k)
    rng = np.random.default_rng(0)
    a, b = rng.normal(size=tzf.shape), rng.normal(size=tzi.shape)
    g = tb.height_tables_vjp(col, 40.0, k, live, a, b)

    def f(c):
        _, p, q = tb.height_tables(c - c.min(), 40.0, k)
        return (p * a).sum() + (q * b).sum()

    for j in (1, 5, 9):
        e = np.zeros(D)
        e[j] = 1e-6
        fd = (f(col + e) - f(col - e)) / 2e-6
        assert abs(fd - g[j]) < 1e-5 * max(1.0, abs(fd))


def test_tall_columns_take_a_longer_box():
    length, k = tb.height_box(15.0, 20.0, 0.5, 41)
    assert abs(length - 30.0) < 1e-12 and k.numel() == 61
    length, k = tb.height_box(9.0, 20.0, 0.5, 41)
    assert length == 20.0 and k.numel() == 41


@pytest.mark.parametrize("ion", [[1, 1, 2], [2, 2, 3], [1, 2, 3], [3, 3, 4], [2, 3, 5]])
def test_lte_level_tables_match_the_oracle(ion):
    from ffnoml_gb300 import lte
    atom = dict(g=[2.0, 8.0, 1.0], ev=[0.0, 10.2, 13.6], ion=ion)
    assert lte.tables(atom, 3) == orc.lte_tables(atom, 3)


def test_lte_level_tables_refuse_a_level_count_mismatch():
    from ffnoml_gb300 import lte
    with pytest.raises(ValueError):
        lte.tables(dict(g=[2.0, 1.0], ev=[0.0, 13.6], ion=[1, 2]), 3)
