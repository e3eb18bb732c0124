"""Shape-constant tables of the two spectral operators, built in float64 on the host and uploaded once (cached by the
executor):

- the real DFT matrices that turn rfft2/irfft2 over (H, W) into contractions (SpectralConv2dFull.forward,
  models/ffno_model.py:441-448);
- the Filon height-transform weights, the inverse phases, mode factors, the column taper and the live-mode count of
  HeightSpectralConv (models/ffno_model.py:37-64, 226-309);
- the frequency-MLP outputs g(k), U(k), V(k) of both operators at the cube's wavenumbers (:346-365, :375-429, :212-220,
  :231-237, :282-300).

Everything here runs once per distinct (shape, spacing, height grid, weights); nothing here is on the per-voxel path.
"""
import math

import numpy as np
import torch
import torch.nn.functional as F


# ------------------------------------------------------------------------------------------------ horizontal DFT
def _angle(n_idx, k_idx, n):
    """2 pi (n k mod n) / n, reduced exactly in integers."""
    return 2.0 * math.pi * (np.outer(k_idx, n_idx) % n) / n


def plane_dft(H, W):
    """Real matrices of rfft2 / irfft2 over one (H, W) plane, float64:
    twf [2Wf][W]   Z = rfft_W(x):          re rows kw, then im rows kw
    thf [2H][2H]   X = fft_H(Z) on [Zre; Zim]
    thi [2H][2H]   P = ifft_H(Y) (no 1/H)
    twi [W][2Wf]   y = c2r_W(P) / (H W), imaginary parts of the DC and Nyquist bins ignored (as irfft2 does)."""
    Wf = W // 2 + 1
    a = _angle(np.arange(W), np.arange(Wf), W)          # [Wf][W]
    twf = np.concatenate([np.cos(a), -np.sin(a)], 0)
    b = _angle(np.arange(H), np.arange(H), H)           # [kh][h]
    c, s = np.cos(b), np.sin(b)
    thf = np.block([[c, s], [-s, c]])
    thi = np.block([[c.T, -s.T], [s.T, c.T]])
    weight = np.full(Wf, 2.0)
    weight[0] = 1.0
    if W % 2 == 0:
        weight[-1] = 1.0
    a2 = _angle(np.arange(Wf), np.arange(W), W)          # [w][kw]
    twi = np.concatenate([np.cos(a2) * weight, -np.sin(a2) * weight], 1) / (H * W)
    return twf, thf, thi, twi


def plane_features(H, W, dx, dy):
    """[H*Wf, 4] frequency-MLP input (k_features, models/ffno_model.py:375-392), float64."""
    ky = torch.fft.fftfreq(H, d=dy, dtype=torch.float64)
    kx = torch.fft.rfftfreq(W, d=dx, dtype=torch.float64)
    ky, kx = torch.meshgrid(ky, kx, indexing="ij")
    ky, kx = ky * 1e5, kx * 1e5
    return torch.stack([kx, ky, torch.sqrt(kx ** 2 + ky ** 2 + 1e-12), torch.sign(ky)], -1).reshape(-1, 4)


# ------------------------------------------------------------------------------------------------ height operator
def base_wavenumbers(modes, length):
    """k_m = 2 pi m / L, rounded as the reference's float32 buffer is (models/ffno_model.py:226)."""
    return (2 * math.pi * torch.arange(modes, dtype=torch.float32) / length).double()


def height_box(span, reference_length, min_wavelength, modes):
    """(length, k [M] float64 of float32-rounded values) for columns whose largest span is `span`
    (HeightSpectralConv.box, models/ffno_model.py:248-259)."""
    if 2 * span <= reference_length:
        return reference_length, base_wavenumbers(modes, reference_length)
    length = 2 * span
    m = int(math.floor(length / min_wavelength)) + 1
    return length, base_wavenumbers(m, length)


def height_features(k, feature_wavelength):
    q = k * feature_wavelength / (2 * math.pi)
    t = q / (1 + q)
    return torch.stack([t, t * t], -1)


def lower_median(values):
    """torch.median's value: the lower of the two middle elements."""
    v = np.sort(np.asarray(values, dtype=np.float64))
    return v[(len(v) - 1) // 2]


def taper(column, k):
    """1 up to 2 pi / (3 dz), half cosine to 0 at pi / dz (HeightSpectralConv.cutoff, models/ffno_model.py:239-246).
    Exactly 0 from the Nyquist wavenumber up."""
    col = np.asarray(column, dtype=np.float64)
    if len(col) < 2:
        raise ValueError("the height operator needs at least two levels")
    dz = lower_median(np.abs(np.diff(col)))
    kn = math.pi / dz
    u = np.clip((k.numpy() - 2 * kn / 3) / (kn / 3), 0.0, 1.0)
    return 0.5 * (1 + np.cos(math.pi * u))


def filon(z, k):
    """Filon weights (q_re, q_im) [..., D, M] of piecewise-linear columns z [..., D] at wavenumbers k [M], float64
    (height_fourier_weights, models/ffno_model.py:37-64): sum_j x_j q_jm = integral of x(z) e^{-i k_m z} dz."""
    z = np.asarray(z, dtype=np.float64)
    k = np.asarray(k, dtype=np.float64)
    za, zb = z[..., :-1, None], z[..., 1:, None]
    lo = np.minimum(za, zb)
    h = np.abs(zb - za)
    th = h * k
    small = np.abs(th) < 1e-2
    t = np.where(small, 1.0, th)
    c, s = np.cos(t), np.sin(t)
    # R = int_0^1 u e^{-i th u} du ; Lw = int_0^1 (1 - u) e^{-i th u} du
    r_re = np.where(small, 0.5 - th ** 2 / 8, (c + t * s - 1) / t ** 2)
    r_im = np.where(small, -th / 3 + th ** 3 / 30, (t * c - s) / t ** 2)
    l_re = np.where(small, 0.5 - th ** 2 / 24, s / t - r_re)
    l_im = np.where(small, -th / 6 + th ** 3 / 120, (c - 1) / t - r_im)
    ph = lo * k
    e_re, e_im = h * np.cos(ph), -h * np.sin(ph)
    lo_re, lo_im = e_re * l_re - e_im * l_im, e_re * l_im + e_im * l_re
    hi_re, hi_im = e_re * r_re - e_im * r_im, e_re * r_im + e_im * r_re
    up = za <= zb
    a_re, a_im = np.where(up, lo_re, hi_re), np.where(up, lo_im, hi_im)
    b_re, b_im = np.where(up, hi_re, lo_re), np.where(up, hi_im, lo_im)
    shape = z.shape + (len(k),)
    q_re, q_im = np.zeros(shape), np.zeros(shape)
    q_re[..., :-1, :] += a_re
    q_im[..., :-1, :] += a_im
    q_re[..., 1:, :] += b_re
    q_im[..., 1:, :] += b_im
    return q_re, q_im


def column_tapers(columns, k):
    """taper() for many columns [ncol, D] at once: [ncol, M]."""
    cols = np.asarray(columns, dtype=np.float64)
    dz = np.sort(np.abs(np.diff(cols, axis=-1)), axis=-1)[..., (cols.shape[-1] - 2) // 2]
    kn = math.pi / dz[..., None]
    u = np.clip((k.numpy()[None] - 2 * kn / 3) / (kn / 3), 0.0, 1.0)
    return 0.5 * (1 + np.cos(math.pi * u))


def percolumn_tables(z_raw, length, k):
    """Per-column tables when the columns' height grids differ (the reference's non-shared path,
    models/ffno_model.py:276-280, 306-308): z_raw [ncol, D] heights of each column (unshifted). Returns live modes M'
    (the largest live count over the columns), tzf [ncol][2M'][D] and tzi [ncol][D][2M'] with each column's own
    taper, float64. The executor builds these tables on the device (ffno_percol_tables); this host statement is what
    the kernel is tested against."""
    z = np.asarray(z_raw, dtype=np.float64)
    z = z - z.min(axis=-1, keepdims=True)
    tap = column_tapers(z, k)
    live = max(1, int((tap > 0).sum(axis=-1).max()))
    kk = k.numpy()[:live]
    q_re, q_im = filon(z, kk)                                   # [ncol, D, M']
    factor = np.full(live, 2.0)
    factor[0] = 1.0
    f = factor[None] * tap[:, :live] / length                   # [ncol, M']
    ph = z[..., None] * kk                                      # [ncol, D, M']
    tzf = np.concatenate([q_re.transpose(0, 2, 1), q_im.transpose(0, 2, 1)], axis=1)
    tzi = np.concatenate([np.cos(ph) * f[:, None], -np.sin(ph) * f[:, None]], axis=2)
    return live, tzf, tzi


def percolumn_prep(z_raw, length, k):
    """What the per-column table kernels (ffno_percol_tables / _vjp) take besides the heights: live modes M' (the
    largest live count over the columns), f [ncol][M'] = factor * taper / length per column and mode, df [ncol][M'] =
    d f / d dz (dz the column's median spacing: the taper's only dependence on the heights) and med [ncol] (int32), the
    index of the median spacing as torch.median returns it (the index autograd differentiates through), float64."""
    z = np.asarray(z_raw, dtype=np.float64)
    z = z - z.min(axis=-1, keepdims=True)           # spacings of the shifted heights, bit for bit as autograd sees them
    sp = torch.from_numpy(np.abs(z[..., 1:] - z[..., :-1]))
    dz_t, med = sp.median(dim=-1)
    dz = dz_t.numpy()[:, None]
    kk = k.numpy()[None]
    kn = math.pi / dz
    u_raw = (kk - 2 * kn / 3) / (kn / 3)
    u = np.clip(u_raw, 0.0, 1.0)
    tap = 0.5 * (1 + np.cos(math.pi * u))
    live = max(1, int((tap > 0).sum(axis=-1).max()))
    factor = np.full(live, 2.0)
    factor[0] = 1.0
    f = factor[None] * tap[:, :live] / length
    # d tap / d dz = -pi/2 sin(pi u) * du/d dz with du/d dz = 3 k / pi where the clamp passes (0 <= u_raw <= 1)
    inside = (u_raw >= 0.0) & (u_raw <= 1.0)
    dtap = np.where(inside, -0.5 * math.pi * np.sin(math.pi * u) * 3 * kk / math.pi, 0.0)
    df = factor[None] * dtap[:, :live] / length
    return live, np.ascontiguousarray(f), np.ascontiguousarray(df), med.numpy().astype(np.int32)


def height_tables(column, length, k):
    """For a shared column (heights shifted to start at 0) and box (length, k):
    live modes M' (taper > 0), forward table tzf [2M'][D] (q_re rows, then q_im rows) and inverse tzi [D][2M']
    (cos, -sin, each scaled by mode factor * taper / length), float64."""
    tap = taper(column, k)
    live = int(np.count_nonzero(tap > 0))
    live = max(live, 1)
    kk = k.numpy()[:live]
    q_re, q_im = filon(column, kk)
    factor = np.full(live, 2.0)
    factor[0] = 1.0
    f = factor * tap[:live] / length
    ph = np.asarray(column, dtype=np.float64)[:, None] * kk[None]
    tzf = np.concatenate([q_re.T, q_im.T], 0)
    tzi = np.concatenate([np.cos(ph) * f, -np.sin(ph) * f], 1)
    return live, tzf, tzi


# ------------------------------------------------------------------------------------------------ frequency MLPs
def freq_tables(params, prefix, features, rank):
    """g [F][2], U [F][C][rank], V [F][rank][C] from the frequency MLPs of one operator, float64. params maps the
    reference's parameter names to tensors."""
    p = lambda n: params[f"{prefix}.{n}"].detach().double().cpu()
    lin = lambda n, v: F.linear(v, p(n + ".weight"), p(n + ".bias"))
    x = features.double()
    g = lin("freq_mlp.4", F.gelu(lin("freq_mlp.2", F.gelu(lin("freq_mlp.0", x)))))
    if not rank:
        return g, None, None
    h = F.gelu(lin("freq_lowrank.2", F.gelu(lin("freq_lowrank.0", x))))
    n = x.shape[0]
    u = lin("freq_u", h).reshape(n, -1, rank)
    v = lin("freq_v", h).reshape(n, rank, -1)
    return g, u, v


# ------------------------------------------------------------------------------------------------ table adjoint
def _filon_torch(z, k):
    """filon() in torch float64 (differentiable in z), columns z [..., D]."""
    za, zb = z[..., :-1, None], z[..., 1:, None]
    lo = torch.minimum(za, zb)
    h = (zb - za).abs()
    th = h * k
    small = th.abs() < 1e-2
    t = torch.where(small, torch.ones_like(th), th)
    c, s = torch.cos(t), torch.sin(t)
    r_re = torch.where(small, 0.5 - th ** 2 / 8, (c + t * s - 1) / t ** 2)
    r_im = torch.where(small, -th / 3 + th ** 3 / 30, (t * c - s) / t ** 2)
    l_re = torch.where(small, 0.5 - th ** 2 / 24, s / t - r_re)
    l_im = torch.where(small, -th / 6 + th ** 3 / 120, (c - 1) / t - r_im)
    ph = lo * k
    e_re, e_im = h * torch.cos(ph), -h * torch.sin(ph)
    lo_re, lo_im = e_re * l_re - e_im * l_im, e_re * l_im + e_im * l_re
    hi_re, hi_im = e_re * r_re - e_im * r_im, e_re * r_im + e_im * r_re
    up = za <= zb
    a_re, a_im = torch.where(up, lo_re, hi_re), torch.where(up, lo_im, hi_im)
    b_re, b_im = torch.where(up, hi_re, lo_re), torch.where(up, hi_im, lo_im)
    pad_end, pad_start = (0, 0, 0, 1), (0, 0, 1, 0)
    return (F.pad(a_re, pad_end) + F.pad(b_re, pad_start), F.pad(a_im, pad_end) + F.pad(b_im, pad_start))


def percolumn_tables_vjp(z_raw, length, k, live, tzf_bar, tzi_bar):
    """Gradient w.r.t. z_raw [ncol, D] of percolumn_tables along (tzf_bar [ncol][2M'][D], tzi_bar [ncol][D][2M']),
    by float64 autograd: each column's shift by its minimum, Filon weights, phases and taper. The executor runs this
    gradient on the device (ffno_percol_tables_vjp); this host statement is what the kernel is tested against."""
    with torch.enable_grad():
        zr = torch.as_tensor(np.asarray(z_raw, dtype=np.float64)).requires_grad_(True)
        z = zr - zr.amin(dim=-1, keepdim=True)
        kk = k[:live].double()
        dz = (z[..., 1:] - z[..., :-1]).abs().median(dim=-1).values[..., None]
        kn = math.pi / dz
        u = ((kk - 2 * kn / 3) / (kn / 3)).clamp(0, 1)
        tap = 0.5 * (1 + torch.cos(math.pi * u))                  # [ncol, M']
        factor = torch.full((live,), 2.0, dtype=torch.float64)
        factor[0] = 1.0
        f = factor * tap / length
        q_re, q_im = _filon_torch(z, kk)                          # [ncol, D, M']
        ph = z[..., None] * kk
        tzf = torch.cat([q_re.transpose(1, 2), q_im.transpose(1, 2)], 1)
        tzi = torch.cat([torch.cos(ph) * f[:, None], -torch.sin(ph) * f[:, None]], 2)
        loss = (tzf * torch.as_tensor(tzf_bar)).sum() + (tzi * torch.as_tensor(tzi_bar)).sum()
        (g,) = torch.autograd.grad(loss, zr)
    return g.numpy()


def height_tables_vjp(column_raw, length, k, live, tzf_bar, tzi_bar):
    """Gradient w.r.t. the raw (unshifted) shared column of heights [D] of the height tables (tzf, tzi) along
    (tzf_bar [2M'][D], tzi_bar [D][2M']), by autograd through the float64 table builder: the column shift by its
    minimum, the Filon weights, the inverse phases and the taper's median spacing (models/ffno_model.py:37-64,
    239-246, 266-275, 302-305)."""
    with torch.enable_grad():
        return _height_tables_vjp(column_raw, length, k, live, tzf_bar, tzi_bar)


def _height_tables_vjp(column_raw, length, k, live, tzf_bar, tzi_bar):
    col_raw = torch.as_tensor(np.asarray(column_raw, dtype=np.float64)).requires_grad_(True)
    col = col_raw - col_raw.amin()
    kk = k[:live].double()
    dz = (col[1:] - col[:-1]).abs().median(dim=-1).values
    kn = math.pi / dz
    u = ((kk - 2 * kn / 3) / (kn / 3)).clamp(0, 1)
    tap = 0.5 * (1 + torch.cos(math.pi * u))
    factor = torch.full((live,), 2.0, dtype=torch.float64)
    factor[0] = 1.0
    f = factor * tap / length
    q_re, q_im = _filon_torch(col, kk)
    ph = col[:, None] * kk[None]
    tzf = torch.cat([q_re.t(), q_im.t()], 0)
    tzi = torch.cat([torch.cos(ph) * f, -torch.sin(ph) * f], 1)
    (g,) = torch.autograd.grad((tzf * torch.as_tensor(tzf_bar)).sum() + (tzi * torch.as_tensor(tzi_bar)).sum(),
                               col_raw)
    return g.numpy()
