"""ORACLE — test infrastructure only, never the product path.

A CPU restatement of the reference FFNO3D forward pass (harshmathur1990/FFNOML, models/ffno_model.py) and of the
service runtime's unit conversions (ffno_fsdp_runtime.py), written as plain functions over a state dict of tensors, in
whatever floating type the caller picks: float64 is the parity oracle, float32 is the CPU baseline that bench.py times.
The input VJP is torch.autograd through these functions.

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline / reference arms may import this module; the
ffnoml_gb300 package never does.

Parity of this restatement with the reference itself is pinned by tests/test_oracle_golden.py against the fixtures in
tests/golden/, which tests/golden/make_golden.py produced by running the reference's own FFNO3D (float64) in this
container.
"""
import math

import torch
import torch.nn.functional as F
from torch.utils.checkpoint import checkpoint

# MULTI3D constants in cgs, as the reference takes them (models/ffno_model.py:111-112)
EE, HH, EM, BK, PI_M3D = 1.602189e-12, 6.626176e-27, 9.109534e-28, 1.380662e-16, 3.14159265359
LN_CCON = math.log(0.5 * (HH / math.sqrt(2.0 * PI_M3D * EM) / math.sqrt(BK)) ** 3)

# service unit conversions (ffno_fsdp_runtime.py:44-46)
Z_METRES_PER_MODEL_UNIT = 1.0e6
VELOCITY_M_S_PER_MODEL_UNIT = 1.0e3
LOG10_POPULATION_LIMIT = 37.0


# ----------------------------------------------------------------------------------------------------------------------
# small helpers
# ----------------------------------------------------------------------------------------------------------------------
def group_count(channels, max_groups=8):
    """Largest divisor of channels not above max_groups (models/ffno_model.py:21-25)."""
    g = min(max_groups, channels)
    while g > 1 and channels % g:
        g -= 1
    return g


def pointwise(x, weight, bias=None):
    """1x1x1 Conv3d, the reference's channel mixing (nn.Conv3d(..., 1))."""
    return F.conv3d(x, weight, bias)


def lte_tables(atom, levels):
    """Per level: ln(g_i/g_1), E_i [eV], Debye multiple ndxi(ion_i), ion_i - ion_1 (models/ffno_model.py:116-128,
    MULTI3D calc_lte_populations)."""
    g = [float(v) for v in atom["g"]]
    ev = [float(v) for v in atom["ev"]]
    ion = [int(v) for v in atom["ion"]]
    if not (len(g) == len(ev) == len(ion) == levels):
        raise ValueError("multi3d_lte atom data does not match the level count")
    stage = [0] * 21
    for i in range(2, 21):
        stage[i] = stage[i - 1] + i - 1
    base = stage[ion[0]]
    # MULTI3D subtracts ndxi(ion_1) from every stage in a loop that zeroes ndxi(ion_1) as it passes it, so the stages
    # after ion_1 keep their values and the ones up to ion_1 are shifted (models/ffno_model.py:124-126)
    for i in range(1, 21):
        sub = base if i <= ion[0] else 0
        stage[i] -= sub
    return ([math.log(v / g[0]) for v in g], ev, [float(stage[i]) for i in ion], [float(max(i - ion[0], 0)) for i in ion])


def lte_log_weights(log10_t, log10_ne, tables):
    """ln of MULTI3D's LTE level weights in float64 (models/ffno_model.py:131-141). log10_t, log10_ne: [B, ...]."""
    log_g, ev, ndxi, dion = tables
    t = torch.pow(10.0, log10_t.double())[:, None]
    ne = torch.pow(10.0, log10_ne.double() - 6.0)[:, None]
    shape = (1, -1) + (1,) * (t.dim() - 2)
    tab = lambda v: torch.tensor(v, dtype=torch.float64).view(shape)
    conl = LN_CCON + torch.log(ne) - 1.5 * torch.log(t)
    dxi = 4.98e-4 * 5040.0 / t * torch.sqrt(ne * BK * t)
    return tab(log_g) - (EE / BK) / t * (tab(ev) - dxi * tab(ndxi)) - tab(dion) * conl


# ----------------------------------------------------------------------------------------------------------------------
# height geometry (models/ffno_model.py:28-74, 231-259)
# ----------------------------------------------------------------------------------------------------------------------
def trapezoid(z):
    """|dz| trapezoid weights along dim 2 of z [B, 1, D, H, W] (models/ffno_model.py:28-34)."""
    if z.shape[2] == 1:
        return torch.ones_like(z)
    half = 0.5 * (z[:, :, 1:] - z[:, :, :-1]).abs()
    return F.pad(half, (0, 0, 0, 0, 0, 1)) + F.pad(half, (0, 0, 0, 0, 1, 0))


def level_weights(z_scale):
    """Each level's share of its column's height, normalised to mean 1 per column (models/ffno_model.py:67-74)."""
    if z_scale.ndim == 4:
        z_scale = z_scale.unsqueeze(1)
    w = trapezoid(z_scale)
    return w / w.mean(dim=2, keepdim=True).clamp_min(1e-12)


def filon_weights(z, k):
    """Filon weights q_jm with sum_j x_j q_jm = integral of the piecewise-linear x(z) exp(-i k_m z) dz
    (models/ffno_model.py:37-64). z [..., D], k [M] -> (re, im) each [..., D, M]."""
    z0, z1 = z[..., :-1, None], z[..., 1:, None]
    bottom = torch.minimum(z0, z1)
    h = (z1 - z0).abs()
    th = h * k
    near0 = th.abs() < 1e-2
    ts = torch.where(near0, torch.ones_like(th), th)
    co, si = torch.cos(ts), torch.sin(ts)
    # integrals over the unit segment of u e^{-i th u} (up) and (1-u) e^{-i th u} (down)
    up_re = torch.where(near0, 0.5 - th ** 2 / 8, (co + ts * si - 1) / ts ** 2)
    up_im = torch.where(near0, -th / 3 + th ** 3 / 30, (ts * co - si) / ts ** 2)
    full_re, full_im = si / ts, (co - 1) / ts
    dn_re = torch.where(near0, 0.5 - th ** 2 / 24, full_re - up_re)
    dn_im = torch.where(near0, -th / 6 + th ** 3 / 120, full_im - up_im)
    ph = bottom * k
    sc_re, sc_im = h * torch.cos(ph), -h * torch.sin(ph)
    low_re, low_im = sc_re * dn_re - sc_im * dn_im, sc_re * dn_im + sc_im * dn_re
    high_re, high_im = sc_re * up_re - sc_im * up_im, sc_re * up_im + sc_im * up_re
    ascending = z0 <= z1
    a_re, a_im = torch.where(ascending, low_re, high_re), torch.where(ascending, low_im, high_im)
    b_re, b_im = torch.where(ascending, high_re, low_re), torch.where(ascending, high_im, low_im)
    return (F.pad(a_re, (0, 0, 0, 1)) + F.pad(b_re, (0, 0, 1, 0)),
            F.pad(a_im, (0, 0, 0, 1)) + F.pad(b_im, (0, 0, 1, 0)))


def base_wavenumbers(modes, reference_length):
    """k_m = 2 pi m / L built in float32 as the reference's buffer is (models/ffno_model.py:226)."""
    return 2 * math.pi * torch.arange(modes, dtype=torch.float32) / reference_length


def height_box(z_scale, reference_length, min_wavelength, base_k, dtype):
    """(length, k, mode factors) for these columns (models/ffno_model.py:248-259)."""
    span = float((z_scale.amax(dim=-3) - z_scale.amin(dim=-3)).max().detach())
    if 2 * span <= reference_length:
        k = base_k.to(dtype)
        length = reference_length
    else:
        length = 2 * span
        modes = int(math.floor(length / min_wavelength)) + 1
        k = 2 * math.pi * torch.arange(modes, dtype=dtype) / length
    factor = torch.full((k.numel(),), 2.0, dtype=dtype)
    factor[0] = 1.0
    return length, k, factor


def height_features(k, feature_wavelength):
    """[M, 2] frequency-MLP input t, t^2 with t = q/(1+q), q = k lambda_f / 2 pi (models/ffno_model.py:231-237)."""
    q = k * feature_wavelength / (2 * math.pi)
    t = q / (1 + q)
    return torch.stack([t, t * t], dim=-1)


def column_taper(columns, k):
    """Half-cosine taper from 2 pi/(3 dz) to pi/dz, dz the median spacing (models/ffno_model.py:239-246)."""
    dz = (columns[..., 1:] - columns[..., :-1]).abs().median(dim=-1).values[..., None]
    k_nyq = math.pi / dz
    u = ((k - 2 * k_nyq / 3) / (k_nyq / 3)).clamp(0, 1)
    return 0.5 * (1 + torch.cos(math.pi * u))


def plane_features(H, W, dx, dy, dtype):
    """[H, Wf, 4] horizontal frequency-MLP input (models/ffno_model.py:375-392, 443-446)."""
    ky = torch.fft.fftfreq(H, d=dy, dtype=dtype)
    kx = torch.fft.rfftfreq(W, d=dx, dtype=dtype)
    ky, kx = torch.meshgrid(ky, kx, indexing="ij")
    ky, kx = ky * 1e5, kx * 1e5
    return torch.stack([kx, ky, torch.sqrt(kx ** 2 + ky ** 2 + 1e-12), torch.sign(ky)], dim=-1)


# ----------------------------------------------------------------------------------------------------------------------
# the oracle model
# ----------------------------------------------------------------------------------------------------------------------
class OracleFFNO3D:
    """The reference FFNO3D as functions of a state dict. `state` holds the reference's state_dict entries (names of
    models/ffno_model.py); `config` the constructor's keyword arguments (species included)."""

    def __init__(self, state, config, dtype=torch.float64, checkpoint_blocks=False):
        self.dtype = dtype
        self.p = {k: torch.as_tensor(v).to(dtype) for k, v in state.items()}
        self.c = dict(config)
        self.width = int(config["width"])
        self.n_layers = int(config["n_layers"])
        self.rank = int(config.get("freq_mix_rank", 8))
        self.ref_len = float(config.get("z_reference_length", 40.0))
        self.min_wl = float(config.get("z_min_wavelength", 0.04))
        self.feat_wl = float(config.get("z_feature_wavelength", 0.3))
        self.modes = int(math.floor(self.ref_len / self.min_wl)) + 1
        self.base_k = base_wavenumbers(self.modes, self.ref_len)
        self.species = config["species"]
        self.levels = [int(s["levels"]) for s in self.species]
        self.total_bound = float(config.get("total_bound", 6.0))
        self.rho_ch = int(config.get("rho_channel", 5))
        self.t_ch = int(config.get("temperature_channel", 0))
        self.ne_ch = int(config.get("ne_channel", 4))
        tabs = [lte_tables(s["multi3d_lte"], s["levels"]) for s in self.species]
        self.tables = tuple([v for t in tabs for v in t[i]] for i in range(4))
        self.groups = group_count(self.width)
        self.checkpoint_blocks = checkpoint_blocks

    # -- parts ---------------------------------------------------------------------------------------------------------
    def _mlp(self, prefix, x, act_last=None):
        """Two 1x1 convs with GELU between: Sequential indices 0 and 2, or 0 and 3 for PointwiseMLP, whose index 2
        is its (identity) dropout (models/ffno_model.py:147-160)."""
        p = self.p
        second = prefix + (".3" if prefix + ".3.weight" in p else ".2")
        h = F.gelu(pointwise(x, p[prefix + ".0.weight"]))
        y = pointwise(h, p[second + ".weight"], p.get(second + ".bias"))
        return torch.sigmoid(y) if act_last == "sigmoid" else y

    def _wgn(self, prefix, x, w, eps=1e-5):
        """Depth-weighted GroupNorm (models/ffno_model.py:77-95)."""
        B, C = x.shape[:2]
        G = self.groups
        g = x.reshape(B, G, C // G, *x.shape[2:])
        wg = w.unsqueeze(1)
        dims = tuple(range(2, g.dim()))
        total = (wg * torch.ones_like(g)).sum(dim=dims, keepdim=True)
        mean = (wg * g).sum(dim=dims, keepdim=True) / total
        var = (wg * (g - mean) ** 2).sum(dim=dims, keepdim=True) / total
        y = ((g - mean) * torch.rsqrt(var + eps)).reshape_as(x)
        shape = (1, C) + (1,) * (x.dim() - 2)
        return y * self.p[prefix + ".weight"].view(shape) + self.p[prefix + ".bias"].view(shape)

    def _freq_tables(self, prefix, feats):
        p = self.p
        lin = lambda name, v: F.linear(v, p[f"{prefix}.{name}.weight"], p[f"{prefix}.{name}.bias"])
        gate = lin("freq_mlp.4", F.gelu(lin("freq_mlp.2", F.gelu(lin("freq_mlp.0", feats)))))
        if not self.rank:
            return gate, None, None
        h = F.gelu(lin("freq_lowrank.2", F.gelu(lin("freq_lowrank.0", feats))))
        return gate, lin("freq_u", h), lin("freq_v", h)

    def spectral(self, prefix, x, dx, dy):
        """SpectralConv2dFull.forward (models/ffno_model.py:431-450) with mix_spectrum (:394-429)."""
        p = self.p
        B, C, D, H, W = x.shape
        xg = x * self._mlp(prefix + ".input_gate", x, "sigmoid")
        xf = torch.fft.rfft2(xg, dim=(-2, -1))
        feats = plane_features(H, W, float(dx), float(dy), self.dtype)
        gate, u, v = self._freq_tables(prefix, feats)
        wc = torch.complex(p[prefix + ".weight_real"], p[prefix + ".weight_imag"])           # [Cin, Cout]
        g = torch.complex(gate[..., 0], gate[..., 1])                                     # [H, Wf]
        out = torch.einsum("bidyx,io->bodyx", xf, wc) * g
        if self.rank:
            u = u.reshape(H, W // 2 + 1, C, self.rank).to(xf.dtype)
            v = v.reshape(H, W // 2 + 1, self.rank, C).to(xf.dtype)
            out = out + torch.einsum("brdyx,yxor->bodyx", torch.einsum("bidyx,yxri->brdyx", xf, v), u)
        y = torch.fft.irfft2(out, s=(H, W), dim=(-2, -1))
        return self._mlp(prefix + ".post", y)

    def vertical(self, prefix, x, z_scale):
        """HeightSpectralConv.forward (models/ffno_model.py:261-309)."""
        p = self.p
        if z_scale.ndim == 4:
            z_scale = z_scale.unsqueeze(1)
        length, k, factor = height_box(z_scale, self.ref_len, self.min_wl, self.base_k, self.dtype)
        M = k.numel()
        xg = x * self._mlp(prefix + ".input_gate", x, "sigmoid") + pointwise(z_scale, p[prefix + ".z_proj.weight"])
        z = z_scale - z_scale.amin(dim=2, keepdim=True)
        shared = bool((z == z[..., :1, :1]).all()) and bool((z == z[:1]).all())
        if shared:
            col = z[0, 0, :, 0, 0]
            q_re, q_im = filon_weights(col, k)
            ph = col[:, None] * k
            x_re = torch.einsum("bcdhw,dm->bcmhw", xg, q_re)
            x_im = torch.einsum("bcdhw,dm->bcmhw", xg, q_im)
            taper = column_taper(col, k)[:, None, None]
        else:
            cols = z[:, 0].permute(0, 2, 3, 1)
            q_re, q_im = filon_weights(cols, k)
            ph = z[:, 0, ..., None] * k
            x_re = torch.einsum("bcdhw,bhwdm->bcmhw", xg, q_re)
            x_im = torch.einsum("bcdhw,bhwdm->bcmhw", xg, q_im)
            taper = column_taper(cols, k).permute(0, 3, 1, 2)[:, None]
        gate, u, v = self._freq_tables(prefix, height_features(k, self.feat_wl))
        wr, wi = p[prefix + ".weight_real"], p[prefix + ".weight_imag"]
        a_re = torch.einsum("bimhw,io->bomhw", x_re, wr) - torch.einsum("bimhw,io->bomhw", x_im, wi)
        a_im = torch.einsum("bimhw,io->bomhw", x_im, wr) + torch.einsum("bimhw,io->bomhw", x_re, wi)
        gr, gi = gate[:, 0, None, None], gate[:, 1, None, None]
        y_re, y_im = a_re * gr - a_im * gi, a_re * gi + a_im * gr
        if self.rank:
            u = u.reshape(M, -1, self.rank)
            v = v.reshape(M, self.rank, -1)
            y_re = y_re + torch.einsum("brmhw,mor->bomhw", torch.einsum("bimhw,mri->brmhw", x_re, v), u)
            y_im = y_im + torch.einsum("brmhw,mor->bomhw", torch.einsum("bimhw,mri->brmhw", x_im, v), u)
        f = factor[:, None, None] * taper
        y_re, y_im = y_re * f, y_im * f
        if shared:
            y = torch.einsum("bomhw,dm->bodhw", y_re, torch.cos(ph)) - torch.einsum("bomhw,dm->bodhw", y_im, torch.sin(ph))
        else:
            y = (torch.einsum("bomhw,bdhwm->bodhw", y_re, torch.cos(ph))
                 - torch.einsum("bomhw,bdhwm->bodhw", y_im, torch.sin(ph)))
        return self._mlp(prefix + ".post", y / length)

    def block(self, i, x, z_scale, dx, dy):
        """FFNOBlock3dBalanced.forward, eval mode (models/ffno_model.py:524-553)."""
        pre = f"blocks.{i}"
        p = self.p
        w = level_weights(z_scale)
        spec = F.gelu(self._wgn(pre + ".norm_spec", self.spectral(pre + ".spec", x, dx, dy), w))
        vert = F.gelu(self._wgn(pre + ".norm_vert", self.vertical(pre + ".vertical", x, z_scale), w))
        gates = self._mlp(pre + ".branch_gate", torch.cat([x, spec, vert], dim=1), "sigmoid")
        sg, vg = gates.chunk(2, dim=1)
        smix, vmix = spec * sg, vert * vg
        fused = self._mlp(pre + ".fuse", torch.cat([smix, vmix], dim=1)) + 0.5 * (smix + vmix)
        fused = F.gelu(self._wgn(pre + ".norm_fuse", fused, w))
        x1 = x + p[pre + ".res_fused"] * fused
        x2 = x1 + p[pre + ".res_pw"] * self._wgn(pre + ".norm_pw", self._mlp(pre + ".pw", x1), w)
        return x2 + p[pre + ".res_mlp"] * self._wgn(pre + ".norm_mlp", self._mlp(pre + ".mlp.net", x2), w)

    def head(self, h, x_in):
        """FFNO3D.head_output (models/ffno_model.py:730-749)."""
        p = self.p
        r, t, e = self.rho_ch, self.t_ch, self.ne_ch
        log10_rho = x_in[:, r] * p["std_X"][r] + p["mean_X"][r]
        lte = lte_log_weights(x_in[:, t].double() * p["std_X"][t].double() + p["mean_X"][t].double(),
                              x_in[:, e].double() * p["std_X"][e].double() + p["mean_X"][e].double(), self.tables)
        outs = []
        c = k = 0
        for s, lv in enumerate(self.levels):
            logits = h[:, c:c + lv].double() + lte[:, k:k + lv]
            frac = (torch.log_softmax(logits, dim=1) / math.log(10.0)).to(h.dtype)
            tot = self.total_bound * torch.tanh(h[:, c + lv] / self.total_bound)
            outs.append((log10_rho - p["log10_particle_mass"][s] + tot)[:, None] + frac)
            c += lv + 1
            k += lv
        y = torch.cat(outs, dim=1)
        return (y - p["mean_Y"][None, :, None, None, None]) / p["std_Y"][None, :, None, None, None]

    def lift(self, x, z_scale):
        """FFNO3D._lift (models/ffno_model.py:782-783): gelu(weighted GroupNorm(lift conv(x)))."""
        return F.gelu(self._wgn("lift.1", pointwise(x, self.p["lift.0.weight"]), level_weights(z_scale)))

    def proj(self, x):
        """The projection of FFNO3D._run_head (models/ffno_model.py:790-798): proj2(gelu(proj1(x)))."""
        p = self.p
        return pointwise(F.gelu(pointwise(x, p["proj1.weight"])), p["proj2.weight"], p["proj2.bias"])

    def forward(self, x, z_scale, dx, dy):
        """FFNO3D.forward (models/ffno_model.py:800-832): normalised inputs -> normalised log10 populations."""
        x_in = x
        use_ckpt = self.checkpoint_blocks and torch.is_grad_enabled()
        x = checkpoint(self.lift, x, z_scale, use_reentrant=False) if use_ckpt else self.lift(x, z_scale)
        for i in range(self.n_layers):
            if use_ckpt:
                x = checkpoint(lambda a, b, i=i: self.block(i, a, b, dx, dy), x, z_scale, use_reentrant=False)
            else:
                x = self.block(i, x, z_scale, dx, dy)
        h = checkpoint(self.proj, x, use_reentrant=False) if use_ckpt else self.proj(x)
        return self.head(h, x_in)

    __call__ = forward

    # -- service level (ffno_fsdp_runtime.py:48-58, 76-78, 265-281) -------------------------------------------------------
    def forward_si(self, features, z_m, dx, dy):
        """SI features (T, vx, vy, vz, log10 ne, log10 rho) [1, 6, D, H, W] and z [1, D, H, W] in metres -> linear
        populations [1, L, D, H, W] in m^-3."""
        p = self.p
        model = torch.cat((torch.log10(features[:, 0:1]), features[:, 1:4] / VELOCITY_M_S_PER_MODEL_UNIT,
                           features[:, 4:6]), dim=1)
        mx, sx = p["mean_X"][None, :, None, None, None], p["std_X"][None, :, None, None, None]
        my, sy = p["mean_Y"][None, :, None, None, None], p["std_Y"][None, :, None, None, None]
        y = self.forward((model - mx) / sx, z_m / Z_METRES_PER_MODEL_UNIT, dx, dy) * sy + my
        return torch.pow(10.0, y.clamp(-LOG10_POPULATION_LIMIT, LOG10_POPULATION_LIMIT))


def vjp(oracle, x, z_scale, dx, dy, cotangent):
    """Input VJP of oracle.forward at (x, z_scale) along cotangent: (y, x_bar, z_bar)."""
    x = x.detach().clone().requires_grad_(True)
    z = z_scale.detach().clone().requires_grad_(True)
    y = oracle.forward(x, z, dx, dy)
    xb, zb = torch.autograd.grad(y, (x, z), cotangent)
    return y.detach(), xb, zb


def jvp(oracle, x, z_scale, dx, dy, x_dot):
    """Forward-mode derivative of oracle.forward at (x, z_scale) along x_dot with the heights fixed (what jvp_local
    computes with dual tensors, ffno_fsdp_runtime.py:350-372): (y, y_dot)."""
    fn = lambda xx: oracle.forward(xx, z_scale, dx, dy)
    return torch.func.jvp(fn, (x,), (x_dot,))


def jvp_si(oracle, features, z_m, dx, dy, feature_tangent):
    """The same at the service level: SI features and their tangent -> (populations, population tangent)."""
    fn = lambda ff: oracle.forward_si(ff, z_m, dx, dy)
    return torch.func.jvp(fn, (features,), (feature_tangent,))
