"""Executor of the FFNO3D forward pass (and, in executor_bwd, its input VJP) on one GPU.

It packs the module's weights into device buffers in the kernels' layouts (once per weight version), keeps the
shape-constant tables resident (DFT matrices per (H, W); frequency-MLP tables per (H, W, dx, dy); height tables per
height grid), and issues the C-ABI kernels of libffnoml_gb300 on the current CUDA stream.

Per cube (batch element), the block is (FFNOBlock3dBalanced.forward, models/ffno_model.py:536-553):
  xs = gate_s(x); xv = gate_v(x) + z_proj z
  spec_pre = post_s(irfft2(mix_s(rfft2(xs))))                       -> GroupNorm statistics
  vert_pre = post_v(iDFT_z(mix_v(DFT_z(xv))))                       -> GroupNorm statistics
  fused_pre = fuse(gate([x, gelu(GN spec_pre), gelu(GN vert_pre)]))   -> statistics
  x1 = x + r_f gelu(GN fused_pre); pw_pre = pw(x1)                    -> statistics
  x2 = x1 + r_pw GN(pw_pre);      mlp_pre = mlp(x2)                   -> statistics
  out = x2 + r_mlp GN(mlp_pre)
"""
import math

import numpy as np
import torch

from . import _native as nat
from . import tables as tb

EPS = 1e-5  # nn.GroupNorm default, DepthWeightedGroupNorm's eps (models/ffno_model.py:77-95)
SUPPORTED_WIDTHS = (16, 32, 64, 96)


def _ptr(t):
    return None if t is None else t.data_ptr()


def _stream():
    return torch.cuda.current_stream().cuda_stream


def _conv_t(conv):
    """Conv3d weight [out, in, 1, 1, 1] -> row-major [in][out] float32."""
    return conv.weight.detach()[:, :, 0, 0, 0].t().contiguous().float()


def _wbig(wr, wi):
    """[[w_re, w_im], [-w_im, w_re]] for out = xhat (w_re + i w_im) on [re | im] rows."""
    wr, wi = wr.detach().float(), wi.detach().float()
    return torch.cat([torch.cat([wr, wi], 1), torch.cat([-wi, wr], 1)], 0).contiguous()


class Packed:
    """Device copies of one model's weights in kernel layouts."""

    def __init__(self, model, device):
        self.device = device
        C = model.width
        dev = lambda t: t.to(device=device, dtype=torch.float32).contiguous()
        self.lift_w = dev(model.lift[0].weight.detach()[:, :, 0, 0, 0].t())          # [cin][C]
        self.lift_g, self.lift_b = dev(model.lift[1].weight.detach()), dev(model.lift[1].bias.detach())
        self.groups = model.lift[1].num_groups
        self.blocks = []
        for b in model.blocks:
            s, v = b.spec, b.vertical
            pk = dict(
                s_g1=dev(_conv_t(s.input_gate[0])), s_g2=dev(_conv_t(s.input_gate[2])),
                s_wbig=dev(_wbig(s.weight_real, s.weight_imag)),
                s_p1=dev(_conv_t(s.post[0])), s_p2=dev(_conv_t(s.post[2])),
                v_g1=dev(_conv_t(v.input_gate[0])), v_g2=dev(_conv_t(v.input_gate[2])),
                v_zp=dev(v.z_proj.weight.detach().reshape(C)),
                v_wbig=dev(_wbig(v.weight_real, v.weight_imag)),
                v_p1=dev(_conv_t(v.post[0])), v_p2=dev(_conv_t(v.post[2])),
                bg1=dev(_conv_t(b.branch_gate[0])), bg2=dev(_conv_t(b.branch_gate[2])),
                bgb=dev(b.branch_gate[2].bias.detach()),
                f1=dev(_conv_t(b.fuse[0])), f2=dev(_conv_t(b.fuse[2])),
                pw1=dev(_conv_t(b.pw[0])), pw2=dev(_conv_t(b.pw[2])),
                m1=dev(_conv_t(b.mlp.net[0])), m2=dev(_conv_t(b.mlp.net[3])),
            )
            for n in ("spec", "vert", "fuse", "pw", "mlp"):
                norm = getattr(b, "norm_" + n)
                pk[n + "_g"] = dev(norm.weight.detach())
                pk[n + "_b"] = dev(norm.bias.detach())
            pk["res"] = (float(b.res_fused.detach()), float(b.res_pw.detach()), float(b.res_mlp.detach()))
            self.blocks.append(pk)
        nh = model.proj2.out_channels
        self.nh = nh
        self.nhp = 16 if nh <= 16 else 32
        if nh > 32:
            raise ValueError("at most 32 head channels are supported")
        self.p1 = dev(_conv_t(model.proj1))
        p2 = torch.zeros(2 * C, self.nhp)
        p2[:, :nh] = _conv_t(model.proj2)
        self.p2 = dev(p2)
        b2 = torch.zeros(self.nhp)
        b2[:nh] = model.proj2.bias.detach().float()
        self.b2 = dev(b2)
        self.head = self._head_params(model)
        # host copies of the parameters the frequency MLPs need (tables are built in float64 on the host)
        self.freq_params = {k: v.detach().cpu() for k, v in model.state_dict().items()
                            if ".freq_" in k}

    @staticmethod
    def _head_params(model):
        hp = nat.HeadParams()
        levels = model.species_levels
        if len(levels) > nat.FFNO_MAX_SPECIES or sum(levels) > nat.FFNO_MAX_LEVELS:
            raise ValueError("too many species or levels for the head kernel")
        if model.in_channels > 8:
            raise ValueError("at most 8 input channels are supported")
        hp.nspecies = len(levels)
        for i, lv in enumerate(levels):
            hp.levels[i] = lv
            hp.log10_particle_mass[i] = float(model.log10_particle_mass[i])
        hp.rho_channel, hp.temperature_channel, hp.ne_channel = (model.rho_channel, model.temperature_channel,
                                                                 model.ne_channel)
        hp.in_channels = model.in_channels
        hp.total_bound = model.total_bound
        for i in range(model.in_channels):
            hp.mean_x[i] = float(model.mean_X[i])
            hp.std_x[i] = float(model.std_X[i])
        for i in range(model.out_channels):
            hp.mean_y[i] = float(model.mean_Y[i])
            hp.std_y[i] = float(model.std_Y[i])
        lg, ev, nd, di = model.lte_tables
        for i in range(len(lg)):
            hp.log_g[i], hp.ev[i], hp.ndxi[i], hp.dion[i] = lg[i], ev[i], nd[i], di[i]
        return hp


def _weights_key(model):
    items = [(t.data_ptr(), t._version) for t in model.parameters()]
    items += [(t.data_ptr(), t._version) for t in model.buffers()]
    return tuple(items)


class Executor:
    def __init__(self, model):
        self.model = model
        self._packed = None
        self._packed_key = None
        self._plane = {}
        self._plane_freq = {}
        self._height = {}

    # -------------------------------------------------------------------------------------------- caches
    def packed(self, device):
        key = (_weights_key(self.model), str(device))
        if self._packed_key != key:
            self._packed = Packed(self.model, device)
            self._packed_key = key
            self._plane_freq.clear()
            self._height.clear()
        return self._packed

    def plane(self, H, W, device):
        key = (H, W, str(device))
        if key not in self._plane:
            twf, thf, thi, twi = tb.plane_dft(H, W)
            f = lambda a: torch.as_tensor(a, dtype=torch.float32, device=device).contiguous()
            self._plane[key] = (f(twf), f(thf), f(thi), f(twi))
        return self._plane[key]

    def plane_freq(self, pk, H, W, dx, dy, device):
        key = (H, W, float(dx), float(dy))
        if key not in self._plane_freq:
            feats = tb.plane_features(H, W, dx, dy)
            rank = self.model.freq_mix_rank
            per_block = []
            for i in range(self.model.n_layers):
                g, u, v = tb.freq_tables(pk.freq_params, f"blocks.{i}.spec", feats, rank)
                per_block.append(self._upload_freq(g, u, v, device))
            self._plane_freq[key] = per_block
        return self._plane_freq[key]

    def height(self, pk, column, length, k, device):
        key = (column.tobytes(), float(length), k.numel())
        if key not in self._height:
            live, tzf, tzi = tb.height_tables(column, length, k)
            feats = tb.height_features(k[:live], self.model.z_feature_wavelength)
            rank = self.model.freq_mix_rank
            per_block = []
            for i in range(self.model.n_layers):
                g, u, v = tb.freq_tables(pk.freq_params, f"blocks.{i}.vertical", feats, rank)
                per_block.append(self._upload_freq(g, u, v, device))
            f = lambda a: torch.as_tensor(a, dtype=torch.float32, device=device).contiguous()
            self._height[key] = (live, f(tzf), f(tzi), per_block)
        return self._height[key]

    @staticmethod
    def _upload_freq(g, u, v, device):
        f = lambda a: None if a is None else a.to(device=device, dtype=torch.float32).contiguous()
        return f(g), f(u), f(v)

    # -------------------------------------------------------------------------------------------- geometry
    def geometry(self, z_scale):
        """Per-batch height analysis: (shared, span, column of sample 0 shifted to 0 as float64 numpy)."""
        B, D = z_scale.shape[0], z_scale.shape[1]
        HW = z_scale.shape[2] * z_scale.shape[3]
        info = torch.empty(B, 2, dtype=torch.float32, device=z_scale.device)
        s = _stream()
        for b in range(B):
            nat.call("ffno_column_info", z_scale[b].data_ptr(), D, HW, info[b].data_ptr(), s)
        col = z_scale[:, :, 0, 0]                                   # [B, D]
        host = torch.cat([info.reshape(-1), col.reshape(-1)]).cpu()
        info_h = host[:2 * B].reshape(B, 2)
        cols = host[2 * B:].reshape(B, D).double().numpy()
        shared_each = bool((info_h[:, 0] > 0.5).all())
        span = float(info_h[:, 1].view(torch.float32).max()) if B else 0.0
        shifted = cols - cols.min(axis=1, keepdims=True)
        shared = shared_each and bool((shifted == shifted[:1]).all())
        return shared, span, shifted[0]

    def box(self, span):
        m = self.model
        modes = int(math.floor(m.z_reference_length / m.z_min_wavelength)) + 1
        return tb.height_box(span, m.z_reference_length, m.z_min_wavelength, modes)

    # -------------------------------------------------------------------------------------------- forward
    def forward(self, x, z_scale, dx, dy):
        """x [B, Cin, D, H, W], z_scale [B, D, H, W] (Mm), float32 CUDA -> [B, L, D, H, W] float32."""
        m = self.model
        if not x.is_cuda:
            raise RuntimeError("ffnoml_gb300 runs on CUDA tensors only")
        if x.dtype != torch.float32 or z_scale.dtype != torch.float32:
            raise TypeError("ffnoml_gb300 FFNO3D takes float32 inputs")
        if m.width not in SUPPORTED_WIDTHS:
            raise ValueError(f"width {m.width} is not supported (supported: {SUPPORTED_WIDTHS})")
        B, Cin, D, H, W = x.shape
        if Cin != m.in_channels:
            raise ValueError(f"expected {m.in_channels} input channels, got {Cin}")
        device = x.device
        pk = self.packed(device)
        x = x.contiguous()
        z_scale = z_scale.contiguous()
        shared, span, column = self.geometry(z_scale)
        if not shared:
            raise NotImplementedError("per-column height grids are not supported by the GB300 path yet")
        length, k = self.box(span)
        hgt = self.height(pk, column, length, k, device)
        pln = self.plane(H, W, device)
        pfr = self.plane_freq(pk, H, W, dx, dy, device)
        out = torch.empty(B, m.out_channels, D, H, W, dtype=torch.float32, device=device)
        for b in range(B):
            self._forward_cube(pk, x[b], z_scale[b], out[b], D, H, W, hgt, pln, pfr)
        return out

    def _forward_cube(self, pk, xin, z, out, D, H, W, hgt, pln, pfr):
        m = self.model
        C = m.width
        V = D * H * W
        HW = H * W
        Wf = W // 2 + 1
        dev = xin.device
        s = _stream()
        lib = nat.lib()
        nparts = lib.ffno_stats_parts(V)
        G = pk.groups
        f32 = dict(dtype=torch.float32, device=dev)
        buf = lambda *shape: torch.empty(*shape, **f32)
        dw = buf(V)
        nat.call("ffno_depth_weights", z.data_ptr(), D, HW, dw.data_ptr(), s)
        partials = torch.empty(nparts * G * 3, dtype=torch.float64, device=dev)
        coefs = {n: buf(3 * C) for n in ("lift", "spec", "vert", "fuse", "pw", "mlp")}

        x = buf(V, C)
        pre = buf(V, C)
        nat.call("ffno_lift_fwd", xin.data_ptr(), m.in_channels, V, C, pk.lift_w.data_ptr(), dw.data_ptr(),
                 pre.data_ptr(), partials.data_ptr(), nparts, G, s)
        nat.call("ffno_gn_finalize", partials.data_ptr(), nparts, C, G, pk.lift_g.data_ptr(), pk.lift_b.data_ptr(),
                 EPS, coefs["lift"].data_ptr(), None, s)
        nat.call("ffno_gn_act", pre.data_ptr(), coefs["lift"].data_ptr(), V, C, 1, x.data_ptr(), s)

        live, tzf, tzi, hfreq = hgt
        twf, thf, thi, twi = pln
        spec_len = D * 2 * H * Wf * C
        sa, sb_ = buf(spec_len), buf(spec_len)
        xs, xv, y = buf(V, C), buf(V, C), buf(V, C)
        va, vb = buf(2 * live * HW * C), buf(2 * live * HW * C)
        spec_pre, vert_pre, fused_pre, pw_pre, mlp_pre = (buf(V, C) for _ in range(5))
        x1, x2 = buf(V, C), buf(V, C)
        descs = self._descs(D, H, W, C, live)
        for i, bp in enumerate(pk.blocks):
            # ---- input gates
            nat.call("ffno_gate_fwd", x.data_ptr(), V, C, bp["s_g1"].data_ptr(), bp["s_g2"].data_ptr(), None, None,
                     xs.data_ptr(), s)
            nat.call("ffno_gate_fwd", x.data_ptr(), V, C, bp["v_g1"].data_ptr(), bp["v_g2"].data_ptr(),
                     bp["v_zp"].data_ptr(), z.data_ptr(), xv.data_ptr(), s)
            # ---- horizontal spectral branch
            g, u, v = pfr[i]
            nat.call("ffno_xform", twf.data_ptr(), xs.data_ptr(), sa.data_ptr(), descs["wf"], 0, s)
            nat.call("ffno_xform", thf.data_ptr(), sa.data_ptr(), sb_.data_ptr(), descs["hf"], 0, s)
            nat.call("ffno_spectral_mix", sb_.data_ptr(), sa.data_ptr(), H * Wf, D, C, 2 * H * Wf * C, H * Wf * C, C,
                     bp["s_wbig"].data_ptr(), g.data_ptr(), _ptr(u), _ptr(v), m.freq_mix_rank, s)
            nat.call("ffno_xform", thi.data_ptr(), sa.data_ptr(), sb_.data_ptr(), descs["hi"], 0, s)
            nat.call("ffno_xform", twi.data_ptr(), sb_.data_ptr(), y.data_ptr(), descs["wi"], 0, s)
            nat.call("ffno_mlp2_fwd", 0, y.data_ptr(), None, None, 0.0, None, V, C, bp["s_p1"].data_ptr(),
                     bp["s_p2"].data_ptr(), dw.data_ptr(), spec_pre.data_ptr(), partials.data_ptr(), nparts, G, s)
            nat.call("ffno_gn_finalize", partials.data_ptr(), nparts, C, G, bp["spec_g"].data_ptr(),
                     bp["spec_b"].data_ptr(), EPS, coefs["spec"].data_ptr(), None, s)
            # ---- vertical (height) branch
            g, u, v = hfreq[i]
            nat.call("ffno_xform", tzf.data_ptr(), xv.data_ptr(), va.data_ptr(), descs["zf"], 0, s)
            nat.call("ffno_spectral_mix", va.data_ptr(), vb.data_ptr(), live, HW, HW * C, C, live * HW * C, C,
                     bp["v_wbig"].data_ptr(), g.data_ptr(), _ptr(u), _ptr(v), m.freq_mix_rank, s)
            nat.call("ffno_xform", tzi.data_ptr(), vb.data_ptr(), y.data_ptr(), descs["zi"], 0, s)
            nat.call("ffno_mlp2_fwd", 0, y.data_ptr(), None, None, 0.0, None, V, C, bp["v_p1"].data_ptr(),
                     bp["v_p2"].data_ptr(), dw.data_ptr(), vert_pre.data_ptr(), partials.data_ptr(), nparts, G, s)
            nat.call("ffno_gn_finalize", partials.data_ptr(), nparts, C, G, bp["vert_g"].data_ptr(),
                     bp["vert_b"].data_ptr(), EPS, coefs["vert"].data_ptr(), None, s)
            # ---- gate + fuse
            nat.call("ffno_fuse_fwd", x.data_ptr(), spec_pre.data_ptr(), coefs["spec"].data_ptr(),
                     vert_pre.data_ptr(), coefs["vert"].data_ptr(), V, C, bp["bg1"].data_ptr(),
                     bp["bg2"].data_ptr(), bp["bgb"].data_ptr(), bp["f1"].data_ptr(), bp["f2"].data_ptr(),
                     dw.data_ptr(), fused_pre.data_ptr(), partials.data_ptr(), nparts, G, s)
            nat.call("ffno_gn_finalize", partials.data_ptr(), nparts, C, G, bp["fuse_g"].data_ptr(),
                     bp["fuse_b"].data_ptr(), EPS, coefs["fuse"].data_ptr(), None, s)
            # ---- residual MLPs
            r_f, r_pw, r_mlp = bp["res"]
            nat.call("ffno_mlp2_fwd", 1, x.data_ptr(), fused_pre.data_ptr(), coefs["fuse"].data_ptr(), r_f,
                     x1.data_ptr(), V, C, bp["pw1"].data_ptr(), bp["pw2"].data_ptr(), dw.data_ptr(),
                     pw_pre.data_ptr(), partials.data_ptr(), nparts, G, s)
            nat.call("ffno_gn_finalize", partials.data_ptr(), nparts, C, G, bp["pw_g"].data_ptr(),
                     bp["pw_b"].data_ptr(), EPS, coefs["pw"].data_ptr(), None, s)
            nat.call("ffno_mlp2_fwd", 2, x1.data_ptr(), pw_pre.data_ptr(), coefs["pw"].data_ptr(), r_pw,
                     x2.data_ptr(), V, C, bp["m1"].data_ptr(), bp["m2"].data_ptr(), dw.data_ptr(),
                     mlp_pre.data_ptr(), partials.data_ptr(), nparts, G, s)
            nat.call("ffno_gn_finalize", partials.data_ptr(), nparts, C, G, bp["mlp_g"].data_ptr(),
                     bp["mlp_b"].data_ptr(), EPS, coefs["mlp"].data_ptr(), None, s)
            nat.call("ffno_resid_out", x2.data_ptr(), mlp_pre.data_ptr(), coefs["mlp"].data_ptr(), r_mlp, V, C,
                     x.data_ptr(), s)
        hp = pk.head
        nat.call("ffno_head_fwd", x.data_ptr(), xin.data_ptr(), V, C, pk.p1.data_ptr(), pk.p2.data_ptr(),
                 pk.b2.data_ptr(), pk.nh, pk.nhp, hp, out.data_ptr(), None, s)

    @staticmethod
    def _descs(D, H, W, C, live):
        Wf = W // 2 + 1
        HW = H * W
        XD = nat.XformDesc
        big = 1 << 30
        d = {}
        # rfft along W: per (d, h) row [W][C] -> [2][Wf] rows of the [D][2][H][Wf][C] spectrum
        d["wf"] = XD(nb=D * H, nb2=H, in_b1=H * W * C, in_b2=W * C, out_b1=2 * H * Wf * C, out_b2=Wf * C,
                     K=W, M=2 * Wf, N=C, in_split=big, in_hi=0, in_lo=C, out_split=Wf, out_hi=H * Wf * C, out_lo=C)
        # complex DFT along H on [2H][Wf*C] per depth
        hd = dict(nb=D, nb2=1, in_b1=2 * H * Wf * C, in_b2=0, out_b1=2 * H * Wf * C, out_b2=0, K=2 * H, M=2 * H,
                  N=Wf * C, in_split=big, in_hi=0, in_lo=Wf * C, out_split=big, out_hi=0, out_lo=Wf * C)
        d["hf"] = XD(**hd)
        d["hi"] = XD(**hd)
        # c2r along W: [2][Wf] rows -> [W][C]
        d["wi"] = XD(nb=D * H, nb2=H, in_b1=2 * H * Wf * C, in_b2=Wf * C, out_b1=H * W * C, out_b2=W * C,
                     K=2 * Wf, M=W, N=C, in_split=Wf, in_hi=H * Wf * C, in_lo=C, out_split=big, out_hi=0, out_lo=C)
        # height transform [D][HW*C] -> [2M'][HW*C] and back
        d["zf"] = XD(nb=1, nb2=1, in_b1=0, in_b2=0, out_b1=0, out_b2=0, K=D, M=2 * live, N=HW * C,
                     in_split=big, in_hi=0, in_lo=HW * C, out_split=big, out_hi=0, out_lo=HW * C)
        d["zi"] = XD(nb=1, nb2=1, in_b1=0, in_b2=0, out_b1=0, out_b2=0, K=2 * live, M=D, N=HW * C,
                     in_split=big, in_hi=0, in_lo=HW * C, out_split=big, out_hi=0, out_lo=HW * C)
        return {k: v for k, v in d.items()}


def ffno_apply(model, x, z_scale, dx, dy):
    """FFNO3D.forward on the GB300 path (autograd-aware once the VJP is registered)."""
    if z_scale.ndim == 5:
        z_scale = z_scale[:, 0]
    dx = _spacing(dx)
    dy = _spacing(dy)
    return model.executor().forward(x, z_scale, dx, dy)


def _spacing(v):
    """_to_spacing_value (models/ffno_model.py:11-18)."""
    if isinstance(v, (float, int)):
        return float(v)
    if torch.is_tensor(v):
        if v.numel() != 1:
            raise ValueError("spacing must be scalar.")
        return float(v.detach().item())
    raise TypeError(f"Unsupported spacing type: {type(v)}")
