"""Executor of the FFNO3D forward pass and its input VJP on one GPU.

It packs the module's weights into device buffers in the kernels' layouts (once per weight version), keeps the
shape-constant tables resident (DFT matrices per (H, W); frequency-MLP tables per (H, W, dx, dy); height tables per
height grid), and issues the C-ABI kernels of libffnoml_gb300 on the current CUDA stream.

Per cube (batch element), a block is (FFNOBlock3dBalanced.forward, models/ffno_model.py:536-553):
  xs = gate_s(x); xv = gate_v(x) + z_proj z
  spec_pre = post_s(irfft2(mix_s(rfft2(xs))))                        -> GroupNorm statistics
  vert_pre = post_v(iDFT_z(mix_v(DFT_z(xv))))                        -> GroupNorm statistics
  fused_pre = fuse(gate([x, gelu(GN spec_pre), gelu(GN vert_pre)]))  -> statistics
  x1 = x + r_f gelu(GN fused_pre); pw_pre = pw(x1)                   -> statistics
  x2 = x1 + r_pw GN(pw_pre);      mlp_pre = mlp(x2)                  -> statistics
  out = x2 + r_mlp GN(mlp_pre)

For the input VJP the forward keeps every block's intermediates when they fit in half the free device memory
(cache_states, the default) and the backward consumes them block by block; otherwise (or with cache_states off, as
the service runs it) it keeps only the block inputs and recomputes each block's intermediates before back-propagating
through it (the reference's per-block activation checkpointing, models/ffno_model.py:751-780). Both give the same
bits. Parameter gradients are not computed: the service's VJP discards them (ffno_fsdp_runtime.py:319-344).
"""
import copy
import hashlib
import math
import threading

import numpy as np
import torch

from . import _native as nat
from . import table_store
from . import tables as tb

EPS = 1e-5  # nn.GroupNorm default, DepthWeightedGroupNorm's eps (models/ffno_model.py:77-95)
SUPPORTED_WIDTHS = (16, 32, 64, 96)
MIX_RANK_TC = 8     # low-rank terms the tensor-core mixing carries; larger ranks mix on the FP32 kernel
NORMS = ("spec", "vert", "fuse", "pw", "mlp")


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


def pack_kmajor(w):
    """A [R][K] matrix (a Conv3d weight [out][in]) as BF16 in the tensor-core canonical K-major order: 8 x 8 core
    matrices, each 8 rows x 16 bytes, the K-blocks of one 8-row group adjacent."""
    R, K = w.shape
    if R % 8 or K % 8:
        raise ValueError("tensor-core operands need dimensions that are multiples of 8")
    return w.detach().float().reshape(R // 8, 8, K // 8, 8).permute(0, 2, 1, 3).contiguous().to(torch.bfloat16)


def _w(conv):
    """Conv3d weight as the [out][in] matrix M of out = in @ M^T."""
    return conv.weight.detach()[:, :, 0, 0, 0].float()


def mix_pack(device, m):
    """Split-BF16 pack of a spectral-mixing matrix m [2C out][2C in] (outputs re 0..C-1 then im 0..C-1) with its output
    rows in the order of ffno_spectral_mix_tc's tensor-memory lanes: slot p = 32 q + l holds part l // 16 (re, im) of
    channel 16 q + l % 16."""
    C = m.shape[0] // 2
    perm = [((p % 32) // 16) * C + 16 * (p // 32) + p % 16 for p in range(2 * C)]
    return tc_pack(device, m[perm])


def tc_pack(device, *mats):
    """Split-BF16 packs of matrices [R][K] back to back: per matrix hi = bf16(M) then lo = bf16(M - hi), each in the
    canonical K-major order (the layout the tensor-core kernels bulk-copy into shared memory)."""
    parts = []
    for m in mats:
        m = m.detach().float().cpu()
        hi = m.to(torch.bfloat16)
        lo = (m - hi.float()).to(torch.bfloat16)
        parts += [pack_kmajor(hi.float()).reshape(-1), pack_kmajor(lo.float()).reshape(-1)]
    return torch.cat(parts).to(device).contiguous()


def _split_kmajor(m):
    """hi = bf16(m), lo = bf16(m - hi) of a float64 [R][K] array, each in the canonical K-major order, as one flat
    BF16 tensor (hi then lo)."""
    t = torch.from_numpy(np.ascontiguousarray(m))
    hi = t.to(torch.bfloat16)
    lo = (t - hi.double()).to(torch.bfloat16)
    return torch.cat([pack_kmajor(hi.float()).reshape(-1), pack_kmajor(lo.float()).reshape(-1)])


XFORM_TC_MAX_K = 512     # the longest contraction one tensor-core transform call takes (RT_MAXK in spectral_tc.cu)
XFORM_TC_KCHUNK = 32     # k per block of the streamed table pack (XKC in spectral_tc.cu)


class TcXform:
    """A transform table T [M][K] (float64 numpy) packed for the tensor-core transforms, in slices of at most 256 rows
    and 512 columns (one kernel call each; the column slices of one row slice accumulate into the same output rows):
    per slice the streamed pack of ffno_xform_tc (split-BF16 per 128-row m-tile and 32-wide k-chunk) and, when the
    slice fits in shared memory, the resident pack of ffno_xform_tcr (the whole [Mp][Kp] table as one canonical
    operand, Mp and Kp rounded up to 16). A production height grid (M = 1001: 680 table rows at D = 256) takes both
    kinds of slices."""

    def __init__(self, T, device):
        T = np.asarray(T, dtype=np.float64)
        self.M, self.K = T.shape
        limit = nat.lib().ffno_xform_tcr_max_table_bytes()
        self.slices = []
        for r0 in range(0, self.M, 256):
            rows = min(256, self.M - r0)
            mt = (rows + 127) // 128
            for c0 in range(0, self.K, XFORM_TC_MAX_K):
                cols = min(XFORM_TC_MAX_K, self.K - c0)
                Kp = (cols + 15) // 16 * 16
                pad = np.zeros((mt * 128, Kp))
                pad[:rows, :cols] = T[r0:r0 + rows, c0:c0 + cols]
                parts = [_split_kmajor(pad[t * 128:(t + 1) * 128, k0:min(Kp, k0 + XFORM_TC_KCHUNK)])
                         for t in range(mt) for k0 in range(0, Kp, XFORM_TC_KCHUNK)]
                packed = torch.cat(parts).to(device).contiguous()
                if packed.numel() * 2 != nat.lib().ffno_xform_tc_pack_bytes(rows, cols):
                    raise RuntimeError("transform pack size mismatch")
                res = None
                Mp = (rows + 15) // 16 * 16
                if 4 * Mp * Kp <= limit:
                    res = (_split_kmajor(pad[:Mp]).to(device).contiguous(), Mp, Kp)
                self.slices.append((r0, rows, c0, cols, packed, res))


class Packed:
    """Device copies of one model's weights in kernel layouts (and their transposes for the VJP)."""

    def __init__(self, model, device):
        self.device = device
        C = model.width
        dev = lambda t: t.to(device=device, dtype=torch.float32).contiguous()
        self.lift_w = dev(model.lift[0].weight.detach()[:, :, 0, 0, 0].t())          # [cin][C]
        self.lift_g, self.lift_b = dev(model.lift[1].weight.detach()), dev(model.lift[1].bias.detach())
        self.groups = model.lift[1].num_groups
        self.tc = bool(nat.lib().ffno_tc_width_supported(C)) and self.groups == 8
        # the channel MLPs (the post-MLPs of both branches, pw, mlp) and the input gates also run on tensor cores at
        # width 96
        self.tc_chan = bool(nat.lib().ffno_tc_channel_width_supported(C)) and self.groups == 8
        self.blocks = []
        for b in model.blocks:
            s, v = b.spec, b.vertical
            mats = dict(
                s_g1=_conv_t(s.input_gate[0]), s_g2=_conv_t(s.input_gate[2]),
                s_p1=_conv_t(s.post[0]), s_p2=_conv_t(s.post[2]),
                v_g1=_conv_t(v.input_gate[0]), v_g2=_conv_t(v.input_gate[2]),
                v_p1=_conv_t(v.post[0]), v_p2=_conv_t(v.post[2]),
                bg1=_conv_t(b.branch_gate[0]), bg2=_conv_t(b.branch_gate[2]),
                f1=_conv_t(b.fuse[0]), f2=_conv_t(b.fuse[2]),
                pw1=_conv_t(b.pw[0]), pw2=_conv_t(b.pw[2]),
                m1=_conv_t(b.mlp.net[0]), m2=_conv_t(b.mlp.net[3]),
                s_wbig=_wbig(s.weight_real, s.weight_imag), v_wbig=_wbig(v.weight_real, v.weight_imag),
            )
            pk = {k: dev(m) for k, m in mats.items()}
            pk.update({k + "t": dev(m.t()) for k, m in mats.items()})               # transposes for the VJP
            pk["v_zp"] = dev(v.z_proj.weight.detach().reshape(C))
            pk["bgb"] = dev(b.branch_gate[2].bias.detach())
            for n in NORMS:
                norm = getattr(b, "norm_" + n)
                pk[n + "_g"] = dev(norm.weight.detach())
                pk[n + "_b"] = dev(norm.bias.detach())
            pk["res"] = (float(b.res_fused.detach()), float(b.res_pw.detach()), float(b.res_mlp.detach()))
            if self.tc:
                self._tc_block(pk, b, device)
            elif self.tc_chan:
                self._tc_chan_block(pk, b, device)
            self.blocks.append(pk)
        nh = model.proj2.out_channels
        self.nh = nh
        self.nhp = 16 if nh <= 16 else 32
        if nh > 32:
            raise ValueError("at most 32 head channels are supported")
        self.p1 = dev(_conv_t(model.proj1))
        self.p1t = dev(_conv_t(model.proj1).t())
        p2 = torch.zeros(2 * C, self.nhp)
        p2[:, :nh] = _conv_t(model.proj2)
        self.p2 = dev(p2)
        self.p2t = dev(p2.t())
        b2 = torch.zeros(self.nhp)
        b2[:nh] = model.proj2.bias.detach().float()
        self.b2 = dev(b2)
        self.head = self._head_params(model)
        # the split-BF16 path evaluates the LTE weights and log-softmax in FP32 (its tolerance is 2e-3 dex; FP32
        # rounding there is ~1e-6 dex), the FP32 path in FP64 as the reference does
        self.head32 = nat.HeadParams.from_buffer_copy(self.head)
        self.head32.math32 = 1
        if self.tc:   # proj1 [2C][C] and proj2 [nhp][2C] for the tensor-core head
            w1, w2 = _w(model.proj1), p2.t()
            self.tc_head = tc_pack(device, w1, w2)
            self.tcb_head = tc_pack(device, w1, w2, w2.t(), w1.t())
        elif self.tc_chan and C == 96:   # width 96: the backward reads the transposes out of the forward's pack
            self.tc_head = self.tcb_head = tc_pack(device, _w(model.proj1), p2.t())
        self.freq_params = {k: v.detach().cpu() for k, v in model.state_dict().items() if ".freq_" in k}
        self.freq_key = table_store.freq_key(self.freq_params)

    @staticmethod
    def _tc_block(pk, b, device):
        """Split-BF16 packs of one block for the tensor-core kernels (matrix order of each entry point)."""
        s, v = b.spec, b.vertical
        for name, (c1, c2) in dict(s_post=(s.post[0], s.post[2]), v_post=(v.post[0], v.post[2]),
                                   pw=(b.pw[0], b.pw[2]), mlp=(b.mlp.net[0], b.mlp.net[3])).items():
            w1, w2 = _w(c1), _w(c2)
            pk["tc_" + name] = tc_pack(device, w1, w2)
            pk["tcb_" + name] = tc_pack(device, w1, w2.t(), w1.t())
        for name, gate in (("s_gate", s.input_gate), ("v_gate", v.input_gate)):
            g1, g2 = _w(gate[0]), _w(gate[2])
            pk["tc_" + name] = tc_pack(device, g1, g2)
            pk["tcb_" + name] = tc_pack(device, g1, g2, g2.t(), g1.t())
        bg0, bg2, f0, f2 = _w(b.branch_gate[0]), _w(b.branch_gate[2]), _w(b.fuse[0]), _w(b.fuse[2])
        pk["tc_fuse1"] = tc_pack(device, bg0, bg2)
        pk["tc_fuse2"] = tc_pack(device, f0, f2)
        pk["tcb_fuse_a"] = tc_pack(device, f0, f2.t())
        pk["tcb_fuse_b"] = tc_pack(device, f0.t(), bg2.t(), bg0.t())
        for name, conv in (("s", s), ("v", v)):
            wb = _wbig(conv.weight_real, conv.weight_imag)
            pk[f"tc_{name}_mix"] = mix_pack(device, wb.t())      # out = xhat @ wbig -> matrix wbig^T
            pk[f"tcb_{name}_mix"] = mix_pack(device, wb)         # adjoint: xhat_bar = y_bar @ wbig^T

    @staticmethod
    def _tc_chan_block(pk, b, device):
        """Split-BF16 packs of one block's channel MLPs, input gates and branch fusion at width 96: [w1, w2] for the
        forward, and the same packs for the backward (its kernels read the transposes out of them)."""
        s, v = b.spec, b.vertical
        for name, (c1, c2) in dict(s_post=(s.post[0], s.post[2]), v_post=(v.post[0], v.post[2]),
                                   pw=(b.pw[0], b.pw[2]), mlp=(b.mlp.net[0], b.mlp.net[3]),
                                   s_gate=(s.input_gate[0], s.input_gate[2]),
                                   v_gate=(v.input_gate[0], v.input_gate[2])).items():
            pk["tc_" + name] = pk["tcb_" + name] = tc_pack(device, _w(c1), _w(c2))
        # the mixing: wbig for the operator, wbig^T for its adjoint
        for name, conv in (("s", s), ("v", v)):
            wb = _wbig(conv.weight_real, conv.weight_imag)
            pk[f"tc_{name}_mix"] = tc_pack(device, wb)
            pk[f"tcb_{name}_mix"] = tc_pack(device, wb.t())
        # the branch fusion: the gates' [wg1, wg2] (also read transposed by the backward), [wf1], [wf2]
        pk["tc_fuse1"] = tc_pack(device, _w(b.branch_gate[0]), _w(b.branch_gate[2]))
        pk["tc_f1"] = tc_pack(device, _w(b.fuse[0]))
        pk["tc_f2"] = tc_pack(device, _w(b.fuse[2]))

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


class FreqTables:
    """g, U, V of one operator of one block on the device, with the adjoint forms (conj g, V^T as U, U^T as V)."""

    def __init__(self, g, u, v, device):
        f = lambda a: None if a is None else a.to(device=device, dtype=torch.float32).contiguous()
        self.g, self.u, self.v = f(g), f(u), f(v)
        self.g_adj = f(torch.stack([g[:, 0], -g[:, 1]], 1))
        self.u_adj = None if v is None else f(v.transpose(1, 2))     # [F][C][r] = V^T
        self.v_adj = None if u is None else f(u.transpose(1, 2))     # [F][r][C] = U^T


class Geometry:
    def __init__(self, shared, span, column, column_raw, length, k, columns=None):
        self.shared, self.span, self.column, self.column_raw, self.length, self.k = (shared, span, column, column_raw,
                                                                                     length, k)
        self.columns = columns      # non-shared grids: every sample's columns [B][H*W][D] (float64, unshifted)


class Workspace:
    """Device buffers for one cube of shape (D, H, W) at width C."""

    def __init__(self, D, H, W, C, live, groups, device):
        V = D * H * W
        HW = H * W
        Wf = W // 2 + 1
        f32 = dict(dtype=torch.float32, device=device)
        self.V = V
        self.live = live
        self.nparts = nat.lib().ffno_stats_parts(V)
        self.nparts_tc = nat.lib().ffno_tc_parts(V)
        nb = lambda *s: torch.empty(*s, **f32)
        self.dw = nb(V)
        self.partials = torch.empty(max(self.nparts, self.nparts_tc, 1) * groups * 3, dtype=torch.float64,
                                    device=device)
        self.err = torch.zeros(1, dtype=torch.int32, device=device)
        self.coefs = {n: nb(3 * C) for n in ("lift",) + NORMS}
        self.gstats = {n: torch.empty(groups * 3, dtype=torch.float64, device=device) for n in ("lift",) + NORMS}
        for n in ("x", "xs", "xv", "yv", "spec_pre", "vert_pre", "fused_pre", "pw_pre", "mlp_pre", "x1", "x2"):
            setattr(self, n, nb(V, C))
        # buffers whose lives do not overlap share storage: the lift pre-activation is dead before block 0 writes
        # spec_pre (and, in the VJP, spec_pre is dead when the lift is recomputed); the gated input xs is dead once
        # the W transform has read it, before the spectral branch writes ys
        self.pre = self.spec_pre
        self.ys = self.xs
        spec_len = D * 2 * H * Wf * C
        self.sa, self.sb = nb(spec_len), nb(spec_len)
        self.gates = nb(V, 2 * C)     # branch gates between the two tensor-core fuse stages
        self.hf = nb(V, 2 * C) if C == 96 else None   # the width-96 fusion's hidden pre-activation
        self.va, self.vb = nb(2 * live * HW * C), nb(2 * live * HW * C)
        self.hg = None                # the gate MLP's hidden pre-activation, kept only by a caching forward

    # the intermediates a block's VJP reads (kept per block when the forward caches block states)
    CACHED = ("xs", "xv", "yv", "spec_pre", "vert_pre", "fused_pre", "pw_pre", "mlp_pre", "x1", "x2", "vb")

    def state_bytes(self, gates):
        """Device bytes of one block's cached intermediates (gates: also the branch gates and the gate MLP's hidden
        layer of the tensor-core fuse)."""
        extra = 3 * self.x.numel() + (self.hf.numel() if self.hf is not None else 0)
        n = sum(getattr(self, n).numel() for n in self.CACHED) + (extra if gates else 0)
        return 4 * n + 2 * len(NORMS) * 8 * 64

    def fork(self, gates):
        """A view of this workspace with its own copies of the cached intermediates and GroupNorm statistics (the
        scratch buffers stay shared): block i of a caching forward writes its state there."""
        w = copy.copy(self)
        for n in self.CACHED:
            setattr(w, n, torch.empty_like(getattr(self, n)))
        if gates:
            w.gates = torch.empty_like(self.gates)
            w.hg = torch.empty_like(self.x)
            if self.hf is not None:
                w.hf = torch.empty_like(self.hf)
        w.ys = w.xs
        w.coefs = dict(self.coefs)
        w.gstats = dict(self.gstats)
        for n in NORMS:
            w.coefs[n] = torch.empty_like(self.coefs[n])
            w.gstats[n] = torch.empty_like(self.gstats[n])
        return w

    def bind(self, state):
        """This workspace's scratch with a block's cached intermediates and statistics (from fork)."""
        w = copy.copy(self)
        for n in self.CACHED + ("ys",):
            setattr(w, n, getattr(state, n))
        if state.hg is not None:
            w.gates, w.hg, w.hf = state.gates, state.hg, state.hf
        w.coefs = dict(self.coefs)
        w.gstats = dict(self.gstats)
        for n in NORMS:
            w.coefs[n] = state.coefs[n]
            w.gstats[n] = state.gstats[n]
        return w


class Executor:
    def __init__(self, model):
        self.model = model
        self._packed = None
        self._packed_key = None
        self._plane = {}
        self._plane_freq = {}
        self._height = {}
        self._lock = threading.RLock()        # caches are shared by concurrent service slots
        # shape-constant tables persist across processes in a TableStore ($FFNO_GB300_TABLE_CACHE, or assigned)
        self.tables = table_store.default_store()
        self._tls = threading.local()         # per-thread mode (a JVP forces the FP32 kernels)
        # A forward for the VJP keeps every block's intermediates instead of recomputing them in the backward when
        # they fit in half the free device memory (models/ffno_model.py:786-791 recomputes each block under
        # checkpoint_blocks). A host that runs several requests at once on the device turns this off (the service
        # does).
        self.cache_states = True
        self.last_cached = False              # whether the last forward for a VJP kept its block states

    # -------------------------------------------------------------------------------------------- caches
    def packed(self, device):
        with self._lock:
            return self._packed_locked(device)

    def _packed_locked(self, device):
        key = (_weights_key(self.model), str(device))
        if self._packed_key != key:
            self._packed = Packed(self.model, device)
            self._packed_key = key
            self._plane_freq.clear()
            self._height.clear()
        return self._packed

    def plane(self, H, W, device):
        with self._lock:
            return self._plane_locked(H, W, device)

    def _plane_locked(self, H, W, device):
        key = (H, W, str(device))
        if key not in self._plane:
            t = table_store.plane_arrays(self.tables, H, W)
            twf, thf, thi, twi = t["twf"], t["thf"], t["thi"], t["twi"]
            f = lambda a: torch.as_tensor(np.ascontiguousarray(a), dtype=torch.float32, device=device)
            # forward tables and the transposes the VJP applies (rows/cols swapped)
            self._plane[key] = dict(twf=f(twf), thf=f(thf), thi=f(thi), twi=f(twi), twf_t=f(twf.T), thf_t=f(thf.T),
                                    thi_t=f(thi.T), twi_t=f(twi.T), np=dict(twf=twf, thf=thf, thi=thi, twi=twi),
                                    device=device)
        return self._plane[key]

    def plane_freq(self, pk, H, W, dx, dy, device):
        with self._lock:
            return self._plane_freq_locked(pk, H, W, dx, dy, device)

    def _plane_freq_locked(self, pk, H, W, dx, dy, device):
        key = (H, W, float(dx), float(dy))
        if key not in self._plane_freq:
            n, rank = self.model.n_layers, self.model.freq_mix_rank
            t = table_store.plane_freq_arrays(self.tables, pk.freq_params, pk.freq_key, n, rank, H, W, dx, dy)
            self._plane_freq[key] = [FreqTables(*gv, device) for gv in table_store.freq_list(t, n)]
        return self._plane_freq[key]

    def height(self, pk, geo, device):
        with self._lock:
            return self._height_locked(pk, geo, device)

    def _height_locked(self, pk, geo, device):
        key = (geo.column.tobytes(), float(geo.length), geo.k.numel())
        if key not in self._height:
            n, rank = self.model.n_layers, self.model.freq_mix_rank
            t = table_store.height_arrays(self.tables, pk.freq_params, pk.freq_key, n, rank, geo.column, geo.length,
                                          geo.k, self.model.z_feature_wavelength)
            live, tzf, tzi = int(t["live"]), t["tzf"], t["tzi"]
            per_block = [FreqTables(*gv, device) for gv in table_store.freq_list(t, n)]
            f = lambda a: torch.as_tensor(np.ascontiguousarray(a), dtype=torch.float32, device=device)
            # what the tables' gradient w.r.t. the shared column takes (ffno_percol_tables_vjp with one column):
            # the column, its live wavenumbers, mode factors, their derivative in the median spacing and its index
            vlive, fcol, dfcol, med = tb.percolumn_prep(np.asarray(geo.column, np.float64)[None], geo.length, geo.k)
            if vlive != live:
                raise RuntimeError("height table live-mode counts disagree")
            f64 = lambda a: torch.as_tensor(np.ascontiguousarray(a), dtype=torch.float64, device=device)
            vjp = dict(z=f64(np.asarray(geo.column, np.float64)[None]), k=f64(geo.k.numpy()[:live]), f=f64(fcol),
                       df=f64(dfcol), med=torch.as_tensor(med, dtype=torch.int32, device=device), med_i=int(med[0]))
            self._height[key] = dict(live=live, tzf=f(tzf), tzi=f(tzi), tzf_t=f(tzf.T), tzi_t=f(tzi.T),
                                     freq=per_block, np=dict(tzf=tzf, tzi=tzi), vjp=vjp, device=device)
        return self._height[key]

    def tc_table(self, tabs, name):
        """The split-BF16 pack of table `name` (a key of the plane or height dict; suffix _t = transposed), built once."""
        key = "tc_" + name
        with self._lock:
            if key not in tabs:
                base = tabs["np"][name[:-2] if name.endswith("_t") else name]
                tabs[key] = TcXform(base.T if name.endswith("_t") else base, tabs["device"])
        return tabs[key]

    def _xf(self, tabs, name, inp, out, desc, ws):
        """out = T_name applied by ffno_xform (FP32) or ffno_xform_tc (split-BF16 tensor cores)."""
        s = _stream()
        if not self._tc_xf():
            nat.call("ffno_xform", tabs[name].data_ptr(), inp.data_ptr(), out.data_ptr(), desc, 0, s, tag=name)
            return
        tx = self.tc_table(tabs, name)
        if tx.M > 256 and desc.out_split < desc.M:
            raise ValueError("a transform taller than 256 rows needs single-level output addressing")
        if tx.K > XFORM_TC_MAX_K and desc.in_split < desc.K:
            raise ValueError("a transform longer than 512 columns needs single-level input addressing")
        for r0, rows, c0, cols, packed, res in tx.slices:
            d = nat.XformDesc.from_buffer_copy(desc)
            d.M, d.K = rows, cols
            src = inp.data_ptr() + 4 * c0 * desc.in_lo
            dst = out.data_ptr() + 4 * r0 * desc.out_lo
            acc = 1 if c0 else 0
            if res is not None:
                nat.call("ffno_xform_tcr", res[0].data_ptr(), res[1], res[2], src, dst, d, acc, ws.err.data_ptr(), s,
                         tag=name)
            else:
                nat.call("ffno_xform_tc", packed.data_ptr(), src, dst, d, acc, ws.err.data_ptr(), s, tag=name)

    # -------------------------------------------------------------------------------------------- geometry
    def geometry(self, z_scale):
        """Per-batch height analysis (HeightSpectralConv.box and shared-grid test, models/ffno_model.py:248-269) of
        the device heights: a column-analysis kernel, whose two numbers per sample are read back (a synchronisation
        with the stream)."""
        B, D = z_scale.shape[0], z_scale.shape[1]
        HW = z_scale.shape[2] * z_scale.shape[3]
        info = torch.empty(B, 2, dtype=torch.float32, device=z_scale.device)
        s = _stream()
        for b in range(B):
            nat.call("ffno_column_info", z_scale[b].data_ptr(), D, HW, info[b].data_ptr(), s)
        col = z_scale[:, :, 0, 0]
        host = torch.cat([info.reshape(-1), col.reshape(-1)]).cpu()
        info_h = host[:2 * B].reshape(B, 2)
        cols32 = host[2 * B:].reshape(B, D).numpy()
        columns = lambda: z_scale.reshape(B, D, HW).transpose(1, 2).double().cpu().numpy()
        return self._geometry(bool((info_h[:, 0] > 0.5).all()), float(info_h[:, 1].max()), cols32, columns)

    def geometry_host(self, z_mm):
        """The same analysis of heights held on the host (float32 numpy [B, D, H, W] in Mm, the values the device
        holds), without touching the device: the service backend decides it once per request, before the model
        runs, so no read-back synchronises the request's stream."""
        z = np.asarray(z_mm, dtype=np.float32)
        B, D = z.shape[0], z.shape[1]
        zd = z.reshape(B, D, -1)                                  # [B][D][HW]: reductions over D run along rows
        zc = zd.transpose(0, 2, 1)                                # [B][HW][D] view
        col0 = np.ascontiguousarray(zc[:, 0, :])                  # [B][D]
        if bool((zd == zd[:, :, :1]).all()):
            # every column equals its sample's column (0, 0): shared grids, one pass over the heights
            span = float((col0.max(axis=1) - col0.min(axis=1)).max())
            return self._geometry(True, span, col0, lambda: zc.astype(np.float64))
        mn = zd.min(axis=1)                                       # [B][HW]
        span = float((zd.max(axis=1) - mn).max())
        shifted = zd - mn[:, None, :]                             # float32, as ffno_column_info compares them
        shared_each = all(bool((shifted[b] == shifted[b, :, :1]).all()) for b in range(B))
        return self._geometry(shared_each, span, col0, lambda: zc.astype(np.float64))

    def geometry_columns(self, zc, columns):
        """geometry_host from columns: zc [B][N][D] float32, every sample's N = H*W columns in any order with column
        (0, 0) first; columns() -> [B][H*W][D] float64 in the model's h*W + w order (built only for per-column
        grids)."""
        mn = zc.min(axis=2)
        span = float((zc.max(axis=2) - mn).max())
        shifted = zc - mn[:, :, None]                      # float32, as ffno_column_info compares them
        shared_each = all(bool((shifted[b] == shifted[b, :1, :]).all()) for b in range(zc.shape[0]))
        return self._geometry(shared_each, span, np.ascontiguousarray(zc[:, 0, :]), columns)

    def _geometry(self, shared_each, span, cols32, columns):
        """Geometry from the per-sample test, the span and every sample's column 0; columns() gives every sample's
        columns [B][H*W][D] (float64), gathered only when the grids are not shared."""
        cols = cols32.astype(np.float64)
        shifted32 = cols32 - cols32.min(axis=1, keepdims=True)       # the test in the model's float32
        shared = shared_each and bool((shifted32 == shifted32[:1]).all())
        shifted = cols - cols.min(axis=1, keepdims=True)
        m = self.model
        modes = int(math.floor(m.z_reference_length / m.z_min_wavelength)) + 1
        length, k = tb.height_box(span, m.z_reference_length, m.z_min_wavelength, modes)
        return Geometry(shared, span, shifted[0], cols[0], length, k, None if shared else columns())

    def height_percol(self, pk, geo, b, device):
        """Per-column tables of sample b when the height grids differ (cached by the sample's heights)."""
        cols = geo.columns[b]
        key = ("percol", hashlib.sha1(cols.tobytes()).hexdigest(), cols.shape, float(geo.length), geo.k.numel())
        with self._lock:
            if key not in self._height:
                # per-column tables are large ([H*W][2M'][D] each): keep only the two most recent samples
                old = [k for k in self._height if k[0] == "percol"]
                for k in old[:-1]:
                    del self._height[k]
                # the tables of every column are built on the device (ffno_percol_tables, FP64); the host decides
                # the live modes, the tapers and their derivative, and the median spacing's index
                live, fcol, dfcol, med = tb.percolumn_prep(cols, geo.length, geo.k)
                ncol, D = cols.shape
                f64 = lambda a: torch.as_tensor(np.ascontiguousarray(a), dtype=torch.float64, device=device)
                zc, kk, fd, dfd = f64(cols), f64(geo.k.numpy()[:live]), f64(fcol), f64(dfcol)
                medd = torch.as_tensor(med, dtype=torch.int32, device=device)
                t32 = lambda *shape: torch.empty(*shape, dtype=torch.float32, device=device)
                tzf, tzi = t32(ncol, 2 * live, D), t32(ncol, D, 2 * live)
                tzf_t, tzi_t = t32(ncol, D, 2 * live), t32(ncol, 2 * live, D)
                nat.call("ffno_percol_tables", zc.data_ptr(), D, ncol, kk.data_ptr(), live, fd.data_ptr(),
                         tzf.data_ptr(), tzi.data_ptr(), tzf_t.data_ptr(), tzi_t.data_ptr(), _stream())
                feats = tb.height_features(geo.k[:live], self.model.z_feature_wavelength)
                rank = self.model.freq_mix_rank
                per_block = [FreqTables(*tb.freq_tables(pk.freq_params, f"blocks.{i}.vertical", feats, rank), device)
                             for i in range(self.model.n_layers)]
                self._height[key] = dict(live=live, percol=True, tzf=tzf, tzi=tzi, tzf_t=tzf_t, tzi_t=tzi_t,
                                         freq=per_block, columns=cols, z=zc, k=kk, f=fd, df=dfd, med=medd)
            return self._height[key]

    # -------------------------------------------------------------------------------------------- setup
    def _setup(self, x, z_scale, dx, dy, geo=None):
        m = self.model
        if not x.is_cuda or not z_scale.is_cuda:
            raise RuntimeError("ffnoml_gb300 runs on CUDA tensors only")
        if x.dtype != torch.float32 or z_scale.dtype != torch.float32:
            raise TypeError("ffnoml_gb300 FFNO3D takes float32 inputs")
        if m.width not in SUPPORTED_WIDTHS:
            raise ValueError(f"width {m.width} is not supported (supported: {SUPPORTED_WIDTHS})")
        if x.dim() != 5 or z_scale.dim() != 4 or z_scale.shape != (x.shape[0],) + tuple(x.shape[2:]):
            raise ValueError(f"x must be [B, Cin, D, H, W] and z_scale [B, D, H, W]; got {tuple(x.shape)}, "
                             f"{tuple(z_scale.shape)}")
        if x.shape[1] != m.in_channels:
            raise ValueError(f"expected {m.in_channels} input channels, got {x.shape[1]}")
        if x.shape[2] < 2:
            raise ValueError("the height operator needs at least two levels")
        device = x.device
        pk = self.packed(device)
        if geo is None:
            geo = self.geometry(z_scale)
        hgt = self.height(pk, geo, device) if geo.shared else None
        B, _, D, H, W = x.shape
        pln = self.plane(H, W, device)
        pfr = self.plane_freq(pk, H, W, dx, dy, device)
        return pk, geo, hgt, pln, pfr

    # -------------------------------------------------------------------------------------------- forward
    def forward(self, x, z_scale, dx, dy, keep=False, geo=None, errs=None):
        """x [B, Cin, D, H, W], z_scale [B, D, H, W] (Mm), float32 CUDA -> [B, L, D, H, W] float32. With keep=True
        also returns the state the VJP needs (block inputs per cube). geo: the heights' analysis when the caller
        already has it (geometry_host), else it is computed on the device. errs: a list that receives the device
        error flag instead of it being read here (a read waits for the stream); the caller checks it with
        check_flags after its own synchronisation."""
        m = self.model
        x = x.contiguous()
        z_scale = z_scale.contiguous()
        pk, geo, hgt, pln, pfr = self._setup(x, z_scale, dx, dy, geo)
        B, _, D, H, W = x.shape
        out = torch.empty(B, m.out_channels, D, H, W, dtype=torch.float32, device=x.device)
        saved, states = [], []
        ws = None
        cache = None
        for b in range(B):
            hgt_b = hgt if geo.shared else self.height_percol(pk, geo, b, x.device)
            if ws is None or ws.live != hgt_b["live"]:
                ws = Workspace(D, H, W, m.width, hgt_b["live"], pk.groups, x.device)
            if keep and cache is None:
                cache = self.cache_states and self._fits(B * m.n_layers * ws.state_bytes(self._keeps_gates()),
                                                         x.device)
                self.last_cached = cache
            xin, z = x[b], z_scale[b]
            self._depth_weights(ws, z, D, H * W)
            # a kept forward writes the lift output and every block output straight into the saved block inputs
            # (block i reads inputs[i] and writes inputs[i + 1] through ws.x), so nothing is copied to keep them
            inputs = [torch.empty_like(ws.x) for _ in range(m.n_layers + 1)] if keep else None
            if keep:
                ws.x = inputs[0]
            self._lift(pk, ws, xin)
            blocks = [] if cache else None
            for i in range(m.n_layers):
                if keep:
                    ws.x = inputs[i + 1]
                wb = ws.fork(self._keeps_gates()) if cache else ws
                self._block(pk, wb, i, z, D, H, W, hgt_b, pln, pfr[i], x_in=inputs[i] if keep else None)
                if cache:
                    blocks.append(wb)
            self._head(pk, ws.x, xin, out[b], ws.err)
            if keep:
                saved.append(inputs)
                states.append(blocks)
        if not keep:
            if errs is None:
                self._check(ws)
            else:
                errs.append(ws.err)
            return out, None
        # a forward kept for the VJP leaves its error flag to the backward, which reads it with its own at the end
        # (one synchronisation for both passes; the flag is sticky): callers that may not run the backward call
        # check_forward
        state = dict(x=x, z=z_scale, dx=dx, dy=dy, inputs=saved, geo=geo, blocks=states if cache else None,
                     err=ws.err)
        return out, state

    def check_forward(self, state):
        """Raise if the forward that made `state` (forward(keep=True)) ran out of a bounded wait."""
        self._check_flag(state["err"])

    @staticmethod
    def check_flags(errs):
        """Raise if any error flag collected by forward / backward(errs=...) is set (reads them: waits for their
        streams)."""
        for e in errs:
            Executor._check_flag(e)

    @staticmethod
    def _fits(nbytes, device):
        free, _ = torch.cuda.mem_get_info(device)
        # memory PyTorch's allocator holds but no tensor uses is free for this process too
        free += torch.cuda.memory_reserved(device) - torch.cuda.memory_allocated(device)
        return nbytes <= 0.5 * free

    @staticmethod
    def _check(ws):
        Executor._check_flag(ws.err)

    @staticmethod
    def _check_flag(err):
        if m_err := int(err.item()):
            raise nat.NativeError(f"a tensor-core kernel's bounded wait ran out (code {m_err})")

    def _depth_weights(self, ws, z, D, HW):
        nat.call("ffno_depth_weights", z.data_ptr(), D, HW, ws.dw.data_ptr(), _stream())

    def _finalize(self, ws, name, gamma, beta, tc=False):
        m = self.model
        nat.call("ffno_gn_finalize", ws.partials.data_ptr(), ws.nparts_tc if tc else ws.nparts, m.width,
                 self._packed.groups,
                 gamma.data_ptr(), beta.data_ptr(), EPS, ws.coefs[name].data_ptr(), ws.gstats[name].data_ptr(),
                 _stream())

    def _lift(self, pk, ws, xin):
        m = self.model
        V, C, s = ws.V, m.width, _stream()
        nat.call("ffno_lift_fwd", xin.data_ptr(), m.in_channels, V, C, pk.lift_w.data_ptr(), ws.dw.data_ptr(),
                 ws.pre.data_ptr(), ws.partials.data_ptr(), ws.nparts, pk.groups, s)
        self._finalize(ws, "lift", pk.lift_g, pk.lift_b)
        nat.call("ffno_gn_act", ws.pre.data_ptr(), ws.coefs["lift"].data_ptr(), V, C, 1, ws.x.data_ptr(), s)

    def _block(self, pk, ws, i, z, D, H, W, hgt, pln, fq, x_in=None):
        """Block i on ws.x (or x_in), leaving every intermediate in ws and the block output in ws.x."""
        m = self.model
        C, V, HW, Wf = m.width, ws.V, H * W, W // 2 + 1
        s = _stream()
        bp = pk.blocks[i]
        G, P = pk.groups, ws.nparts
        x = ws.x if x_in is None else x_in
        live = hgt["live"]
        d = _descs(D, H, W, C, live)
        if self._tc_chan():
            nat.call("ffno_gate_fwd_tc", x.data_ptr(), V, C, bp["tc_s_gate"].data_ptr(), None, None, ws.xs.data_ptr(),
                     ws.err.data_ptr(), s)
            nat.call("ffno_gate_fwd_tc", x.data_ptr(), V, C, bp["tc_v_gate"].data_ptr(), bp["v_zp"].data_ptr(),
                     z.data_ptr(), ws.xv.data_ptr(), ws.err.data_ptr(), s)
        else:
            nat.call("ffno_gate_fwd", x.data_ptr(), V, C, bp["s_g1"].data_ptr(), bp["s_g2"].data_ptr(), None, None,
                     ws.xs.data_ptr(), s)
            nat.call("ffno_gate_fwd", x.data_ptr(), V, C, bp["v_g1"].data_ptr(), bp["v_g2"].data_ptr(),
                     bp["v_zp"].data_ptr(), z.data_ptr(), ws.xv.data_ptr(), s)
        # horizontal spectral branch: rfft2 -> mix -> irfft2 as contractions
        self._xf(pln, "twf", ws.xs, ws.sa, d["wf"], ws)
        self._xf(pln, "thf", ws.sa, ws.sb, d["hf"], ws)
        self._mix(ws, "s", bp, fq, ws.sb, ws.sa, H * Wf, D, C, 2 * H * Wf * C, H * Wf * C, False)
        self._xf(pln, "thi", ws.sa, ws.sb, d["hf"], ws)
        self._xf(pln, "twi", ws.sb, ws.ys, d["wi"], ws)
        tc = self._mlp2(ws, 0, ws.ys, None, None, 0.0, None, bp["s_p1"], bp["s_p2"], bp.get("tc_s_post"),
                        ws.spec_pre)
        self._finalize(ws, "spec", bp["spec_g"], bp["spec_b"], tc)
        # vertical (height) branch
        hq = hgt["freq"][i]
        if hgt.get("percol"):
            nat.call("ffno_xform_pt", hgt["tzf"].data_ptr(), 2 * live * D, ws.xv.data_ptr(), ws.va.data_ptr(),
                     d["pcf"], 0, s)
            self._mix(ws, "v", bp, hq, ws.va, ws.vb, live, HW, HW * C, C, live * HW * C, False)
            nat.call("ffno_xform_pt", hgt["tzi"].data_ptr(), 2 * live * D, ws.vb.data_ptr(), ws.yv.data_ptr(),
                     d["pci"], 0, s)
        else:
            self._xf(hgt, "tzf", ws.xv, ws.va, d["zf"], ws)
            self._mix(ws, "v", bp, hq, ws.va, ws.vb, live, HW, HW * C, C, live * HW * C, False)
            self._xf(hgt, "tzi", ws.vb, ws.yv, d["zi"], ws)
        tc = self._mlp2(ws, 0, ws.yv, None, None, 0.0, None, bp["v_p1"], bp["v_p2"], bp.get("tc_v_post"),
                        ws.vert_pre)
        self._finalize(ws, "vert", bp["vert_g"], bp["vert_b"], tc)
        # gate + fuse
        if self._tc():
            self._fuse1_tc(ws, bp, x, ws.hg)
            nat.call("ffno_fuse2_tc", ws.spec_pre.data_ptr(), ws.coefs["spec"].data_ptr(), ws.vert_pre.data_ptr(),
                     ws.coefs["vert"].data_ptr(), ws.gates.data_ptr(), V, C, bp["tc_fuse2"].data_ptr(),
                     ws.dw.data_ptr(), ws.fused_pre.data_ptr(), ws.partials.data_ptr(), ws.nparts_tc, G,
                     ws.err.data_ptr(), s)
            self._finalize(ws, "fuse", bp["fuse_g"], bp["fuse_b"], True)
        elif self._tc_fuse96():
            self._fuse1_tc(ws, bp, x, ws.hg)
            sp, cs, vp, cv = (ws.spec_pre.data_ptr(), ws.coefs["spec"].data_ptr(), ws.vert_pre.data_ptr(),
                              ws.coefs["vert"].data_ptr())
            nat.call("ffno_fuse_hidden_tc", sp, cs, vp, cv, ws.gates.data_ptr(), V, C, bp["tc_f1"].data_ptr(),
                     ws.hf.data_ptr(), ws.err.data_ptr(), s)
            nat.call("ffno_fuse_out_tc", sp, cs, vp, cv, ws.gates.data_ptr(), ws.hf.data_ptr(), V, C,
                     bp["tc_f2"].data_ptr(), ws.dw.data_ptr(), ws.fused_pre.data_ptr(), ws.partials.data_ptr(),
                     ws.nparts_tc, G, ws.err.data_ptr(), s)
            self._finalize(ws, "fuse", bp["fuse_g"], bp["fuse_b"], True)
        else:
            nat.call("ffno_fuse_fwd", x.data_ptr(), ws.spec_pre.data_ptr(), ws.coefs["spec"].data_ptr(),
                     ws.vert_pre.data_ptr(), ws.coefs["vert"].data_ptr(), V, C, bp["bg1"].data_ptr(),
                     bp["bg2"].data_ptr(), bp["bgb"].data_ptr(), bp["f1"].data_ptr(), bp["f2"].data_ptr(),
                     ws.dw.data_ptr(), ws.fused_pre.data_ptr(), ws.partials.data_ptr(), P, G, s)
            self._finalize(ws, "fuse", bp["fuse_g"], bp["fuse_b"])
        r_f, r_pw, r_mlp = bp["res"]
        tc = self._mlp2(ws, 1, x, ws.fused_pre, ws.coefs["fuse"], r_f, ws.x1, bp["pw1"], bp["pw2"], bp.get("tc_pw"),
                        ws.pw_pre)
        self._finalize(ws, "pw", bp["pw_g"], bp["pw_b"], tc)
        tc = self._mlp2(ws, 2, ws.x1, ws.pw_pre, ws.coefs["pw"], r_pw, ws.x2, bp["m1"], bp["m2"], bp.get("tc_mlp"),
                        ws.mlp_pre)
        self._finalize(ws, "mlp", bp["mlp_g"], bp["mlp_b"], tc)
        nat.call("ffno_resid_out", ws.x2.data_ptr(), ws.mlp_pre.data_ptr(), ws.coefs["mlp"].data_ptr(), r_mlp, V, C,
                 ws.x.data_ptr(), s)

    def _mix(self, ws, branch, bp, fq, inp, out, F, nb, sf, sb, s_im, adjoint):
        """Per-frequency channel mixing (or its adjoint) on FP32 cores or tensor cores."""
        m = self.model
        s = _stream()
        g, u, v = (fq.g_adj, fq.u_adj, fq.v_adj) if adjoint else (fq.g, fq.u, fq.v)
        if (self._tc() or self._tc_fuse96()) and m.freq_mix_rank <= MIX_RANK_TC:
            w = bp[("tcb_" if adjoint else "tc_") + branch + "_mix"]
            nat.call("ffno_spectral_mix_tc", inp.data_ptr(), out.data_ptr(), F, nb, sf, sb, s_im, m.width,
                     w.data_ptr(), g.data_ptr(), _ptr(u), _ptr(v), m.freq_mix_rank, ws.err.data_ptr(), s)
        else:
            w = bp[branch + "_wbig" + ("t" if adjoint else "")]
            nat.call("ffno_spectral_mix", inp.data_ptr(), out.data_ptr(), F, nb, sf, sb, s_im, m.width, w.data_ptr(),
                     g.data_ptr(), _ptr(u), _ptr(v), m.freq_mix_rank, s)

    def _outer(self, ws, a, ma, b, mb, n, part, nsplit, out):
        """out [ma][mb] += a [ma][n] @ b [mb][n]^T (double): a height-transform table's gradient. The tensor-core
        kernel holds the longer side in 128-row tiles and the shorter (rounded up to 16) as the MMA's N, at most 512
        accumulator columns in all; a longer product (a production height grid: 2 M' = 680 rows at D = 256) runs as
        slices of the longer side, each its own call into its rows or columns of out. A shorter side above 256 runs on
        the FP32 kernel."""
        plan = _outer_tc_slices(ma, mb)
        s = _stream()
        if self._tc_xf() and plan is not None:
            if len(plan) == 1:
                nat.call("ffno_outer_tc", a.data_ptr(), n, ma, b.data_ptr(), n, mb, n, part.data_ptr(), nsplit,
                         out.data_ptr(), 1, ws.err.data_ptr(), s)
                return
            for r0, rows in plan:
                if ma >= mb:      # slices of a: rows r0 .. r0 + rows of out
                    pa, sa, pb, sb, po = a.data_ptr() + 4 * r0 * n, rows, b.data_ptr(), mb, out.data_ptr() + 8 * r0 * mb
                else:             # slices of b: columns r0 .. r0 + rows of out
                    pa, sa, pb, sb, po = a.data_ptr(), ma, b.data_ptr() + 4 * r0 * n, rows, out.data_ptr() + 8 * r0
                ns = max(1, min(_sm_count(out.device), part.numel() // (sa * sb), (n + 1023) // 1024))
                nat.call("ffno_outer_tc_ld", pa, n, sa, pb, n, sb, n, part.data_ptr(), ns, po, mb, 1,
                         ws.err.data_ptr(), s)
            return
        nat.call("ffno_outer", a.data_ptr(), n, ma, b.data_ptr(), n, mb, n, part.data_ptr(), nsplit,
                 out.data_ptr(), 1, s)

    def _tc(self):
        """Whether the split-BF16 tensor-core kernels run (precision 'bf16' at a width they support; never inside a
        JVP, which is FP32)."""
        return self.model.precision == "bf16" and self._packed.tc and not getattr(self._tls, "fp32", False)

    def _tc_chan(self):
        """Whether the channel MLPs and input gates run on the split-BF16 tensor-core kernels: wherever _tc() does,
        and at width 96."""
        return self.model.precision == "bf16" and self._packed.tc_chan and not getattr(self._tls, "fp32", False)

    def _tc_fuse96(self):
        """Whether the branch fusion (gates, hidden layer, output; three backward kernels), the mixing and the head
        run on the width-96 tensor-core kernels."""
        return self._tc_chan() and not self._packed.tc and self.model.width == 96

    def _keeps_gates(self):
        """Whether a caching forward keeps the fusion's gates and hidden layers (the tensor-core fusion)."""
        return self._tc() or self._tc_fuse96()

    def _tc_xf(self):
        """Whether the transforms and the height-table gradients run on the split-BF16 tensor-core kernels: precision
        'bf16' at any width (their operands are tables and data columns, not channel matrices), never inside a JVP.
        At a width the channel kernels do not support (96, the production model) the rest of the model stays on the
        FP32 kernels."""
        return self.model.precision == "bf16" and not getattr(self._tls, "fp32", False)

    def _fuse1_tc(self, ws, bp, x, hg):
        m = self.model
        nat.call("ffno_fuse1_tc", x.data_ptr(), ws.spec_pre.data_ptr(), ws.coefs["spec"].data_ptr(),
                 ws.vert_pre.data_ptr(), ws.coefs["vert"].data_ptr(), ws.V, m.width, bp["tc_fuse1"].data_ptr(),
                 bp["bgb"].data_ptr(), ws.gates.data_ptr(), _ptr(hg), ws.err.data_ptr(), _stream())

    def _mlp2(self, ws, mode, inp, prev, pcoefs, res, xout, w1, w2, pack, pre):
        """ffno_mlp2_fwd (FP32) or its tensor-core twin; returns whether the tensor-core path ran."""
        m = self.model
        C, V, s, G = m.width, ws.V, _stream(), self._packed.groups
        if self._tc_chan():
            nat.call("ffno_mlp2_fwd_tc", mode, inp.data_ptr(), _ptr(prev), _ptr(pcoefs), res, _ptr(xout), V, C,
                     pack.data_ptr(), ws.dw.data_ptr(), pre.data_ptr(), ws.partials.data_ptr(), ws.nparts_tc, G,
                     ws.err.data_ptr(), s)
            return True
        nat.call("ffno_mlp2_fwd", mode, inp.data_ptr(), _ptr(prev), _ptr(pcoefs), res, _ptr(xout), V, C,
                 w1.data_ptr(), w2.data_ptr(), ws.dw.data_ptr(), pre.data_ptr(), ws.partials.data_ptr(), ws.nparts,
                 G, s)
        return False

    def _head(self, pk, x, xin, out, err, V=None):
        """The level-fraction head of V voxels (default: all rows of x): x [V][C], xin [Cin][V] -> out [L][V]."""
        m = self.model
        V = x.shape[0] if V is None else V
        if self._tc() or self._tc_fuse96():
            nat.call("ffno_head_fwd_tc", x.data_ptr(), xin.data_ptr(), V, m.width, pk.tc_head.data_ptr(),
                     pk.b2.data_ptr(), pk.nh, pk.nhp, pk.head32, out.data_ptr(), None, err.data_ptr(), _stream())
            return
        nat.call("ffno_head_fwd", x.data_ptr(), xin.data_ptr(), V, m.width, pk.p1.data_ptr(), pk.p2.data_ptr(),
                 pk.b2.data_ptr(), pk.nh, pk.nhp, pk.head, out.data_ptr(), None, _stream())

    # -------------------------------------------------------------------------------------------- JVP
    def jvp(self, x, z_scale, dx, dy, x_dot):
        """Forward-mode derivative of FFNO3D.forward along the input tangent x_dot (heights fixed; what jvp_local gets
        from dual tensors, ffno_fsdp_runtime.py:350-372): x, x_dot [B, Cin, D, H, W], z_scale [B, D, H, W] ->
        (y, y_dot) [B, L, D, H, W] (normalised log10 n). FP32 kernels whatever the model's precision; the primal
        is computed block by block next to its tangent."""
        m = self.model
        x = x.contiguous()
        z_scale = z_scale.contiguous()
        x_dot = x_dot.contiguous()
        if x_dot.shape != x.shape or x_dot.dtype != torch.float32 or x_dot.device != x.device:
            raise ValueError(f"x_dot must match x: {tuple(x_dot.shape)} {x_dot.dtype} vs {tuple(x.shape)}")
        self._tls.fp32 = True
        try:
            pk, geo, hgt, pln, pfr = self._setup(x, z_scale, dx, dy)
            B, Cin, D, H, W = x.shape
            C, V, HW = m.width, D * H * W, H * W
            dev, s = x.device, _stream()
            y = torch.empty(B, m.out_channels, D, H, W, dtype=torch.float32, device=dev)
            out = torch.empty_like(y)
            ws = tw = None
            for b in range(B):
                hgt_b = hgt if geo.shared else self.height_percol(pk, geo, b, dev)
                if ws is None or ws.live != hgt_b["live"]:
                    ws = Workspace(D, H, W, C, hgt_b["live"], pk.groups, dev)
                    tw = _TangentBuffers(D, H, W, C, hgt_b["live"], pk.groups, ws.nparts, dev)
                xin, z, xin_dot = x[b], z_scale[b], x_dot[b]
                self._depth_weights(ws, z, D, HW)
                self._lift(pk, ws, xin)
                nat.call("ffno_lift_fwd", xin_dot.data_ptr(), Cin, V, C, pk.lift_w.data_ptr(), ws.dw.data_ptr(),
                         tw.pre.data_ptr(), tw.scratch_parts.data_ptr(), ws.nparts, pk.groups, s)
                self._gn_jvp(ws, tw, ws.pre, tw.pre, pk.lift_g, pk.lift_b, "lift", 1, None, 1.0, tw.x)
                for i in range(m.n_layers):
                    tw.xp.copy_(ws.x)
                    self._block(pk, ws, i, z, D, H, W, hgt_b, pln, pfr[i], x_in=tw.xp)
                    self._block_jvp(pk, ws, tw, i, tw.xp, D, H, W, hgt_b, pln, pfr[i])
                self._head(pk, ws.x, xin, y[b], ws.err)
                nat.call("ffno_head_jvp", ws.x.data_ptr(), tw.x.data_ptr(), xin.data_ptr(), xin_dot.data_ptr(), V, C,
                         pk.p1.data_ptr(), pk.p2.data_ptr(), pk.b2.data_ptr(), pk.nhp, pk.head,
                         out[b].data_ptr(), s)
            self._check(ws)
        finally:
            self._tls.fp32 = False
        return y, out

    def _gn_jvp(self, ws, tw, pre, pre_dot, gamma, beta, name, act, base, res, out):
        m = self.model
        G, s = self._packed.groups, _stream()
        nat.call("ffno_gn_jvp_stats", pre.data_ptr(), pre_dot.data_ptr(), ws.gstats[name].data_ptr(),
                 ws.dw.data_ptr(), ws.V, m.width, G, tw.parts.data_ptr(), ws.nparts, s)
        nat.call("ffno_gn_bwd_final", tw.parts.data_ptr(), ws.nparts, G, tw.sums.data_ptr(), s)
        nat.call("ffno_gn_jvp_apply", pre.data_ptr(), pre_dot.data_ptr(), gamma.data_ptr(), beta.data_ptr(),
                 ws.gstats[name].data_ptr(), tw.sums.data_ptr(), act, _ptr(base), res, ws.V, m.width, G,
                 out.data_ptr(), s)

    def _block_jvp(self, pk, ws, tw, i, x, D, H, W, hgt, pln, fq):
        """Tangent of block i: tw.x (tangent of its input x) -> tw.x (tangent of its output), with the primal
        intermediates of the same block in ws."""
        m = self.model
        C, V, HW, Wf = m.width, ws.V, H * W, W // 2 + 1
        s = _stream()
        bp = pk.blocks[i]
        r_f, r_pw, r_mlp = bp["res"]
        live = hgt["live"]
        d = _descs(D, H, W, C, live)
        nat.call("ffno_gate_jvp", x.data_ptr(), tw.x.data_ptr(), V, C, bp["s_g1"].data_ptr(), bp["s_g2"].data_ptr(),
                 tw.xs.data_ptr(), s)
        nat.call("ffno_gate_jvp", x.data_ptr(), tw.x.data_ptr(), V, C, bp["v_g1"].data_ptr(), bp["v_g2"].data_ptr(),
                 tw.xv.data_ptr(), s)
        # the spectral operators are linear in their input: the forward kernels on the tangent
        self._xf(pln, "twf", tw.xs, tw.sa, d["wf"], ws)
        self._xf(pln, "thf", tw.sa, tw.sb, d["hf"], ws)
        self._mix(ws, "s", bp, fq, tw.sb, tw.sa, H * Wf, D, C, 2 * H * Wf * C, H * Wf * C, False)
        self._xf(pln, "thi", tw.sa, tw.sb, d["hf"], ws)
        self._xf(pln, "twi", tw.sb, tw.ys, d["wi"], ws)
        nat.call("ffno_mlp2_jvp", ws.ys.data_ptr(), tw.ys.data_ptr(), V, C, bp["s_p1"].data_ptr(),
                 bp["s_p2"].data_ptr(), tw.spec_pre.data_ptr(), s)
        hq = hgt["freq"][i]
        if hgt.get("percol"):
            nat.call("ffno_xform_pt", hgt["tzf"].data_ptr(), 2 * live * D, tw.xv.data_ptr(), tw.va.data_ptr(),
                     d["pcf"], 0, s)
            self._mix(ws, "v", bp, hq, tw.va, tw.vb, live, HW, HW * C, C, live * HW * C, False)
            nat.call("ffno_xform_pt", hgt["tzi"].data_ptr(), 2 * live * D, tw.vb.data_ptr(), tw.yv.data_ptr(),
                     d["pci"], 0, s)
        else:
            self._xf(hgt, "tzf", tw.xv, tw.va, d["zf"], ws)
            self._mix(ws, "v", bp, hq, tw.va, tw.vb, live, HW, HW * C, C, live * HW * C, False)
            self._xf(hgt, "tzi", tw.vb, tw.yv, d["zi"], ws)
        nat.call("ffno_mlp2_jvp", ws.yv.data_ptr(), tw.yv.data_ptr(), V, C, bp["v_p1"].data_ptr(),
                 bp["v_p2"].data_ptr(), tw.vert_pre.data_ptr(), s)
        # branch outputs gelu(GN(.)), then gate + fuse
        self._gn_jvp(ws, tw, ws.spec_pre, tw.spec_pre, bp["spec_g"], bp["spec_b"], "spec", 1, None, 1.0, tw.sd)
        self._gn_jvp(ws, tw, ws.vert_pre, tw.vert_pre, bp["vert_g"], bp["vert_b"], "vert", 1, None, 1.0, tw.vd)
        nat.call("ffno_fuse_jvp", x.data_ptr(), tw.x.data_ptr(), ws.spec_pre.data_ptr(), ws.coefs["spec"].data_ptr(),
                 ws.vert_pre.data_ptr(), ws.coefs["vert"].data_ptr(), tw.sd.data_ptr(), tw.vd.data_ptr(), V, C,
                 bp["bg1"].data_ptr(), bp["bg2"].data_ptr(), bp["bgb"].data_ptr(), bp["f1"].data_ptr(),
                 bp["f2"].data_ptr(), tw.fused.data_ptr(), s)
        # residual tail: x1 = x + r_f gelu(GN(fused)), x2 = x1 + r_pw GN(pw(x1)), out = x2 + r_mlp GN(mlp(x2))
        self._gn_jvp(ws, tw, ws.fused_pre, tw.fused, bp["fuse_g"], bp["fuse_b"], "fuse", 1, tw.x, r_f, tw.x1)
        nat.call("ffno_mlp2_jvp", ws.x1.data_ptr(), tw.x1.data_ptr(), V, C, bp["pw1"].data_ptr(), bp["pw2"].data_ptr(),
                 tw.pw.data_ptr(), s)
        self._gn_jvp(ws, tw, ws.pw_pre, tw.pw, bp["pw_g"], bp["pw_b"], "pw", 0, tw.x1, r_pw, tw.x2)
        nat.call("ffno_mlp2_jvp", ws.x2.data_ptr(), tw.x2.data_ptr(), V, C, bp["m1"].data_ptr(), bp["m2"].data_ptr(),
                 tw.mlp.data_ptr(), s)
        self._gn_jvp(ws, tw, ws.mlp_pre, tw.mlp, bp["mlp_g"], bp["mlp_b"], "mlp", 0, tw.x2, r_mlp, tw.x)

    # -------------------------------------------------------------------------------------------- VJP
    def backward(self, state, ybar, errs=None):
        """Input VJP: ybar [B, L, D, H, W] -> (x_bar [B, Cin, D, H, W], z_bar [B, D, H, W]). errs: as in forward
        (the backward's flag and that of the forward that made the state)."""
        m = self.model
        x, z_scale, dx, dy = state["x"], state["z"], state["dx"], state["dy"]
        pk, geo, hgt, pln, pfr = self._setup(x, z_scale, dx, dy, state.get("geo"))
        B, Cin, D, H, W = x.shape
        C, V, HW = m.width, D * H * W, H * W
        dev = x.device
        s = _stream()
        ybar = ybar.contiguous()
        xbar_in = torch.zeros_like(x)
        zbar = torch.zeros_like(z_scale)
        tc = self._tc()
        ws = gb = None
        if geo.shared:
            live = hgt["live"]
            tzf_bar = torch.zeros(2 * live, D, dtype=torch.float64, device=dev)
            tzi_bar = torch.zeros(D, 2 * live, dtype=torch.float64, device=dev)
        for b in range(B):
            hgt_b = hgt if geo.shared else self.height_percol(pk, geo, b, dev)
            live = hgt_b["live"]
            if ws is None or ws.live != live:
                ws = Workspace(D, H, W, C, live, pk.groups, dev)
                gb = _GradBuffers(D, H, W, C, live, pk.groups, ws.nparts, dev)
            if not geo.shared:
                # this sample's per-column table gradients: [HW][2M'][D] and [HW][D][2M']
                tzf_bar = torch.zeros(HW, 2 * live, D, dtype=torch.float64, device=dev)
                tzi_bar = torch.zeros(HW, D, 2 * live, dtype=torch.float64, device=dev)
            xin, z = x[b], z_scale[b]
            inputs = state["inputs"][b]
            self._depth_weights(ws, z, D, HW)
            gb.wbar.zero_()
            # head
            if tc or self._tc_fuse96():
                nat.call("ffno_head_bwd_tc", inputs[-1].data_ptr(), xin.data_ptr(), ybar[b].data_ptr(), V, C,
                         pk.tcb_head.data_ptr(), pk.b2.data_ptr(), pk.nhp, pk.head32, gb.xbar.data_ptr(),
                         xbar_in[b].data_ptr(), ws.err.data_ptr(), s)
            else:
                nat.call("ffno_head_bwd", inputs[-1].data_ptr(), xin.data_ptr(), ybar[b].data_ptr(), V, C,
                         pk.p1.data_ptr(), pk.p2.data_ptr(), pk.b2.data_ptr(), pk.p2t.data_ptr(), pk.p1t.data_ptr(),
                         pk.nhp, pk.head, gb.xbar.data_ptr(), xbar_in[b].data_ptr(), s)
            cached = state.get("blocks")
            for i in reversed(range(m.n_layers)):
                if cached and cached[b][i] is not None:
                    # a block's cached state is consumed by its VJP (a second backward over the same state
                    # recomputes the block)
                    wb = ws.bind(cached[b][i])
                    cached[b][i] = None
                else:
                    wb = ws
                    self._block(pk, ws, i, z, D, H, W, hgt_b, pln, pfr[i], x_in=inputs[i])
                self._block_bwd(pk, wb, gb, i, inputs[i], z, zbar[b], D, H, W, hgt_b, pln, pfr[i], tzf_bar, tzi_bar)
            # lift: x0 = gelu(GN(pre0))
            self._lift(pk, ws, xin)
            self._gn_bwd(ws, gb, 1, gb.xbar, 1.0, ws.pre, pk.lift_g, pk.lift_b, "lift", gb.pbar)
            nat.call("ffno_lift_bwd", gb.pbar.data_ptr(), Cin, V, C, pk.lift_w.data_ptr(), xbar_in[b].data_ptr(), s)
            nat.call("ffno_depth_weights_bwd", z.data_ptr(), gb.wbar.data_ptr(), D, HW, zbar[b].data_ptr(), s)
            if not geo.shared:
                # every column's own tables depend on that column's heights (ffno_percol_tables_vjp, FP64)
                nat.call("ffno_percol_tables_vjp", hgt_b["z"].data_ptr(), D, HW, hgt_b["k"].data_ptr(), live,
                         hgt_b["f"].data_ptr(), hgt_b["df"].data_ptr(), hgt_b["med"].data_ptr(), tzf_bar.data_ptr(),
                         tzi_bar.data_ptr(), zbar[b].data_ptr(), s)
        if geo.shared:
            # the height tables depend on the shared column (sample 0, column (0, 0)): their gradient goes there, on
            # the device in FP64, spread over the column's (mode, node) pairs
            self._column_tables_vjp(hgt, D, tzf_bar, tzi_bar, zbar[0], H * W)
        flags = [ws.err] + ([state["err"]] if state.get("err") is not None else [])
        if errs is None:
            self.check_flags(flags)
        else:
            errs.extend(flags)
        return xbar_in, zbar

    def _gn_bwd(self, ws, gb, mode, u, r, pre, gamma, beta, name, pbar):
        m = self.model
        C, V, s = m.width, ws.V, _stream()
        G = self._packed.groups
        nat.call("ffno_gn_bwd_stats", mode, u.data_ptr(), r, pre.data_ptr(), gamma.data_ptr(), beta.data_ptr(),
                 ws.gstats[name].data_ptr(), V, C, G, gb.bpart.data_ptr(), ws.nparts, s)
        nat.call("ffno_gn_bwd_final", gb.bpart.data_ptr(), ws.nparts, G, gb.sums.data_ptr(), s)
        nat.call("ffno_gn_bwd_apply", mode, u.data_ptr(), r, pre.data_ptr(), gamma.data_ptr(), beta.data_ptr(),
                 ws.gstats[name].data_ptr(), gb.sums.data_ptr(), ws.dw.data_ptr(), V, C, G, EPS, pbar.data_ptr(),
                 gb.wbar.data_ptr(), s)

    @staticmethod
    def _column_tables_vjp(hgt, D, tzf_bar, tzi_bar, zbar, stride):
        """z_bar[j * stride] += the gradient of the shared grid's height tables (along tzf_bar, tzi_bar) w.r.t. its
        column's heights (ffno_column_tables_vjp)."""
        hv, live = hgt["vjp"], hgt["live"]
        scratch = torch.empty(3 * live * D, dtype=torch.float64, device=tzf_bar.device)
        nat.call("ffno_column_tables_vjp", hv["z"].data_ptr(), D, hv["k"].data_ptr(), live, hv["f"].data_ptr(),
                 hv["df"].data_ptr(), hv["med_i"], tzf_bar.data_ptr(), tzi_bar.data_ptr(), scratch.data_ptr(),
                 zbar.data_ptr(), stride, _stream())

    def _block_bwd(self, pk, ws, gb, i, x, z, zbar, D, H, W, hgt, pln, fq, tzf_bar, tzi_bar):
        """gb.xbar (gradient of the block output) -> gb.xbar (gradient of the block input x); accumulates the
        depth-weight gradient in gb.wbar, the z_proj gradient in zbar and the height-table gradients."""
        m = self.model
        C, V, HW, Wf = m.width, ws.V, H * W, W // 2 + 1
        s = _stream()
        bp = pk.blocks[i]
        r_f, r_pw, r_mlp = bp["res"]
        live = hgt["live"]
        d = _descs(D, H, W, C, live)
        tc, tc_chan, fuse96 = self._tc(), self._tc_chan(), self._tc_fuse96()
        err = ws.err.data_ptr()

        def mlp_bwd(a, pb, base, out, w1, w2t, w1t, pack):
            if tc_chan:
                nat.call("ffno_mlp2_bwd_tc", a.data_ptr(), pb.data_ptr(), _ptr(base), V, C, bp[pack].data_ptr(),
                         out.data_ptr(), err, s)
            else:
                nat.call("ffno_mlp2_bwd", a.data_ptr(), pb.data_ptr(), _ptr(base), V, C, bp[w1].data_ptr(),
                         bp[w2t].data_ptr(), bp[w1t].data_ptr(), out.data_ptr(), s)

        # out = x2 + r_mlp GN(mlp_pre); mlp_pre = mlp(x2)
        self._gn_bwd(ws, gb, 0, gb.xbar, r_mlp, ws.mlp_pre, bp["mlp_g"], bp["mlp_b"], "mlp", gb.pbar)
        mlp_bwd(ws.x2, gb.pbar, gb.xbar, gb.g2, "m1", "m2t", "m1t", "tcb_mlp")
        # x2 = x1 + r_pw GN(pw_pre); pw_pre = pw(x1)
        self._gn_bwd(ws, gb, 0, gb.g2, r_pw, ws.pw_pre, bp["pw_g"], bp["pw_b"], "pw", gb.pbar)
        mlp_bwd(ws.x1, gb.pbar, gb.g2, gb.g1, "pw1", "pw2t", "pw1t", "tcb_pw")
        # GELU after a GroupNorm: the tensor-core forward applies the A&S activation (mode 2), the FP32 one erf's; the
        # fuse norm's GELU is applied by the pw MLP's prologue, the spec / vert norms' by the fusion
        act = 2 if tc or fuse96 else 1
        # x1 = x + r_f gelu(GN(fused_pre)); fused_pre = fuse(x, spec, vert)
        self._gn_bwd(ws, gb, 2 if tc_chan else 1, gb.g1, r_f, ws.fused_pre, bp["fuse_g"], bp["fuse_b"], "fuse",
                     gb.pbar)
        if tc:
            hg = ws.hg                     # gates and hidden layer kept from the forward, else recomputed
            if hg is None:
                hg = gb.hg
                self._fuse1_tc(ws, bp, x, hg)
            cs, cv = ws.coefs["spec"].data_ptr(), ws.coefs["vert"].data_ptr()
            nat.call("ffno_fuse_bwd_a_tc", ws.spec_pre.data_ptr(), cs, ws.vert_pre.data_ptr(), cv,
                     ws.gates.data_ptr(), gb.pbar.data_ptr(), V, C, bp["tcb_fuse_a"].data_ptr(), gb.hfb.data_ptr(),
                     err, s)
            nat.call("ffno_fuse_bwd_b_tc", ws.spec_pre.data_ptr(), cs, ws.vert_pre.data_ptr(), cv,
                     ws.gates.data_ptr(), hg.data_ptr(), gb.pbar.data_ptr(), gb.hfb.data_ptr(), gb.g1.data_ptr(),
                     V, C, bp["tcb_fuse_b"].data_ptr(), gb.xacc.data_ptr(), gb.sbar.data_ptr(), gb.vbar.data_ptr(),
                     err, s)
        elif fuse96:
            sp, cs, vp, cv = (ws.spec_pre.data_ptr(), ws.coefs["spec"].data_ptr(), ws.vert_pre.data_ptr(),
                              ws.coefs["vert"].data_ptr())
            # the gates and hf are this block's (kept from the forward, or just recomputed into ws by it); the gate
            # hidden layer hg is kept only by a caching forward, else recomputed here
            hg, hf = ws.hg, ws.hf
            if hg is None:
                hg = gb.hg
                self._fuse1_tc(ws, bp, x, hg)
            nat.call("ffno_fuse_bwd_h_tc", gb.pbar.data_ptr(), hf.data_ptr(), V, C, bp["tc_f2"].data_ptr(),
                     gb.hfb.data_ptr(), err, s)
            nat.call("ffno_fuse_bwd_q_tc", sp, cs, vp, cv, ws.gates.data_ptr(), gb.pbar.data_ptr(), gb.hfb.data_ptr(),
                     V, C, bp["tc_f1"].data_ptr(), gb.sbar.data_ptr(), gb.vbar.data_ptr(), gb.hfb.data_ptr(), err, s)
            nat.call("ffno_fuse_bwd_x_tc", gb.hfb.data_ptr(), hg.data_ptr(), gb.g1.data_ptr(), V, C,
                     bp["tc_fuse1"].data_ptr(), gb.xacc.data_ptr(), gb.sbar.data_ptr(), gb.vbar.data_ptr(), err, s)
        else:
            nat.call("ffno_fuse_bwd", x.data_ptr(), ws.spec_pre.data_ptr(), ws.coefs["spec"].data_ptr(),
                     ws.vert_pre.data_ptr(), ws.coefs["vert"].data_ptr(), gb.pbar.data_ptr(), gb.g1.data_ptr(), V, C,
                     bp["bg1"].data_ptr(), bp["bg2"].data_ptr(), bp["bgb"].data_ptr(), bp["f1"].data_ptr(),
                     bp["f2t"].data_ptr(), bp["f1t"].data_ptr(), bp["bg2t"].data_ptr(), bp["bg1t"].data_ptr(),
                     gb.xacc.data_ptr(), gb.sbar.data_ptr(), gb.vbar.data_ptr(), s)
        # spec = gelu(GN(spec_pre)), spec_pre = post_s(ys); vert likewise
        self._gn_bwd(ws, gb, act, gb.sbar, 1.0, ws.spec_pre, bp["spec_g"], bp["spec_b"], "spec", gb.pbar)
        mlp_bwd(ws.ys, gb.pbar, None, gb.ysb, "s_p1", "s_p2t", "s_p1t", "tcb_s_post")
        self._gn_bwd(ws, gb, act, gb.vbar, 1.0, ws.vert_pre, bp["vert_g"], bp["vert_b"], "vert", gb.pbar)
        mlp_bwd(ws.yv, gb.pbar, None, gb.yvb, "v_p1", "v_p2t", "v_p1t", "tcb_v_post")
        # horizontal transposes: ys = twi thi mix thf twf xs  ->  xs_bar = twf^T thf^T mix^T thi^T twi^T ys_bar
        self._xf(pln, "twi_t", gb.ysb, ws.sa, d["wf"], ws)
        self._xf(pln, "thi_t", ws.sa, ws.sb, d["hf"], ws)
        self._mix(ws, "s", bp, fq, ws.sb, ws.sa, H * Wf, D, C, 2 * H * Wf * C, H * Wf * C, True)
        self._xf(pln, "thf_t", ws.sa, ws.sb, d["hf"], ws)
        self._xf(pln, "twf_t", ws.sb, gb.xsb, d["wi"], ws)
        # vertical transposes (ws.vb holds the mixed modes, ws.xv the transform input)
        hq = hgt["freq"][i]
        N = HW * C
        if hgt.get("percol"):
            nat.call("ffno_col_outer", gb.yvb.data_ptr(), D, ws.vb.data_ptr(), 2 * live, HW, C, N,
                     tzi_bar.data_ptr(), 1, s)
            nat.call("ffno_xform_pt", hgt["tzi_t"].data_ptr(), 2 * live * D, gb.yvb.data_ptr(), ws.va.data_ptr(),
                     d["pcf"], 0, s)
            self._mix(ws, "v", bp, hq, ws.va, ws.vb, live, HW, HW * C, C, live * HW * C, True)
            nat.call("ffno_col_outer", ws.vb.data_ptr(), 2 * live, ws.xv.data_ptr(), D, HW, C, N,
                     tzf_bar.data_ptr(), 1, s)
            nat.call("ffno_xform_pt", hgt["tzf_t"].data_ptr(), 2 * live * D, ws.vb.data_ptr(), gb.xvb.data_ptr(),
                     d["pci"], 0, s)
        else:
            self._outer(ws, gb.yvb, D, ws.vb, 2 * live, N, gb.opart, gb.osplit_i, tzi_bar)
            self._xf(hgt, "tzi_t", gb.yvb, ws.va, d["zf"], ws)
            self._mix(ws, "v", bp, hq, ws.va, ws.vb, live, HW, HW * C, C, live * HW * C, True)
            self._outer(ws, ws.vb, 2 * live, ws.xv, D, N, gb.opart, gb.osplit_f, tzf_bar)
            self._xf(hgt, "tzf_t", ws.vb, gb.xvb, d["zi"], ws)
        # input gates (and z_proj)
        if tc_chan:
            nat.call("ffno_gate_bwd_tc", x.data_ptr(), gb.xsb.data_ptr(), gb.xacc.data_ptr(), V, C,
                     bp["tcb_s_gate"].data_ptr(), None, gb.xbar.data_ptr(), None, err, s)
            nat.call("ffno_gate_bwd_tc", x.data_ptr(), gb.xvb.data_ptr(), gb.xbar.data_ptr(), V, C,
                     bp["tcb_v_gate"].data_ptr(), bp["v_zp"].data_ptr(), gb.xbar.data_ptr(), zbar.data_ptr(), err, s)
        else:
            nat.call("ffno_gate_bwd", x.data_ptr(), gb.xsb.data_ptr(), gb.xvb.data_ptr(), gb.xacc.data_ptr(), V, C,
                     bp["s_g1"].data_ptr(), bp["s_g2"].data_ptr(), bp["s_g2t"].data_ptr(), bp["s_g1t"].data_ptr(),
                     bp["v_g1"].data_ptr(), bp["v_g2"].data_ptr(), bp["v_g2t"].data_ptr(), bp["v_g1t"].data_ptr(),
                     bp["v_zp"].data_ptr(), gb.xbar.data_ptr(), zbar.data_ptr(), s)


class _GradBuffers:
    def __init__(self, D, H, W, C, live, groups, nparts, device):
        V = D * H * W
        f32 = dict(dtype=torch.float32, device=device)
        for n in ("xbar", "g2", "g1", "xacc", "sbar", "vbar", "pbar", "hg"):
            setattr(self, n, torch.empty(V, C, **f32))
        self.hfb = torch.empty(V, 2 * C, **f32)
        # within a block's VJP g2 and g1 are dead (after the pw and fuse stages) before the branch post-MLP gradients
        # ysb, yvb are written, and hg, hfb (fuse stage) before the transform gradients xsb, xvb
        self.ysb, self.yvb = self.g2, self.g1
        self.xsb, self.xvb = self.hg, self.hfb.reshape(-1)[:V * C].view(V, C)
        self.wbar = torch.zeros(V, **f32)
        self.bpart = torch.empty(max(nparts, 1) * groups * 2, dtype=torch.float64, device=device)
        self.sums = torch.empty(groups * 2, dtype=torch.float64, device=device)
        N = H * W * C
        lib = nat.lib()
        self.osplit_i = lib.ffno_outer_parts(D, 2 * live, N)
        self.osplit_f = lib.ffno_outer_parts(2 * live, D, N)
        need = max(self.osplit_i, self.osplit_f) * D * 2 * live
        plan = _outer_tc_slices(D, 2 * live)
        if plan is not None and len(plan) > 1:      # one split per SM for each sliced tensor-core call
            need = max(need, _sm_count(device) * max(r for _, r in plan) * min(D, 2 * live))
        self.opart = torch.empty(need, **f32)


class _TangentBuffers:
    """Tangent twins of the forward intermediates of one cube (JVP), with buffers whose lives do not overlap
    sharing storage."""

    def __init__(self, D, H, W, C, live, groups, nparts, device):
        V, HW, Wf = D * H * W, H * W, W // 2 + 1
        f32 = dict(dtype=torch.float32, device=device)
        nb = lambda *s: torch.empty(*s, **f32)
        for n in ("x", "xp", "xs", "xv", "yv", "spec_pre", "vert_pre", "sd", "vd", "fused", "x1", "x2"):
            setattr(self, n, nb(V, C))
        self.pre = self.spec_pre      # the lift tangent is dead before block 0 writes spec_pre
        self.ys = self.xs             # xs is dead once the W transform has read it
        self.pw = self.spec_pre       # spec_pre (and its GN tangent sd) are consumed by the fuse tangent
        self.mlp = self.vert_pre
        spec_len = D * 2 * H * Wf * C
        self.sa, self.sb = nb(spec_len), nb(spec_len)
        self.va, self.vb = nb(2 * live * HW * C), nb(2 * live * HW * C)
        self.parts = torch.empty(max(nparts, 1) * groups * 2, dtype=torch.float64, device=device)
        self.sums = torch.empty(groups * 2, dtype=torch.float64, device=device)
        self.scratch_parts = torch.empty(max(nparts, 1) * groups * 3, dtype=torch.float64, device=device)


def _outer_tc_slices(ma, mb):
    """The calls ffno_outer_tc makes of an [ma][mb] product: (first row, rows) of the longer side per call, TI tiles of
    128 rows each, NB = the shorter side rounded up to 16 (the MMA's N), with TI NB <= 512 accumulator columns and
    one k-chunk stage of (128 TI + NB) x 64 split-BF16 operands within shared memory ((128 TI + NB) <= 900); None when
    the shorter side exceeds 256."""
    lo, hi = min(ma, mb), max(ma, mb)
    nb = (lo + 15) // 16 * 16
    if nb > 256:
        return None
    rows = 128 * min(512 // nb, (900 - nb) // 128)
    return [(r0, min(rows, hi - r0)) for r0 in range(0, hi, rows)]


_SMS = {}


def _sm_count(device):
    device = torch.device(device)
    if device.type != "cuda":
        return 1
    idx = device.index if device.index is not None else torch.cuda.current_device()
    if idx not in _SMS:
        _SMS[idx] = torch.cuda.get_device_properties(idx).multi_processor_count
    return _SMS[idx]


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
    d["hf"] = XD(nb=D, nb2=1, in_b1=2 * H * Wf * C, in_b2=0, out_b1=2 * H * Wf * C, out_b2=0, K=2 * H, M=2 * H,
                 N=Wf * C, in_split=big, in_hi=0, in_lo=Wf * C, out_split=big, out_hi=0, out_lo=Wf * C)
    # c2r along W: [2][Wf] rows -> [W][C]
    d["wi"] = XD(nb=D * H, nb2=H, in_b1=2 * H * Wf * C, in_b2=Wf * C, out_b1=H * W * C, out_b2=W * C,
                 K=2 * Wf, M=W, N=C, in_split=Wf, in_hi=H * Wf * C, in_lo=C, out_split=big, out_hi=0, out_lo=C)
    # height transform [D][HW*C] -> [2M'][HW*C] and back
    d["zf"] = XD(nb=1, nb2=1, in_b1=0, in_b2=0, out_b1=0, out_b2=0, K=D, M=2 * live, N=HW * C,
                 in_split=big, in_hi=0, in_lo=HW * C, out_split=big, out_hi=0, out_lo=HW * C)
    d["zi"] = XD(nb=1, nb2=1, in_b1=0, in_b2=0, out_b1=0, out_b2=0, K=2 * live, M=D, N=HW * C,
                 in_split=big, in_hi=0, in_lo=HW * C, out_split=big, out_hi=0, out_lo=HW * C)
    # per-column height transforms (a table per column, batch = column, n = channel)
    d["pcf"] = XD(nb=HW, nb2=1, in_b1=C, in_b2=0, out_b1=C, out_b2=0, K=D, M=2 * live, N=C,
                  in_split=big, in_hi=0, in_lo=HW * C, out_split=big, out_hi=0, out_lo=HW * C)
    d["pci"] = XD(nb=HW, nb2=1, in_b1=C, in_b2=0, out_b1=C, out_b2=0, K=2 * live, M=D, N=C,
                  in_split=big, in_hi=0, in_lo=HW * C, out_split=big, out_hi=0, out_lo=HW * C)
    return d


class _FFNOFunction(torch.autograd.Function):
    """FFNO3D.forward with the hand-written input VJP."""

    @staticmethod
    def forward(ctx, x, z_scale, executor, dx, dy):
        y, state = executor.forward(x, z_scale, dx, dy, keep=True)
        executor.check_forward(state)        # the caller may never run the backward
        ctx.executor = executor
        ctx.state = state
        return y

    @staticmethod
    def backward(ctx, ybar):
        xbar, zbar = ctx.executor.backward(ctx.state, ybar)
        ctx.state = None
        return xbar, zbar, None, None, None


def ffno_apply(model, x, z_scale, dx, dy):
    """FFNO3D.forward on the GB300 path; differentiable in x and z_scale (reverse mode: autograd) and in x (forward
    mode: a dual x under torch.autograd.forward_ad gives a dual output, as the reference's jvp_local uses it)."""
    import torch.autograd.forward_ad as fwAD
    if z_scale.ndim == 5:
        z_scale = z_scale[:, 0]
    dx = _spacing(dx)
    dy = _spacing(dy)
    ex = model.executor()
    x_primal, x_tangent = fwAD.unpack_dual(x)
    z_primal, z_tangent = fwAD.unpack_dual(z_scale)
    if x_tangent is not None or z_tangent is not None:
        if z_tangent is not None:
            raise NotImplementedError("forward-mode derivatives along z_scale are not supported (heights are fixed)")
        if torch.is_grad_enabled() and (x_primal.requires_grad or z_primal.requires_grad):
            raise NotImplementedError("forward- and reverse-mode derivatives in one call are not supported")
        y, y_dot = ex.jvp(x_primal, z_primal, dx, dy, x_tangent.float())
        return fwAD.make_dual(y, y_dot)
    if torch.is_grad_enabled() and (x.requires_grad or z_scale.requires_grad):
        return _FFNOFunction.apply(x, z_scale, ex, dx, dy)
    y, _ = ex.forward(x, z_scale, dx, dy)
    return y


def _spacing(v):
    """_to_spacing_value (models/ffno_model.py:11-18)."""
    if isinstance(v, (float, int)):
        return float(v)
    if torch.is_tensor(v):
        if v.numel() != 1:
            raise ValueError("spacing must be scalar.")
        return float(v.detach().item())
    raise TypeError(f"Unsupported spacing type: {type(v)}")


# ------------------------------------------------------------------------------------------------ module pieces
# FFNO3D._run_lift, _run_head and head_output (models/ffno_model.py:785-798, 730-749) on their own, for the reference's
# callers that compose the model from them (ffno_batched_backend.py:280-283, FFNONet.py:1419, 1478). Each runs the
# CUDA kernels of the whole-model path and is differentiable through the same hand-written backward kernels. The
# lift output (the hidden state [B, C, D, H, W]) is a channels-first view of channels-last storage, the layout the
# kernels use; _run_head takes such a view without a copy.

class _LiftSpace:
    """The buffers of one cube's lift (a Workspace's lift-related subset)."""

    def __init__(self, V, C, groups, device):
        f32 = dict(dtype=torch.float32, device=device)
        self.V = V
        self.nparts = nat.lib().ffno_stats_parts(V)
        self.dw = torch.empty(V, **f32)
        self.pre = torch.empty(V, C, **f32)
        self.partials = torch.empty(max(self.nparts, 1) * groups * 3, dtype=torch.float64, device=device)
        self.coefs = {"lift": torch.empty(3 * C, **f32)}
        self.gstats = {"lift": torch.empty(groups * 3, dtype=torch.float64, device=device)}


def _check_cuda_f32(*ts):
    for t in ts:
        if not t.is_cuda:
            raise RuntimeError("ffnoml_gb300 runs on CUDA tensors only")
        if t.dtype != torch.float32:
            raise TypeError("ffnoml_gb300 FFNO3D takes float32 inputs")


def _channels_last(h):
    """[B, C, D, H, W] -> its channels-last storage [B, D, H, W, C] (no copy when h is already a view of it)."""
    cl = h.permute(0, 2, 3, 4, 1)
    return cl if cl.is_contiguous() else cl.contiguous()


def run_lift(ex, x, z_scale):
    """_run_lift forward: x [B, Cin, D, H, W], z_scale [B, D, H, W] -> (hidden [B, C, D, H, W] view, per-cube lift
    spaces for the backward)."""
    m = ex.model
    _check_cuda_f32(x, z_scale)
    if x.dim() != 5 or x.shape[1] != m.in_channels or z_scale.shape != (x.shape[0],) + tuple(x.shape[2:]):
        raise ValueError(f"x must be [B, {m.in_channels}, D, H, W] and z_scale [B, D, H, W]; got {tuple(x.shape)}, "
                         f"{tuple(z_scale.shape)}")
    x, z_scale = x.contiguous(), z_scale.contiguous()
    pk = ex.packed(x.device)
    B, _, D, H, W = x.shape
    V, C = D * H * W, m.width
    out = torch.empty(B, D, H, W, C, dtype=torch.float32, device=x.device)
    spaces = []
    for b in range(B):
        ls = _LiftSpace(V, C, pk.groups, x.device)
        nat.call("ffno_depth_weights", z_scale[b].data_ptr(), D, H * W, ls.dw.data_ptr(), _stream())
        ex._lift(pk, _LiftOut(ls, out[b]), x[b])
        spaces.append(ls)
    return out.permute(0, 4, 1, 2, 3), spaces


class _LiftOut:
    """A lift space whose output row buffer is a given [V][C] view (what Executor._lift writes to as ws.x)."""

    def __init__(self, ls, x):
        self.__dict__.update(ls.__dict__)
        self.x = x


def run_lift_bwd(ex, x, z_scale, spaces, hbar):
    """_run_lift backward: hbar [B, C, D, H, W] -> (x_bar [B, Cin, D, H, W], z_bar [B, D, H, W])."""
    m = ex.model
    pk = ex.packed(x.device)
    B, Cin, D, H, W = x.shape
    V, C, HW = D * H * W, m.width, H * W
    z_scale = z_scale.contiguous()
    hb = _channels_last(hbar.float())
    xbar = torch.zeros(B, Cin, D, H, W, dtype=torch.float32, device=x.device)
    zbar = torch.zeros(B, D, H, W, dtype=torch.float32, device=x.device)
    s = _stream()
    G = pk.groups
    for b, ls in enumerate(spaces):
        bpart = torch.empty(max(ls.nparts, 1) * G * 2, dtype=torch.float64, device=x.device)
        sums = torch.empty(G * 2, dtype=torch.float64, device=x.device)
        pbar = torch.empty(V, C, dtype=torch.float32, device=x.device)
        wbar = torch.zeros(V, dtype=torch.float32, device=x.device)
        u = hb[b]
        nat.call("ffno_gn_bwd_stats", 1, u.data_ptr(), 1.0, ls.pre.data_ptr(), pk.lift_g.data_ptr(),
                 pk.lift_b.data_ptr(), ls.gstats["lift"].data_ptr(), V, C, G, bpart.data_ptr(), ls.nparts, s)
        nat.call("ffno_gn_bwd_final", bpart.data_ptr(), ls.nparts, G, sums.data_ptr(), s)
        nat.call("ffno_gn_bwd_apply", 1, u.data_ptr(), 1.0, ls.pre.data_ptr(), pk.lift_g.data_ptr(),
                 pk.lift_b.data_ptr(), ls.gstats["lift"].data_ptr(), sums.data_ptr(), ls.dw.data_ptr(), V, C, G, EPS,
                 pbar.data_ptr(), wbar.data_ptr(), s)
        nat.call("ffno_lift_bwd", pbar.data_ptr(), Cin, V, C, pk.lift_w.data_ptr(), xbar[b].data_ptr(), s)
        nat.call("ffno_depth_weights_bwd", z_scale[b].data_ptr(), wbar.data_ptr(), D, HW, zbar[b].data_ptr(), s)
    return xbar, zbar


def run_head(ex, h):
    """_run_head forward: hidden [B, C, D, H, W] -> head channels [B, nh, D, H, W] = proj2(gelu(proj1(h)))."""
    m = ex.model
    _check_cuda_f32(h)
    if h.dim() != 5 or h.shape[1] != m.width:
        raise ValueError(f"expected the hidden state [B, {m.width}, D, H, W], got {tuple(h.shape)}")
    pk = ex.packed(h.device)
    cl = _channels_last(h)
    B, D, H, W, C = cl.shape
    V = D * H * W
    out = torch.empty(B, pk.nh, D, H, W, dtype=torch.float32, device=h.device)
    for b in range(B):
        nat.call("ffno_proj_fwd", cl[b].data_ptr(), V, C, pk.p1.data_ptr(), pk.p2.data_ptr(), pk.b2.data_ptr(), pk.nh,
                 pk.nhp, out[b].data_ptr(), _stream())
    return out


def run_head_bwd(ex, h, gbar):
    """_run_head backward: gbar [B, nh, D, H, W] -> h_bar [B, C, D, H, W] (a channels-first view)."""
    pk = ex.packed(h.device)
    cl = _channels_last(h)
    B, D, H, W, C = cl.shape
    V = D * H * W
    gbar = gbar.float().contiguous()
    hbar = torch.empty(B, D, H, W, C, dtype=torch.float32, device=h.device)
    for b in range(B):
        nat.call("ffno_proj_bwd", cl[b].data_ptr(), gbar[b].data_ptr(), V, C, pk.p1.data_ptr(), pk.p2.data_ptr(),
                 pk.b2.data_ptr(), pk.p2t.data_ptr(), pk.p1t.data_ptr(), pk.nh, pk.nhp, hbar[b].data_ptr(),
                 _stream())
    return hbar.permute(0, 4, 1, 2, 3)


def _head_params_for(ex, device):
    pk = ex.packed(device)
    return pk, (pk.head32 if ex.model.precision == "bf16" else pk.head)


def head_output(ex, head, x_in):
    """head_output forward: head channels [B, nh, D, H, W], normalised inputs x_in [B, Cin, D, H, W] -> normalised
    log10 n [B, L, D, H, W]. The FP32 path evaluates the LTE weights and log-softmax in FP64 as the reference does;
    precision 'bf16' in FP32 with a compensated sum."""
    m = ex.model
    _check_cuda_f32(head, x_in)
    pk, hp = _head_params_for(ex, head.device)
    if head.dim() != 5 or head.shape[1] != pk.nh or x_in.dim() != 5 or x_in.shape[1] != m.in_channels or \
            head.shape[0] != x_in.shape[0] or head.shape[2:] != x_in.shape[2:]:
        raise ValueError(f"head_output takes head [B, {pk.nh}, D, H, W] and x_in [B, {m.in_channels}, D, H, W]; got "
                         f"{tuple(head.shape)}, {tuple(x_in.shape)}")
    head, x_in = head.contiguous(), x_in.contiguous()
    B = head.shape[0]
    V = head[0, 0].numel()
    out = torch.empty(B, m.out_channels, *head.shape[2:], dtype=torch.float32, device=head.device)
    for b in range(B):
        nat.call("ffno_head_output", head[b].data_ptr(), x_in[b].data_ptr(), V, pk.nh, hp, out[b].data_ptr(),
                 _stream())
    return out


def head_output_bwd(ex, head, x_in, ybar):
    pk, hp = _head_params_for(ex, head.device)
    head, x_in, ybar = head.contiguous(), x_in.contiguous(), ybar.float().contiguous()
    B = head.shape[0]
    V = head[0, 0].numel()
    hbar = torch.empty_like(head)
    xbar = torch.empty_like(x_in)
    for b in range(B):
        nat.call("ffno_head_output_bwd", head[b].data_ptr(), x_in[b].data_ptr(), ybar[b].data_ptr(), V, pk.nh, hp,
                 hbar[b].data_ptr(), xbar[b].data_ptr(), _stream())
    return hbar, xbar


class _LiftFunction(torch.autograd.Function):
    @staticmethod
    def forward(ctx, x, z_scale, ex):
        h, spaces = run_lift(ex, x, z_scale)
        ctx.ex, ctx.spaces = ex, spaces
        ctx.save_for_backward(x, z_scale)
        return h

    @staticmethod
    def backward(ctx, hbar):
        x, z_scale = ctx.saved_tensors
        xbar, zbar = run_lift_bwd(ctx.ex, x, z_scale, ctx.spaces, hbar)
        ctx.spaces = None
        return xbar, zbar, None


class _HeadFunction(torch.autograd.Function):
    @staticmethod
    def forward(ctx, h, ex):
        ctx.ex = ex
        ctx.save_for_backward(h)
        return run_head(ex, h)

    @staticmethod
    def backward(ctx, gbar):
        (h,) = ctx.saved_tensors
        return run_head_bwd(ctx.ex, h, gbar), None


class _HeadOutputFunction(torch.autograd.Function):
    @staticmethod
    def forward(ctx, head, x_in, ex):
        ctx.ex = ex
        ctx.save_for_backward(head, x_in)
        return head_output(ex, head, x_in)

    @staticmethod
    def backward(ctx, ybar):
        head, x_in = ctx.saved_tensors
        hbar, xbar = head_output_bwd(ctx.ex, head, x_in, ybar)
        return hbar, xbar, None


def _needs_grad(*ts):
    return torch.is_grad_enabled() and any(t.requires_grad for t in ts)


def lift_apply(model, x, z_scale):
    if z_scale.ndim == 5:
        z_scale = z_scale[:, 0]
    ex = model.executor()
    if _needs_grad(x, z_scale):
        return _LiftFunction.apply(x, z_scale, ex)
    return run_lift(ex, x, z_scale)[0]


def head_apply(model, h):
    ex = model.executor()
    if _needs_grad(h):
        return _HeadFunction.apply(h, ex)
    return run_head(ex, h)


def head_output_apply(model, head, x_in):
    ex = model.executor()
    if _needs_grad(head, x_in):
        return _HeadOutputFunction.apply(head, x_in, ex)
    return head_output(ex, head, x_in)
