"""FFNO3D drop-in: the reference module's parameter tree and call signature (harshmathur1990/FFNOML,
models/ffno_model.py:614-832), computed by the sm_103a kernels of libffnoml_gb300 through ffnoml_gb300.executor.

The parameter and buffer names, shapes, creation order and initialisation follow the reference exactly, so that
  - load_state_dict(reference_checkpoint["model_state"], strict=True) works (ffno_fsdp_runtime.py:155), and
  - torch.manual_seed(s) followed by construction gives the same weights as the reference's constructor.
The forward pass never runs these submodules: they are parameter containers. forward(x, z_scale, dx, dy) packs the
weights into device buffers (once per weight version) and runs the CUDA path; its input VJP is the hand-written
backward of ffnoml_gb300.executor behind a torch.autograd.Function.
"""
import math

import torch
import torch.nn as nn

from . import lte


def _group_count(channels, max_groups=8):
    g = min(max_groups, channels)
    while g > 1 and channels % g != 0:
        g -= 1
    return g


class DepthWeightedGroupNorm(nn.GroupNorm):
    """Parameter container with nn.GroupNorm's parameters (models/ffno_model.py:77-95); normalisation runs in the
    kernels."""


def _wgn(channels):
    return DepthWeightedGroupNorm(_group_count(channels), channels)


class PointwiseMLP(nn.Module):
    """models/ffno_model.py:147-160: net = Conv3d, GELU, Identity (dropout 0), Conv3d."""

    def __init__(self, width, expansion=3, dropout=0.0):
        super().__init__()
        hidden = width * expansion
        self.net = nn.Sequential(nn.Conv3d(width, hidden, 1, bias=False), nn.GELU(),
                                 nn.Dropout(dropout) if dropout > 0 else nn.Identity(),
                                 nn.Conv3d(hidden, width, 1, bias=False))


class HeightSpectralConv(nn.Module):
    """Parameters of the vertical branch (models/ffno_model.py:166-309)."""

    def __init__(self, channels, reference_length, min_wavelength, feature_wavelength, hidden=128, rank=0):
        super().__init__()
        if reference_length <= 0 or min_wavelength <= 0 or feature_wavelength <= 0:
            raise ValueError("the height operator needs z_reference_length, z_min_wavelength and z_feature_wavelength > 0")
        self.reference_length = float(reference_length)
        self.min_wavelength = float(min_wavelength)
        self.feature_wavelength = float(feature_wavelength)
        self.modes = int(math.floor(self.reference_length / self.min_wavelength)) + 1
        self.rank = int(rank)
        scale = 1.0 / math.sqrt(channels)
        self.weight_real = nn.Parameter(scale * torch.randn(channels, channels))
        self.weight_imag = nn.Parameter(scale * torch.randn(channels, channels))
        self.input_gate = nn.Sequential(nn.Conv3d(channels, channels, 1, bias=False), nn.GELU(),
                                        nn.Conv3d(channels, channels, 1, bias=False), nn.Sigmoid())
        self.z_proj = nn.Conv3d(1, channels, 1, bias=False)
        self.freq_mlp = nn.Sequential(nn.Linear(2, hidden), nn.GELU(), nn.Linear(hidden, hidden), nn.GELU(),
                                      nn.Linear(hidden, 2))
        if self.rank:
            self.freq_lowrank = nn.Sequential(nn.Linear(2, hidden), nn.GELU(), nn.Linear(hidden, hidden), nn.GELU())
            self.freq_u = nn.Linear(hidden, channels * self.rank)
            self.freq_v = nn.Linear(hidden, self.rank * channels)
            with torch.no_grad():
                self.freq_u.weight.zero_()
                self.freq_u.bias.zero_()
        self.post = nn.Sequential(nn.Conv3d(channels, 2 * channels, 1, bias=False), nn.GELU(),
                                  nn.Conv3d(2 * channels, channels, 1, bias=False))
        k = 2 * math.pi * torch.arange(self.modes, dtype=torch.float32) / self.reference_length
        self.register_buffer("k", k, persistent=False)
        self.register_buffer("mode_factor", torch.cat([torch.ones(1), 2 * torch.ones(self.modes - 1)]),
                             persistent=False)


class SpectralConv2dFull(nn.Module):
    """Parameters of the horizontal branch (models/ffno_model.py:315-373)."""

    def __init__(self, in_channels, out_channels, hidden=128, post_mix_expansion=2, rank=0):
        super().__init__()
        self.rank = int(rank)
        scale = 1.0 / math.sqrt(in_channels)
        self.weight_real = nn.Parameter(scale * torch.randn(in_channels, out_channels, dtype=torch.float32))
        self.weight_imag = nn.Parameter(scale * torch.randn(in_channels, out_channels, dtype=torch.float32))
        self.input_gate = nn.Sequential(nn.Conv3d(in_channels, in_channels, 1, bias=False), nn.GELU(),
                                        nn.Conv3d(in_channels, in_channels, 1, bias=False), nn.Sigmoid())
        self.freq_mlp = nn.Sequential(nn.Linear(4, hidden), nn.GELU(), nn.Linear(hidden, hidden), nn.GELU(),
                                      nn.Linear(hidden, 2))
        if self.rank:
            self.freq_lowrank = nn.Sequential(nn.Linear(4, hidden), nn.GELU(), nn.Linear(hidden, hidden), nn.GELU())
            self.freq_u = nn.Linear(hidden, out_channels * self.rank)
            self.freq_v = nn.Linear(hidden, self.rank * in_channels)
            with torch.no_grad():
                self.freq_u.weight.zero_()
                self.freq_u.bias.zero_()
        post_hidden = out_channels * post_mix_expansion
        self.post = nn.Sequential(nn.Conv3d(out_channels, post_hidden, 1, bias=False), nn.GELU(),
                                  nn.Conv3d(post_hidden, out_channels, 1, bias=False))


class FFNOBlock3dBalanced(nn.Module):
    """Parameters of one block (models/ffno_model.py:456-522)."""

    def __init__(self, width=96, dropout=0.0, spec_dropout=0.0, vertical_dropout=0.0, hidden_spectral=128,
                 hidden_vertical=128, freq_mix_rank=8, z_reference_length=40.0, z_min_wavelength=0.04,
                 z_feature_wavelength=0.3):
        super().__init__()
        self.spec = SpectralConv2dFull(width, width, hidden=hidden_spectral, post_mix_expansion=2, rank=freq_mix_rank)
        self.vertical = HeightSpectralConv(width, z_reference_length, z_min_wavelength, z_feature_wavelength,
                                           hidden=hidden_vertical, rank=freq_mix_rank)
        self.pw = nn.Sequential(nn.Conv3d(width, width * 2, 1, bias=False), nn.GELU(),
                                nn.Conv3d(width * 2, width, 1, bias=False))
        self.mlp = PointwiseMLP(width, expansion=2, dropout=dropout)
        self.norm_spec = _wgn(width)
        self.norm_vert = _wgn(width)
        self.branch_gate = nn.Sequential(nn.Conv3d(3 * width, width, 1, bias=False), nn.GELU(),
                                         nn.Conv3d(width, 2 * width, 1, bias=True), nn.Sigmoid())
        self.fuse = nn.Sequential(nn.Conv3d(2 * width, 2 * width, 1, bias=False), nn.GELU(),
                                  nn.Conv3d(2 * width, width, 1, bias=False))
        self.norm_fuse = _wgn(width)
        self.norm_pw = _wgn(width)
        self.norm_mlp = _wgn(width)
        self.res_fused = nn.Parameter(torch.tensor([1.0]))
        self.res_pw = nn.Parameter(torch.tensor([0.5]))
        self.res_mlp = nn.Parameter(torch.tensor([0.5]))
        self.act = nn.GELU()
        self.spec_drop = nn.Dropout(spec_dropout) if spec_dropout > 0 else nn.Identity()
        self.vert_drop = nn.Dropout(vertical_dropout) if vertical_dropout > 0 else nn.Identity()


def _layer_dropout(rate, layers, index):
    if not layers:
        return 0.0
    return float(rate) if index in set(layers) else 0.0


class FFNO3D(nn.Module):
    """Drop-in for the reference FFNO3D (models/ffno_model.py:614-832) computed on GB300.

    forward(x, z_scale, dx, dy, collect_stats=False, branch_mask=None):
      x [B, Cin, D, H, W] normalised inputs, z_scale [B, D, H, W] or [B, 1, D, H, W] heights in Mm, dx, dy spacings in
      metres (float or one-element tensor) -> [B, L, D, H, W] normalised log10 populations. Differentiable in x and
      z_scale. The diagnostic arguments collect_stats / branch_mask of the reference's training code are not part of
      this path and raise NotImplementedError.
    Inputs must be CUDA float32 tensors (precision="fp32") — the reference's dtype; the optional precision="bf16"
    runs the GEMM operands in bfloat16 with float32 accumulation."""

    def __init__(self, in_channels=6, out_channels=6, width=96, n_layers=4, dropout=0.0, spec_dropout=0.0,
                 vertical_dropout=0.0, spec_dropout_layers=None, vertical_dropout_layers=None, checkpoint_blocks=True,
                 hidden_spectral=128, hidden_vertical=128, freq_mix_rank=8, z_reference_length=40.0,
                 z_min_wavelength=0.04, z_feature_wavelength=0.3, species=None, rho_channel=5, total_bound=6.0,
                 temperature_channel=0, ne_channel=4):
        super().__init__()
        if not species:
            raise ValueError("FFNO3D needs species (config.ATOM_CONFIG: levels, log10_particle_mass, multi3d_lte)")
        self.species_levels = [int(s["levels"]) for s in species]
        if sum(self.species_levels) != out_channels:
            raise ValueError(f"species levels {self.species_levels} do not add up to out_channels={out_channels}")
        head_channels = out_channels + len(self.species_levels)
        self.total_bound = float(total_bound)
        self.rho_channel = int(rho_channel)
        self.register_buffer("log10_particle_mass",
                             torch.tensor([float(s["log10_particle_mass"]) for s in species], dtype=torch.float32))
        self.register_buffer("mean_X", torch.zeros(in_channels))
        self.register_buffer("std_X", torch.ones(in_channels))
        self.register_buffer("mean_Y", torch.zeros(out_channels))
        self.register_buffer("std_Y", torch.ones(out_channels))
        missing = [i for i, s in enumerate(species) if "multi3d_lte" not in s]
        if missing:
            raise ValueError(f"the level-fraction head needs each species' multi3d_lte atom data (g, ev, ion); "
                             f"missing for {missing}")
        self.temperature_channel, self.ne_channel = int(temperature_channel), int(ne_channel)
        tables = [lte.tables(s["multi3d_lte"], s["levels"]) for s in species]
        self.lte_tables = tuple([v for t in tables for v in t[i]] for i in range(4))
        self.checkpoint_blocks = checkpoint_blocks
        self.external_block_checkpointing = False
        self.in_channels, self.out_channels, self.width, self.n_layers = in_channels, out_channels, width, n_layers
        self.freq_mix_rank = int(freq_mix_rank)
        self.z_reference_length = float(z_reference_length)
        self.z_min_wavelength = float(z_min_wavelength)
        self.z_feature_wavelength = float(z_feature_wavelength)
        self.lift = nn.Sequential(nn.Conv3d(in_channels, width, 1, bias=False), _wgn(width), nn.GELU())
        self.blocks = nn.ModuleList([
            FFNOBlock3dBalanced(width=width, dropout=dropout,
                                spec_dropout=_layer_dropout(spec_dropout, spec_dropout_layers, i),
                                vertical_dropout=_layer_dropout(vertical_dropout, vertical_dropout_layers, i),
                                hidden_spectral=hidden_spectral, hidden_vertical=hidden_vertical,
                                freq_mix_rank=freq_mix_rank, z_reference_length=z_reference_length,
                                z_min_wavelength=z_min_wavelength, z_feature_wavelength=z_feature_wavelength)
            for i in range(n_layers)])
        self.proj1 = nn.Conv3d(width, width * 2, 1, bias=False)
        self.proj2 = nn.Conv3d(width * 2, head_channels, 1)
        with torch.no_grad():
            c = 0
            for levels in self.species_levels:
                self.proj2.weight[c + levels].zero_()
                self.proj2.bias[c + levels].zero_()
                c += levels + 1
        self.act = nn.GELU()
        self.precision = "fp32"
        self._executor = None

    def set_normalization(self, mean_X, std_X, mean_Y, std_Y):
        """Copy the dataset's normalisation into the head (models/ffno_model.py:724-728)."""
        for name, value in (("mean_X", mean_X), ("std_X", std_X), ("mean_Y", mean_Y), ("std_Y", std_Y)):
            buffer = getattr(self, name)
            buffer.copy_(torch.as_tensor(value, dtype=buffer.dtype).broadcast_to(buffer.shape))

    def set_precision(self, precision):
        """'fp32' (the reference's arithmetic, the default) or 'bf16' (bfloat16 GEMM operands, float32 accumulation,
        float32 residual stream, statistics and head)."""
        if precision not in ("fp32", "bf16"):
            raise ValueError(precision)
        self.precision = precision
        return self

    def executor(self):
        from .executor import Executor
        if self._executor is None:
            self._executor = Executor(self)
        return self._executor

    def _check_mode(self, collect_stats=False, branch_mask=None):
        if collect_stats or branch_mask is not None:
            raise NotImplementedError("collect_stats / branch_mask are training diagnostics outside this path")
        if self.training and any(isinstance(mod, nn.Dropout) and mod.p > 0 for mod in self.modules()):
            # the reference applies its dropout layers in training mode (models/ffno_model.py:519-521, 155); this
            # path computes the inference operator only, so it refuses rather than return eval-mode results
            raise RuntimeError("this FFNO3D has dropout layers and is in training mode; the GB300 path computes the "
                               "inference operator only: call model.eval() first")

    def head_output(self, head, x_in):
        """Normalised log10 populations from the head channels [B, L+S, D, H, W] and the normalised inputs x_in
        [B, Cin, D, H, W] (models/ffno_model.py:730-749), on the GPU; differentiable in both."""
        from .executor import head_output_apply
        return head_output_apply(self, head, x_in)

    def _run_lift(self, x, z_scale, collect_stats=False):
        """gelu(DepthWeightedGroupNorm(lift(x), depth_weights(z_scale))) (models/ffno_model.py:782-788): the hidden
        state [B, width, D, H, W], a channels-first view of channels-last storage; differentiable in x and z_scale."""
        self._check_mode(collect_stats)
        from .executor import lift_apply
        return lift_apply(self, x, z_scale)

    def _run_head(self, x, collect_stats=False):
        """proj2(gelu(proj1(x))) (models/ffno_model.py:790-798): the head channels [B, L+S, D, H, W] of the hidden
        state x [B, width, D, H, W]; differentiable in x."""
        self._check_mode(collect_stats)
        from .executor import head_apply
        return head_apply(self, x)

    def forward(self, x, z_scale, dx, dy, collect_stats=False, branch_mask=None):
        self._check_mode(collect_stats, branch_mask)
        from .executor import ffno_apply
        return ffno_apply(self, x, z_scale, dx, dy)
