"""The drop-in module's pieces that the reference's own callers compose (ffno_batched_backend.py:280-283,
FFNONet.py:1419, 1478): head_output, _run_lift and _run_head run the CUDA kernels, against the reference's float64
head (tests/golden/head.npz) and the float64 oracle, with their VJPs; and the level-fraction head's shares add up to
one per voxel within 1e-6 in both precisions."""
import math

import numpy as np
import pytest
import torch

from golden_io import ATOMS, load, model_config

pytestmark = pytest.mark.gpu

HEAD_CFG = dict(width=16, n_layers=1, hidden_spectral=16, hidden_vertical=16, z_min_wavelength=0.5)


def _head_model(precision):
    from ffnoml_gb300 import FFNO3D
    meta, state, a = load("head")
    cfg = model_config(dict(HEAD_CFG, atoms=meta["atoms"]))
    m = FFNO3D(**cfg)
    m.load_state_dict({k: v.float() for k, v in state.items()}, strict=True)
    return m.cuda().eval().set_precision(precision), state, cfg, a


@pytest.mark.parametrize("precision", ["fp32", "bf16"])
def test_head_output_matches_reference(precision):
    from oracle.ffno_oracle import OracleFFNO3D
    model, state, cfg, a = _head_model(precision)
    head, x = a["head"].float(), a["x"].float()
    y = model.head_output(head.cuda(), x.cuda()).double().cpu()
    err = (y - a["y64"]).abs().max().item()
    # the same float32 head channels through the float64 oracle: the FP32 path keeps the head in FP64, so it differs
    # from it by the rounding of the float32 output only
    ref = OracleFFNO3D(state, cfg, torch.float64).head(head.double(), x.double())
    err_rounded = ((y - ref).abs() / ref.abs().clamp_min(1.0)).max().item()
    print(f"{precision}: head_output max |d| vs reference {err:.2e}, vs float64 on the same inputs {err_rounded:.2e}")
    assert err < 1e-5
    # FP32 path: the head in FP64, so only the output's rounding (half an ulp); BF16 path: the head in FP32
    assert err_rounded <= (2.0 ** -23 if precision == "fp32" else 1e-5)


@pytest.mark.parametrize("precision", ["fp32", "bf16"])
def test_head_output_vjp_matches_oracle(precision):
    from oracle.ffno_oracle import OracleFFNO3D
    model, state, cfg, a = _head_model(precision)
    head, x = a["head"].float(), a["x"].float()
    cot = torch.randn(a["y64"].shape, generator=torch.Generator().manual_seed(4), dtype=torch.float64)
    hc, xc = head.cuda().requires_grad_(True), x.cuda().requires_grad_(True)
    model.head_output(hc, xc).backward(cot.float().cuda())
    oracle = OracleFFNO3D(state, cfg, torch.float64)
    hr, xr = head.double().requires_grad_(True), x.double().requires_grad_(True)
    hb, xb = torch.autograd.grad(oracle.head(hr, xr), (hr, xr), cot)
    eh = ((hc.grad.double().cpu() - hb).abs().max() / hb.abs().max()).item()
    ex = ((xc.grad.double().cpu() - xb).abs().max() / xb.abs().max()).item()
    print(f"{precision}: head_output VJP rel error: head {eh:.2e}, x_in {ex:.2e}")
    assert eh < 1e-5 and ex < 1e-5


@pytest.mark.parametrize("precision", ["fp32", "bf16"])
def test_lift_and_head_compose_like_the_reference(precision):
    """head_output(_run_head(_run_lift(x, z)), x) against the oracle's float64 lift, projection and head, forward and
    VJP in x and z (the composition FFNONet.py:1419-1478 uses, without the blocks)."""
    from oracle.ffno_oracle import OracleFFNO3D
    meta, state, a = load("w32_m16")
    cfg = model_config(meta)
    from ffnoml_gb300 import FFNO3D
    model = FFNO3D(**cfg)
    model.load_state_dict({k: v.float() for k, v in state.items()}, strict=True)
    model = model.cuda().eval().set_precision(precision)
    x = a["x"].float().cuda().requires_grad_(True)
    z = a["z"].float().cuda().requires_grad_(True)
    h = model._run_lift(x, z)
    assert h.shape == (1, cfg["width"]) + tuple(x.shape[2:])
    heads = model._run_head(h)
    y = model.head_output(heads, x)
    cot = torch.randn(y.shape, generator=torch.Generator().manual_seed(6), dtype=torch.float64)
    y.backward(cot.float().cuda())
    oracle = OracleFFNO3D(state, cfg, torch.float64)
    xr, zr = a["x"].double().requires_grad_(True), a["z"].double().requires_grad_(True)
    h64 = oracle.lift(xr, zr)
    heads64 = oracle.proj(h64)
    y64 = oracle.head(heads64, xr)
    xb, zb = torch.autograd.grad(y64, (xr, zr), cot)
    rel = lambda p, q: ((p.double().cpu() - q).abs().max() / q.abs().max()).item()
    e_h, e_p = rel(h.detach(), h64.detach()), rel(heads.detach(), heads64.detach())
    e_y = (y.detach().double().cpu() - y64.detach()).abs().max().item()
    e_x, e_z = rel(x.grad, xb), rel(z.grad, zb)
    print(f"{precision}: lift {e_h:.2e}, proj {e_p:.2e}, head |d| {e_y:.2e}, x_bar {e_x:.2e}, z_bar {e_z:.2e}")
    assert e_h < 1e-5 and e_p < 1e-5 and e_y < 1e-5
    assert e_x < 1e-4 and e_z < 1e-3


def _share_setup(V, seed, nh_std=1.0):
    """Head channels and inputs for the level-share check: T, ne from the synthetic distributions, rho fixed at
    1e-8 kg m^-3 (its normalised value 0), mean_Y per level = log10(rho / m_species), std_Y = 1, so that each output is
    log10 share + the total term s (a few units: the float32 output rounding stays near 1e-7 dex)."""
    from ffnoml_gb300 import FFNO3D
    cfg = model_config(dict(HEAD_CFG, atoms=["H", "CA"]))
    torch.manual_seed(seed)
    model = FFNO3D(**cfg)
    with torch.no_grad():
        for c in (6, 13):                        # the species' total-correction rows, zero at initialisation
            model.proj2.weight[c].normal_(0.0, 0.3)
            model.proj2.bias[c].normal_(0.0, 0.3)
    g = torch.Generator().manual_seed(seed)
    mean_x = np.array([4.75, 0, 0, 0, 17.5, -8.0], np.float32)
    std_x = np.array([2.5 / math.sqrt(12), 5, 5, 5, 7 / math.sqrt(12), 8 / math.sqrt(12)], np.float32)
    masses = [ATOMS["H"]["log10_particle_mass"], ATOMS["CA"]["log10_particle_mass"]]
    mean_y = np.array([-8.0 - m for m in masses for _ in range(6)])
    model.set_normalization(mean_x, std_x, mean_y, np.ones(12))
    x = torch.empty(6, V)
    x[0] = (3.5 + 2.5 * torch.rand(V, generator=g) - 4.75) / (2.5 / math.sqrt(12))
    x[1:4] = torch.randn(3, V, generator=g)
    x[4] = (14 + 7 * torch.rand(V, generator=g) - 17.5) / (7 / math.sqrt(12))
    x[5] = 0.0
    head = nh_std * torch.randn(14, V, generator=g)
    return model.cuda().eval(), x, head, masses


def _share_sums(y, head, model):
    """Per voxel and species sum_i 10^(log10 n_i) / (rho / m 10^s), from the normalised outputs y [12][V] and the head
    channels [14][V]: log10 n_i = y_i std_Y + mean_Y and log10 rho - log10 m with the model's own float32 buffers,
    in float64 arithmetic."""
    y = y.double().cpu()
    head = head.double().cpu()
    mean_y, std_y = model.mean_Y.double().cpu()[:, None], model.std_Y.double().cpu()[:, None]
    log10_n = y * std_y + mean_y
    log10_rho = float(model.mean_X[5].double())          # the inputs' normalised rho channel is 0
    tb = model.total_bound
    sums = []
    for s in range(2):
        u = head[7 * s + 6]
        base = log10_rho - float(model.log10_particle_mass[s].double()) + tb * torch.tanh(u / tb)
        sums.append(torch.pow(10.0, log10_n[6 * s:6 * s + 6] - base[None]).sum(0))
    return torch.stack(sums)


@pytest.mark.parametrize("precision", ["fp32", "bf16"])
@pytest.mark.parametrize("V", [4096, 256 * 128 * 128], ids=["small", "config1_cube"])
def test_level_shares_sum_to_one_head_output(precision, V):
    model, x, head, _ = _share_setup(V, 11)
    model.set_precision(precision)
    y = model.head_output(head.reshape(1, 14, V, 1, 1).cuda(), x.reshape(1, 6, V, 1, 1).cuda())
    err = (_share_sums(y.reshape(12, V), head, model) - 1.0).abs().max().item()
    print(f"{precision} V={V}: max |sum of shares - 1| = {err:.2e}")
    assert err <= 1e-6


@pytest.mark.parametrize("precision", ["fp32", "bf16"])
def test_level_shares_sum_to_one_model_head_kernels(precision):
    """The same property of the whole-model head kernels (proj1, proj2 and the head in one kernel: ffno_head_fwd on
    the FP32 path, ffno_head_fwd_tc on the split-BF16 path), called through the C ABI with their head-channel
    output, on a config-1-sized cube of random hidden states."""
    from ffnoml_gb300 import _native as nat
    V = 256 * 128 * 128
    model, x, _, _ = _share_setup(V, 12)
    model.set_precision(precision)
    ex = model.executor()
    pk = ex.packed(torch.device("cuda"))
    C = model.width
    hidden = torch.randn(V, C, generator=torch.Generator().manual_seed(13)).cuda()
    xin = x.cuda().contiguous()
    out = torch.empty(12, V, device="cuda")
    head = torch.empty(pk.nh, V, device="cuda")
    err = torch.zeros(1, dtype=torch.int32, device="cuda")
    s = torch.cuda.current_stream().cuda_stream
    if precision == "bf16" and pk.tc:
        nat.call("ffno_head_fwd_tc", hidden.data_ptr(), xin.data_ptr(), V, C, pk.tc_head.data_ptr(), pk.b2.data_ptr(),
                 pk.nh, pk.nhp, pk.head32, out.data_ptr(), head.data_ptr(), err.data_ptr(), s)
    else:
        nat.call("ffno_head_fwd", hidden.data_ptr(), xin.data_ptr(), V, C, pk.p1.data_ptr(), pk.p2.data_ptr(),
                 pk.b2.data_ptr(), pk.nh, pk.nhp, pk.head, out.data_ptr(), head.data_ptr(), s)
    torch.cuda.synchronize()
    assert int(err.item()) == 0
    e = (_share_sums(out, head, model) - 1.0).abs().max().item()
    print(f"{precision}: whole-model head kernel, max |sum of shares - 1| = {e:.2e}")
    assert e <= 1e-6
