"""GPU parity of the forward-mode derivative (JVP): the model called on a dual input (torch.autograd.forward_ad, as
the reference's jvp_local calls it) against the float64 oracle's forward-mode derivative on the golden cases, and the
service-level jvp_local against the oracle at SI level."""
import numpy as np
import pytest
import torch
import torch.autograd.forward_ad as fwAD

from golden_io import CASES, load, model_config

pytestmark = pytest.mark.gpu


def _model(meta, state, precision="fp32"):
    from ffnoml_gb300 import FFNO3D
    m = FFNO3D(**model_config(meta))
    m.load_state_dict({k: v.float() for k, v in state.items()}, strict=True)
    return m.cuda().eval().set_precision(precision)


def _tangent(shape, seed):
    return torch.randn(shape, generator=torch.Generator().manual_seed(seed), dtype=torch.float64)


def _dual_forward(model, x, z, meta, xd):
    with torch.no_grad(), fwAD.dual_level():
        y = model(fwAD.make_dual(x.float().cuda(), xd.float().cuda()), z.float().cuda(), meta["dx"], meta["dy"])
        yp, yt = fwAD.unpack_dual(y)
        return yp.double().cpu(), yt.double().cpu()


@pytest.mark.parametrize("name", CASES)
def test_jvp_matches_the_float64_oracle(name):
    from oracle.ffno_oracle import OracleFFNO3D, jvp
    meta, state, a = load(name)
    model = _model(meta, state)
    xd = _tangent(a["x"].shape, 7)
    y, yd = _dual_forward(model, a["x"], a["z"], meta, xd)
    oracle = OracleFFNO3D({k: v.double() for k, v in state.items()}, model_config(meta), torch.float64)
    _, ref = jvp(oracle, a["x"].double(), a["z"].double(), meta["dx"], meta["dy"], xd)
    err = ((yd - ref).abs().max() / ref.abs().max()).item()
    print(f"{name}: JVP rel {err:.2e}")
    assert (y - a["y64"]).abs().max().item() < 1e-5       # the primal of the dual call is the FP32 forward
    assert err < 1e-4                                      # FP32 forward-mode derivative vs float64


def test_jvp_runs_in_fp32_whatever_the_model_precision():
    meta, state, a = load("w64_m32")
    xd = _tangent(a["x"].shape, 9)
    _, t32 = _dual_forward(_model(meta, state, "fp32"), a["x"], a["z"], meta, xd)
    _, t16 = _dual_forward(_model(meta, state, "bf16"), a["x"], a["z"], meta, xd)
    assert torch.equal(t32, t16)


def test_jvp_local_matches_the_oracle_at_si_level():
    from ffnoml_gb300.runtime import GB300Backend
    from oracle.ffno_oracle import OracleFFNO3D, jvp_si
    meta, state, a = load("hca_stretched")
    cfg = model_config(meta)
    model = _model(meta, state)
    backend = GB300Backend(model, [f"l{i}" for i in range(model.out_channels)])
    g = np.random.default_rng(5)
    _, _, D, H, W = a["x"].shape
    feat = np.empty((6, D, H, W), np.float32)
    feat[0] = 10.0 ** g.uniform(3.6, 5.5, (D, H, W))
    feat[1:4] = g.normal(0.0, 4e3, (3, D, H, W))
    feat[4] = g.uniform(15.0, 20.0, (D, H, W))
    feat[5] = g.uniform(-11.0, -5.0, (D, H, W))
    z = (a["z"][0].numpy() * 1e6).astype(np.float32)
    tan = np.empty_like(feat)
    tan[0] = feat[0] * g.normal(0.0, 0.01, (D, H, W))
    tan[1:4] = g.normal(0.0, 50.0, (3, D, H, W))
    tan[4:6] = g.normal(0.0, 0.01, (2, D, H, W))
    got = backend.jvp_local(feat, z, meta["dx"], meta["dy"], tan)
    oracle = OracleFFNO3D({k: v.double() for k, v in state.items()}, cfg, torch.float64)
    _, ref = jvp_si(oracle, torch.from_numpy(feat).double()[None], torch.from_numpy(z).double()[None], meta["dx"],
                    meta["dy"], torch.from_numpy(tan).double()[None])
    ref = ref[0].permute(1, 2, 3, 0).numpy()               # (nz, nx, ny, L)
    scale = np.abs(ref).max(axis=(0, 1, 2), keepdims=True)  # per level: populations span many decades
    err = float((np.abs(got - ref) / scale).max())
    print(f"jvp_local rel {err:.2e}")
    assert got.shape == ref.shape and err < 1e-4
