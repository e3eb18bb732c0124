"""The oracle (oracle/ffno_oracle.py) against the reference's own float64 outputs and VJPs (tests/golden/)."""
import pytest
import torch

from golden_io import CASES, load, model_config
from oracle.ffno_oracle import OracleFFNO3D, jvp, lte_tables, vjp


@pytest.mark.parametrize("name", CASES)
def test_oracle_forward_matches_reference(name):
    meta, state, a = load(name)
    oracle = OracleFFNO3D(state, model_config(meta), torch.float64)
    with torch.no_grad():
        y = oracle.forward(a["x"], a["z"], meta["dx"], meta["dy"])
    assert (y - a["y64"]).abs().max().item() < 1e-10


@pytest.mark.parametrize("name", CASES)
def test_oracle_vjp_matches_reference(name):
    meta, state, a = load(name)
    oracle = OracleFFNO3D(state, model_config(meta), torch.float64)
    _, xb, zb = vjp(oracle, a["x"], a["z"], meta["dx"], meta["dy"], a["cot"])
    assert ((xb - a["xbar"]).abs().max() / a["xbar"].abs().max()).item() < 1e-9
    assert ((zb - a["zbar"]).abs().max() / a["zbar"].abs().max()).item() < 1e-8


def test_oracle_float32_is_within_the_reference_float32_envelope():
    meta, state, a = load("w32_m16")
    oracle = OracleFFNO3D(state, model_config(meta), torch.float32)
    with torch.no_grad():
        y = oracle.forward(a["x"].float(), a["z"].float(), meta["dx"], meta["dy"]).double()
    ref_err = (a["y32"] - a["y64"]).abs().max().item()
    assert (y - a["y64"]).abs().max().item() < max(2 * ref_err, 1e-5)


def test_head_matches_reference():
    meta, state, a = load("head")
    cfg = model_config(dict(width=16, n_layers=1, hidden_spectral=16, hidden_vertical=16, z_min_wavelength=0.5,
                            atoms=meta["atoms"]))
    oracle = OracleFFNO3D(state, cfg, torch.float64)
    y = oracle.head(a["head"], a["x"])
    assert (y - a["y64"]).abs().max().item() < 1e-12


def test_lte_debye_stage_table():
    # MULTI3D's ndxi after the shift by ion_1 (models/ffno_model.py:121-128): H (ion 1, 2) and Ca II (ion 2, 3)
    _, _, ndxi_h, dion_h = lte_tables(dict(g=[2.0, 1.0], ev=[0.0, 13.6], ion=[1, 2]), 2)
    assert ndxi_h == [0.0, 1.0] and dion_h == [0.0, 1.0]
    _, _, ndxi_ca, dion_ca = lte_tables(dict(g=[2.0, 1.0], ev=[0.0, 11.9], ion=[2, 3]), 2)
    assert ndxi_ca == [0.0, 3.0] and dion_ca == [0.0, 1.0]


@pytest.mark.parametrize("name", ["h_uniform", "batch2"])
def test_oracle_jvp_matches_central_differences(name):
    # the forward-mode derivative along a random direction against (f(x + h d) - f(x - h d)) / 2h in float64
    meta, state, a = load(name)
    oracle = OracleFFNO3D(state, model_config(meta), torch.float64)
    x, z = a["x"].double(), a["z"].double()
    d = torch.randn(x.shape, generator=torch.Generator().manual_seed(3), dtype=torch.float64)
    _, yd = jvp(oracle, x, z, meta["dx"], meta["dy"], d)
    h = 1e-5
    with torch.no_grad():
        fd = (oracle.forward(x + h * d, z, meta["dx"], meta["dy"])
              - oracle.forward(x - h * d, z, meta["dx"], meta["dy"])) / (2 * h)
    assert ((yd - fd).abs().max() / yd.abs().max()).item() < 1e-6


@pytest.mark.parametrize("name", ["tall_box", "per_column"])
def test_oracle_jvp_is_the_transpose_of_the_vjp(name):
    # <cot, J d> == <J^T cot, d>: the forward- and reverse-mode derivatives of the oracle are one Jacobian
    meta, state, a = load(name)
    oracle = OracleFFNO3D(state, model_config(meta), torch.float64)
    x, z = a["x"].double(), a["z"].double()
    d = torch.randn(x.shape, generator=torch.Generator().manual_seed(5), dtype=torch.float64)
    _, yd = jvp(oracle, x, z, meta["dx"], meta["dy"], d)
    _, xb, _ = vjp(oracle, x, z, meta["dx"], meta["dy"], a["cot"].double())
    lhs, rhs = (a["cot"].double() * yd).sum().item(), (xb * d).sum().item()
    assert abs(lhs - rhs) <= 1e-10 * max(abs(lhs), abs(rhs))


def test_oracle_si_level_matches_the_reference_service_conversions():
    # tests/golden/si_hca.npz: the reference's _model_inputs / linear_populations around its FFNO3D, float64
    from oracle.ffno_oracle import jvp_si
    meta, state, a = load("si_hca")
    oracle = OracleFFNO3D(state, model_config(meta), torch.float64)
    f, z, dx, dy = a["features"][None], a["z_m"][None], meta["dx"], meta["dy"]
    canon = lambda t: t[0].permute(1, 2, 3, 0)                  # (nz, nx, ny, L) as predict_local returns it
    fr, zr = f.clone().requires_grad_(True), z.clone().requires_grad_(True)
    pops = canon(oracle.forward_si(fr, zr, dx, dy))
    assert ((pops - a["pops"]).abs() / a["pops"]).max().item() < 1e-10
    fb, zb = torch.autograd.grad(pops, (fr, zr), a["cot"])
    for got, ref in ((fb[0], a["features_bar"]), (zb[0], a["z_bar"])):
        for c in range(ref.shape[0] if ref.dim() == 4 else 1):     # per feature: their units differ by decades
            g, r = (got[c], ref[c]) if ref.dim() == 4 else (got, ref)
            assert ((g - r).abs().max() / r.abs().max()).item() < 1e-9
    _, pdot = jvp_si(oracle, f, z, dx, dy, a["tangent"][None])
    # per element, relative to the population (the tangent of ln n): populations span 34 decades
    assert ((canon(pdot) - a["pops_dot"]).abs() / a["pops"]).max().item() < 1e-9


# ------------------------------------------------------------------------------------------------ recipe fixtures
def _recipe_oracle(meta, dtype):
    from golden_io import recipe_model
    state = {k: v.detach().clone() for k, v in recipe_model(meta, device="cpu").state_dict().items()}
    return OracleFFNO3D(state, model_config(meta), dtype)


@pytest.mark.parametrize("name", ["cfg0", "cfg3_fd", "w96_p_d64", "w96_p_d256", "w64_p_d256"])
def test_oracle_matches_reference_at_benchmark_architectures(name):
    """The oracle against the reference's float64 forward and VJP on the benchmark models (the recipe's weights are
    reproduced bit for bit first: recipe_model checks the fixture's digest)."""
    from golden_io import load_recipe
    meta, a = load_recipe(name)
    oracle = _recipe_oracle(meta, torch.float64)
    y, xb, zb = vjp(oracle, a["x"], a["z"], meta["dx"], meta["dy"], a["cot"])
    assert (y - a["y64"]).abs().max().item() < 1e-10
    assert ((xb - a["xbar"]).abs().max() / a["xbar"].abs().max()).item() < 1e-9
    assert ((zb - a["zbar"]).abs().max() / a["zbar"].abs().max()).item() < 1e-8
