"""The host-RAM streaming forward (hidden states in pinned host memory, the cube on the device a depth slab or a slab of
column rows at a time) against the resident forward through the service backend: the same kernels on the same
voxels, with GroupNorm statistics merged over the slabs' partials instead of the whole cube's, so the populations
agree to rounding (ffno_batched_backend.py's own chunking test allows 2e-4)."""
import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


def _model(width, precision):
    import bench
    from ffnoml_gb300 import create_ffno3d
    torch.manual_seed(3)
    m = create_ffno3d(6, 12, atoms=["H", "CA"], width=width, n_layers=2, z_min_wavelength=40.0 / 15)
    with torch.no_grad():
        for name, p in m.named_parameters():
            if ".freq_u." in name:
                p.normal_(0.0, 0.1)
    m.set_normalization(bench.MEAN_X, bench.STD_X, np.zeros(12), np.ones(12))
    return m.cuda().eval().set_precision(precision)


@pytest.mark.parametrize("width,precision,tol", [(32, "fp32", 1e-4), (64, "fp32", 1e-4), (64, "bf16", 2e-3),
                                                 (96, "bf16", 2e-3)])
def test_streaming_matches_resident(width, precision, tol):
    import bench
    from ffnoml_gb300.runtime import GB300Backend
    from ffnoml_gb300.streaming import StreamingForward
    model = _model(width, precision)
    f, z = bench.synthetic_si((37, 24, 20), seed=5)
    ref = GB300Backend(model, [f"l{i}" for i in range(12)]).predict_local(f, z, 48e3, 48e3)
    sf = StreamingForward(model, chunk_depth=8, chunk_rows=7)
    got = sf(f, z, 48e3, 48e3)
    assert got.shape == ref.shape == (37, 24, 20, 12)
    assert sf.slabs > 2 * 5 * 6            # several depth slabs and row slabs per block stage
    err = np.abs(np.log10(got) - np.log10(ref)).max()
    print(f"w{width} {precision}: max |dlog10 n| streaming vs resident {err:.2e}")
    assert err < tol


def test_streaming_rejects_bad_shapes():
    from ffnoml_gb300.streaming import StreamingForward
    sf = StreamingForward(_model(32, "fp32"))
    with pytest.raises(ValueError):
        sf(np.zeros((5, 4, 4, 4), np.float32), np.zeros((4, 4, 4), np.float32), 1.0, 1.0)


def test_streaming_backend_log10_and_si():
    """predict_log10 (model units in, de-normalised log10 n out) against the resident model, and predict_si."""
    import bench
    from ffnoml_gb300.streaming import StreamingBackend
    model = _model(32, "fp32")
    f, z = bench.synthetic_si((19, 16, 12), seed=7)
    x, zmm = bench.normalised(f, z)
    with torch.no_grad():
        ref = model(torch.from_numpy(x).cuda(), torch.from_numpy(zmm).cuda(), 48e3, 48e3)[0].cpu().numpy()
    sb = StreamingBackend(model, [f"l{i}" for i in range(12)], chunk_depth=4, chunk_rows=5)
    units = f.astype(np.float64).copy()
    units[0] = np.log10(units[0])
    units[1:4] /= 1e3
    got = sb.predict_log10(units, z / 1e6, 48e3, 48e3)
    assert got.shape == (12, 19, 16, 12)
    assert np.abs(got - ref).max() < 1e-4
    pop = sb.predict_si(f, z, 48e3, 48e3)
    assert np.abs(np.log10(pop) - got.transpose(1, 2, 3, 0)).max() < 1e-4
    with pytest.raises(ValueError):
        bad = f.copy()
        bad[0, 0, 0, 0] = -1.0
        sb.predict_si(bad, z, 48e3, 48e3)


def _rel_per_channel(got, ref):
    """max over the feature channels of max |got - ref| / max |ref| (their SI units differ by decades)."""
    return max(float(np.abs(got[c] - ref[c]).max() / np.abs(ref[c]).max()) for c in range(ref.shape[0]))


@pytest.mark.parametrize("width,precision,tol", [(32, "fp32", 1e-4), (64, "fp32", 1e-4), (64, "bf16", 1e-2),
                                                 (96, "bf16", 1e-2)])
def test_streaming_vjp_matches_resident(width, precision, tol):
    """The streaming VJP (block inputs in pinned host memory, blocks recomputed and back-propagated slab by slab)
    against the resident VJP through the service backend: the same kernels on the same voxels; only the GroupNorm
    sums' merge order differs."""
    import bench
    from ffnoml_gb300.runtime import GB300Backend
    from ffnoml_gb300.streaming import StreamingVJP
    model = _model(width, precision)
    f, z = bench.synthetic_si((23, 14, 10), seed=9)
    cot = np.random.default_rng(10).normal(size=(23, 14, 10, 12)).astype(np.float32)
    pop = GB300Backend(model, [f"l{i}" for i in range(12)]).predict_local(f, z, 48e3, 48e3)
    cot = cot / pop                          # the cotangent of ln n, as the inversion's gradients scale
    ref = GB300Backend(model, [f"l{i}" for i in range(12)]).vjp_local(f, z, 48e3, 48e3, cot)
    sv = StreamingVJP(model, chunk_depth=6, chunk_rows=4)
    got = sv(f, z, 48e3, 48e3, cot)
    assert got["features"].shape == (6, 23, 14, 10) and got["z_scale"].shape == (23, 14, 10)
    ef = _rel_per_channel(got["features"], ref["features"])
    ez = float(np.abs(got["z_scale"] - ref["z_scale"]).max() / np.abs(ref["z_scale"]).max())
    print(f"w{width} {precision}: streaming vs resident VJP: features {ef:.2e}, z {ez:.2e}, {sv.slabs} slabs")
    assert ef < tol
    assert ez < 10 * tol


def test_streaming_vjp_against_the_float64_oracle():
    """The streaming VJP in FP32 against the float64 oracle's SI-level VJP (its forward_si through autograd)."""
    import bench
    from ffnoml_gb300.config import species_of
    from ffnoml_gb300.streaming import StreamingBackend
    from oracle.ffno_oracle import OracleFFNO3D
    model = _model(32, "fp32")
    f, z = bench.synthetic_si((17, 10, 12), seed=11)
    state = {k: v.detach().cpu().clone() for k, v in model.state_dict().items()}
    cfg = dict(width=32, n_layers=2, z_min_wavelength=40.0 / 15, species=species_of(["H", "CA"]), in_channels=6,
               out_channels=12)
    oracle = OracleFFNO3D({k: v.double() for k, v in state.items()}, cfg, torch.float64)
    fr = torch.from_numpy(f.astype(np.float64))[None].requires_grad_(True)
    zr = torch.from_numpy(z.astype(np.float64))[None].requires_grad_(True)
    pops = oracle.forward_si(fr, zr, 48e3, 48e3)[0].permute(1, 2, 3, 0)
    cot = (np.random.default_rng(12).normal(size=pops.shape) / pops.detach().numpy()).astype(np.float32)
    fb, zb = torch.autograd.grad(pops, (fr, zr), torch.from_numpy(cot.astype(np.float64)))
    sb = StreamingBackend(model, [f"l{i}" for i in range(12)], chunk_depth=5, chunk_rows=3)
    got = sb.vjp_local(f, z, 48e3, 48e3, cot)
    ef = _rel_per_channel(got["features"], fb[0].numpy())
    ez = float(np.abs(got["z_scale"] - zb[0].numpy()).max() / np.abs(zb[0].numpy()).max())
    print(f"streaming VJP vs float64 oracle: features {ef:.2e}, z {ez:.2e}")
    assert ef < 1e-4
    assert ez < 1e-3


def _per_column_si(shape, seed):
    """SI features and heights [m] whose columns each have their own grid (stretched and shifted per column)."""
    import bench
    f, z = bench.synthetic_si(shape, seed=seed)
    zc = bench.per_column_heights(torch.from_numpy(z / 1e6)[None])[0].numpy() * 1e6
    return f, zc.astype(np.float32)


@pytest.mark.parametrize("precision,tol,vtol", [("fp32", 1e-4, 1e-4), ("bf16", 2e-3, 1e-2)])
def test_streaming_per_column_grids_match_resident(precision, tol, vtol):
    """Per-column height grids (every column its own tables): the streaming forward and VJP, row slabs addressing
    their own columns' tables and table gradients, against the resident path through the service backend."""
    from ffnoml_gb300.runtime import GB300Backend
    from ffnoml_gb300.streaming import StreamingForward, StreamingVJP
    model = _model(32, precision)
    f, z = _per_column_si((21, 12, 10), seed=13)
    ex = model.executor()
    assert not ex.geometry_host((z / np.float32(1e6))[None]).shared
    names = [f"l{i}" for i in range(12)]
    ref = GB300Backend(model, names).predict_local(f, z, 48e3, 48e3)
    got = StreamingForward(model, chunk_depth=6, chunk_rows=5)(f, z, 48e3, 48e3)
    err = np.abs(np.log10(got) - np.log10(ref)).max()
    cot = (np.random.default_rng(14).normal(size=ref.shape) / ref).astype(np.float32)
    vref = GB300Backend(model, names).vjp_local(f, z, 48e3, 48e3, cot)
    vgot = StreamingVJP(model, chunk_depth=6, chunk_rows=5)(f, z, 48e3, 48e3, cot)
    ef = _rel_per_channel(vgot["features"], vref["features"])
    ez = float(np.abs(vgot["z_scale"] - vref["z_scale"]).max() / np.abs(vref["z_scale"]).max())
    print(f"per-column {precision}: forward {err:.2e}, VJP features {ef:.2e}, z {ez:.2e}")
    assert err < tol
    assert ef < vtol and ez < 10 * vtol
