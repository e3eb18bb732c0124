"""Each split-BF16 tensor-core kernel against its FP32 counterpart, through the C ABI, on a ragged voxel count (V not
a multiple of the 128-voxel tile). Split-BF16 products carry ~2^-16 relative error, so the bar is 2e-4 relative."""
import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu

V = 1000
G = 8


def _nat():
    from ffnoml_gb300 import _native as nat
    return nat


def _s():
    return torch.cuda.current_stream().cuda_stream


def _rand(*shape, seed=0, scale=1.0):
    g = torch.Generator().manual_seed(seed)
    return (torch.randn(*shape, generator=g) * scale).cuda().contiguous()


_KEEP = []


def _hold(t):
    """data_ptr of a tensor kept alive until the test ends (kernels run asynchronously after the call returns)."""
    _KEEP.append(t)
    return t.data_ptr()


@pytest.fixture(autouse=True)
def _release():
    yield
    torch.cuda.synchronize()
    _KEEP.clear()


def _close(a, b, tol=2e-4):
    err = ((a - b).abs().max() / b.abs().max().clamp_min(1e-12)).item()
    assert err < tol, err


class _Packed:
    def __init__(self, t):
        self.t = t

    def data_ptr(self):
        return _hold(self.t)


def _pack(*mats):
    from ffnoml_gb300.executor import tc_pack
    return _Packed(tc_pack(torch.device("cuda"), *[m.cpu() for m in mats]))


def _coefs(C, seed):
    g = torch.Generator().manual_seed(seed)
    c = torch.stack([torch.randn(C, generator=g) * 0.1, 1 + 0.2 * torch.randn(C, generator=g),
                     0.1 * torch.randn(C, generator=g)])
    return c.reshape(-1).cuda().contiguous()


@pytest.mark.parametrize("C,V", [(16, V), (32, V), (64, V), (64, 152 * 128 * 5 + 77), (96, V),
                                 (96, 152 * 128 * 3 + 77)])
@pytest.mark.parametrize("mode", [0, 1, 2])
def test_mlp2_fwd_tc(C, V, mode):
    """Also at a voxel count that sends several tiles through every CTA's two-stage ring, with a ragged last tile; and
    at width 96 (one pipeline a CTA, the hidden layer in two K-halves, GroupNorm groups of 12 channels)."""
    nat = _nat()
    x, prev = _rand(V, C, seed=1), _rand(V, C, seed=2)
    pc = _coefs(C, 3)
    w1, w2 = _rand(2 * C, C, seed=4, scale=C ** -0.5), _rand(C, 2 * C, seed=5, scale=(2 * C) ** -0.5)
    dw = (1 + 0.1 * _rand(V, seed=6)).contiguous()
    err = torch.zeros(1, dtype=torch.int32, device="cuda")
    outs = []
    for tc in (False, True):
        pre, xo = torch.empty(V, C, device="cuda"), torch.zeros(V, C, device="cuda")
        P = nat.lib().ffno_tc_parts(V) if tc else nat.lib().ffno_stats_parts(V)
        part = torch.empty(P * G * 3, dtype=torch.float64, device="cuda")
        coefs = torch.empty(3 * C, device="cuda")
        gst = torch.empty(G * 3, dtype=torch.float64, device="cuda")
        args = (mode, x.data_ptr(), prev.data_ptr(), pc.data_ptr(), 0.7, xo.data_ptr(), V, C)
        if tc:
            nat.call("ffno_mlp2_fwd_tc", *args, _pack(w1, w2).data_ptr(), dw.data_ptr(), pre.data_ptr(),
                     part.data_ptr(), P, G, err.data_ptr(), _s())
        else:
            nat.call("ffno_mlp2_fwd", *args, _hold(w1.t().contiguous()), _hold(w2.t().contiguous()),
                     dw.data_ptr(), pre.data_ptr(), part.data_ptr(), P, G, _s())
        ones = torch.ones(C, device="cuda")
        zeros = torch.zeros(C, device="cuda")
        nat.call("ffno_gn_finalize", part.data_ptr(), P, C, G, ones.data_ptr(), zeros.data_ptr(), 1e-5,
                 coefs.data_ptr(), gst.data_ptr(), _s())
        torch.cuda.synchronize()
        outs.append((pre, xo, gst))
    assert int(err.item()) == 0
    _close(outs[1][0], outs[0][0])
    if mode:
        _close(outs[1][1], outs[0][1], 1e-6)
    assert torch.allclose(outs[1][2], outs[0][2], rtol=1e-4, atol=1e-6)


@pytest.mark.parametrize("C,V", [(16, V), (32, V), (64, V), (64, 152 * 128 * 5 + 77), (96, V),
                                 (96, 152 * 128 * 3 + 77)])
@pytest.mark.parametrize("with_z", [False, True])
def test_gate_fwd_tc(C, V, with_z):
    """Widths 32 and 64 run the warp-specialised kernel; also at a voxel count that cycles every CTA's ring; width 96
    the two-pipeline kernel with rows of 12 octets."""
    nat = _nat()
    x = _rand(V, C, seed=1)
    g1, g2 = _rand(C, C, seed=2, scale=C ** -0.5), _rand(C, C, seed=3, scale=C ** -0.5)
    zp, z = (_rand(C, seed=4), _rand(V, seed=5)) if with_z else (None, None)
    ptr = lambda t: None if t is None else t.data_ptr()
    err = torch.zeros(1, dtype=torch.int32, device="cuda")
    a, b = torch.empty(V, C, device="cuda"), torch.empty(V, C, device="cuda")
    nat.call("ffno_gate_fwd", x.data_ptr(), V, C, _hold(g1.t().contiguous()), _hold(g2.t().contiguous()),
             ptr(zp), ptr(z), a.data_ptr(), _s())
    nat.call("ffno_gate_fwd_tc", x.data_ptr(), V, C, _pack(g1, g2).data_ptr(), ptr(zp), ptr(z), b.data_ptr(),
             err.data_ptr(), _s())
    torch.cuda.synchronize()
    assert int(err.item()) == 0
    _close(b, a)


def _fuse_weights(C):
    return (_rand(C, 3 * C, seed=11, scale=(3 * C) ** -0.5), _rand(2 * C, C, seed=12, scale=C ** -0.5),
            _rand(2 * C, seed=13), _rand(2 * C, 2 * C, seed=14, scale=(2 * C) ** -0.5),
            _rand(C, 2 * C, seed=15, scale=(2 * C) ** -0.5))


@pytest.mark.parametrize("C,V", [(16, V), (32, V), (64, V), (32, 152 * 128 * 3 + 77), (64, 152 * 128 * 5 + 77)])
def test_fuse_fwd_tc(C, V):
    """fuse2 at widths 32 and 64 is the warp-specialised kernel (three-stage ring of 32-channel phases)."""
    nat = _nat()
    x, sp, vp = _rand(V, C, seed=1), _rand(V, C, seed=2), _rand(V, C, seed=3)
    sc, vc = _coefs(C, 4), _coefs(C, 5)
    bg0, bg2, bb, f0, f2 = _fuse_weights(C)
    dw = (1 + 0.1 * _rand(V, seed=6)).contiguous()
    err = torch.zeros(1, dtype=torch.int32, device="cuda")
    P0, P1 = nat.lib().ffno_stats_parts(V), nat.lib().ffno_tc_parts(V)
    part0 = torch.empty(P0 * G * 3, dtype=torch.float64, device="cuda")
    part1 = torch.empty(P1 * G * 3, dtype=torch.float64, device="cuda")
    a, b = torch.empty(V, C, device="cuda"), torch.empty(V, C, device="cuda")
    T = lambda m: _hold(m.t().contiguous())
    nat.call("ffno_fuse_fwd", x.data_ptr(), sp.data_ptr(), sc.data_ptr(), vp.data_ptr(), vc.data_ptr(), V, C, T(bg0),
             T(bg2), bb.data_ptr(), T(f0), T(f2), dw.data_ptr(), a.data_ptr(), part0.data_ptr(), P0, G, _s())
    gates = torch.empty(V, 2 * C, device="cuda")
    nat.call("ffno_fuse1_tc", x.data_ptr(), sp.data_ptr(), sc.data_ptr(), vp.data_ptr(), vc.data_ptr(), V, C,
             _pack(bg0, bg2).data_ptr(), bb.data_ptr(), gates.data_ptr(), None, err.data_ptr(), _s())
    nat.call("ffno_fuse2_tc", sp.data_ptr(), sc.data_ptr(), vp.data_ptr(), vc.data_ptr(), gates.data_ptr(), V, C,
             _pack(f0, f2).data_ptr(), dw.data_ptr(), b.data_ptr(), part1.data_ptr(), P1, G, err.data_ptr(), _s())
    torch.cuda.synchronize()
    assert int(err.item()) == 0
    _close(b, a)


@pytest.mark.parametrize("C,V", [(16, V), (32, V), (64, V), (32, 152 * 128 * 5 + 77), (64, 152 * 128 * 5 + 77),
                                 (96, V), (96, 152 * 128 * 3 + 77)])
def test_mlp2_bwd_tc(C, V):
    """Also at a voxel count that sends several tiles through every CTA's two-stage ring, with a ragged last tile. At
    width 96 the pack is the forward's [w1, w2]: the kernel reads W2 and W1 as MN-major operands (their transposes)."""
    nat = _nat()
    a, pb, base = _rand(V, C, seed=1), _rand(V, C, seed=2), _rand(V, C, seed=3)
    w1, w2 = _rand(2 * C, C, seed=4, scale=C ** -0.5), _rand(C, 2 * C, seed=5, scale=(2 * C) ** -0.5)
    err = torch.zeros(1, dtype=torch.int32, device="cuda")
    r0, r1 = torch.empty(V, C, device="cuda"), torch.empty(V, C, device="cuda")
    # FP32 kernel wants w1 [C][2C] (in x out), w2t = W2^T laid [C][2C], w1t [2C][C]
    nat.call("ffno_mlp2_bwd", a.data_ptr(), pb.data_ptr(), base.data_ptr(), V, C, _hold(w1.t().contiguous()),
             _hold(w2.contiguous()), _hold(w1.contiguous()), r0.data_ptr(), _s())
    pack = _pack(w1, w2) if C == 96 else _pack(w1, w2.t(), w1.t())
    nat.call("ffno_mlp2_bwd_tc", a.data_ptr(), pb.data_ptr(), base.data_ptr(), V, C, pack.data_ptr(), r1.data_ptr(),
             err.data_ptr(), _s())
    torch.cuda.synchronize()
    assert int(err.item()) == 0
    _close(r1, r0)


@pytest.mark.parametrize("C,V", [(16, V), (32, V), (64, V), (32, 2 * 128 + 5), (64, 152 * 128 * 5 + 77), (96, V),
                                 (96, 152 * 128 * 3 + 77)])
def test_gate_bwd_tc(C, V):
    """Widths 32 and 64 run the warp-specialised kernel (tiles in pairs): also one CTA with an odd tile count and
    every CTA with a ragged last pair; the second call writes x_bar over its own base. Width 96: one pipeline a CTA,
    the pack [g1, g2] (the transposes read out of it)."""
    nat = _nat()
    x, xsb, xvb, base = _rand(V, C, seed=1), _rand(V, C, seed=2), _rand(V, C, seed=3), _rand(V, C, seed=4)
    s1, s2 = _rand(C, C, seed=5, scale=C ** -0.5), _rand(C, C, seed=6, scale=C ** -0.5)
    v1, v2 = _rand(C, C, seed=7, scale=C ** -0.5), _rand(C, C, seed=8, scale=C ** -0.5)
    zp = _rand(C, seed=9)
    err = torch.zeros(1, dtype=torch.int32, device="cuda")
    r0, r1 = torch.empty(V, C, device="cuda"), torch.empty(V, C, device="cuda")
    z0, z1 = torch.zeros(V, device="cuda"), torch.zeros(V, device="cuda")
    T = lambda m: _hold(m.t().contiguous())
    Nn = lambda m: _hold(m.contiguous())
    nat.call("ffno_gate_bwd", x.data_ptr(), xsb.data_ptr(), xvb.data_ptr(), base.data_ptr(), V, C, T(s1), T(s2),
             Nn(s2), Nn(s1), T(v1), T(v2), Nn(v2), Nn(v1), zp.data_ptr(), r0.data_ptr(), z0.data_ptr(), _s())
    pk = (lambda g1, g2: _pack(g1, g2)) if C == 96 else (lambda g1, g2: _pack(g1, g2, g2.t(), g1.t()))
    nat.call("ffno_gate_bwd_tc", x.data_ptr(), xsb.data_ptr(), base.data_ptr(), V, C, pk(s1, s2).data_ptr(), None,
             r1.data_ptr(), None, err.data_ptr(), _s())
    nat.call("ffno_gate_bwd_tc", x.data_ptr(), xvb.data_ptr(), r1.data_ptr(), V, C, pk(v1, v2).data_ptr(),
             zp.data_ptr(), r1.data_ptr(), z1.data_ptr(), err.data_ptr(), _s())
    torch.cuda.synchronize()
    assert int(err.item()) == 0
    _close(r1, r0)
    _close(z1, z0, 1e-5)


@pytest.mark.parametrize("C,V", [(16, V), (32, V), (64, V), (64, 152 * 128 * 5 + 77)])
def test_fuse_bwd_tc(C, V):
    """Also at a voxel count that sends several tiles through every CTA of the warp-specialised stage b."""
    nat = _nat()
    x, sp, vp = _rand(V, C, seed=1), _rand(V, C, seed=2), _rand(V, C, seed=3)
    sc, vc = _coefs(C, 4), _coefs(C, 5)
    fb, base = _rand(V, C, seed=6), _rand(V, C, seed=7)
    bg0, bg2, bb, f0, f2 = _fuse_weights(C)
    err = torch.zeros(1, dtype=torch.int32, device="cuda")
    o = [torch.empty(V, C, device="cuda") for _ in range(6)]
    T = lambda m: _hold(m.t().contiguous())
    Nn = lambda m: _hold(m.contiguous())
    nat.call("ffno_fuse_bwd", x.data_ptr(), sp.data_ptr(), sc.data_ptr(), vp.data_ptr(), vc.data_ptr(), fb.data_ptr(),
             base.data_ptr(), V, C, T(bg0), T(bg2), bb.data_ptr(), T(f0), Nn(f2), Nn(f0), Nn(bg2), Nn(bg0),
             o[0].data_ptr(), o[1].data_ptr(), o[2].data_ptr(), _s())
    gates, hg, hfb = (torch.empty(V, 2 * C, device="cuda"), torch.empty(V, C, device="cuda"),
                      torch.empty(V, 2 * C, device="cuda"))
    nat.call("ffno_fuse1_tc", x.data_ptr(), sp.data_ptr(), sc.data_ptr(), vp.data_ptr(), vc.data_ptr(), V, C,
             _pack(bg0, bg2).data_ptr(), bb.data_ptr(), gates.data_ptr(), hg.data_ptr(), err.data_ptr(), _s())
    nat.call("ffno_fuse_bwd_a_tc", sp.data_ptr(), sc.data_ptr(), vp.data_ptr(), vc.data_ptr(), gates.data_ptr(),
             fb.data_ptr(), V, C, _pack(f0, f2.t()).data_ptr(), hfb.data_ptr(), err.data_ptr(), _s())
    nat.call("ffno_fuse_bwd_b_tc", sp.data_ptr(), sc.data_ptr(), vp.data_ptr(), vc.data_ptr(), gates.data_ptr(),
             hg.data_ptr(), fb.data_ptr(), hfb.data_ptr(), base.data_ptr(), V, C,
             _pack(f0.t(), bg2.t(), bg0.t()).data_ptr(), o[3].data_ptr(), o[4].data_ptr(), o[5].data_ptr(),
             err.data_ptr(), _s())
    torch.cuda.synchronize()
    assert int(err.item()) == 0
    for i in range(3):
        _close(o[3 + i], o[i])


@pytest.mark.parametrize("which", ["wf", "hf", "wi", "zf", "zi"])
@pytest.mark.parametrize("C", [16, 64])
@pytest.mark.parametrize("kind", ["streamed", "resident"])
def test_xform_tc_matches_fp32(which, C, kind):
    from ffnoml_gb300 import tables as tb
    from ffnoml_gb300.executor import TcXform, _descs
    nat = _nat()
    D, H, W, live = 12, 24, 20, 13
    Wf = W // 2 + 1
    twf, thf, thi, twi = tb.plane_dft(H, W)
    g = np.random.default_rng(3)
    tzf, tzi = g.normal(size=(2 * live, D)), g.normal(size=(D, 2 * live))
    T = dict(wf=twf, hf=thf, wi=twi, zf=tzf, zi=tzi)[which]
    d = _descs(D, H, W, C, live)[which]
    n_in = {"wf": D * H * W * C, "hf": D * 2 * H * Wf * C, "wi": D * 2 * H * Wf * C, "zf": D * H * W * C,
            "zi": 2 * live * H * W * C}[which]
    n_out = {"wf": D * 2 * H * Wf * C, "hf": D * 2 * H * Wf * C, "wi": D * H * W * C, "zf": 2 * live * H * W * C,
             "zi": D * H * W * C}[which]
    x = _rand(n_in, seed=7)
    a, b = torch.zeros(n_out, device="cuda"), torch.zeros(n_out, device="cuda")
    Tf = torch.as_tensor(T, dtype=torch.float32).cuda().contiguous()
    err = torch.zeros(1, dtype=torch.int32, device="cuda")
    nat.call("ffno_xform", Tf.data_ptr(), x.data_ptr(), a.data_ptr(), d, 0, _s())
    tx = TcXform(T, torch.device("cuda"))
    for r0, rows, c0, cols, packed, res in tx.slices:
        dd = nat.XformDesc.from_buffer_copy(d)
        dd.M, dd.K = rows, cols
        src, dst, acc = x.data_ptr() + 4 * c0 * d.in_lo, b.data_ptr() + 4 * r0 * d.out_lo, 1 if c0 else 0
        if kind == "resident":
            assert res is not None
            nat.call("ffno_xform_tcr", _hold(res[0]), res[1], res[2], src, dst, dd, acc, err.data_ptr(), _s())
        else:
            nat.call("ffno_xform_tc", _hold(packed), src, dst, dd, acc, err.data_ptr(), _s())
    torch.cuda.synchronize()
    assert int(err.item()) == 0
    _close(b, a)


@pytest.mark.parametrize("C", [16, 32, 64, 96])
@pytest.mark.parametrize("rank", [0, 3, 8])
@pytest.mark.parametrize("layout", ["horizontal", "height"])
@pytest.mark.parametrize("nb", [150, 100])
def test_spectral_mix_tc(C, rank, layout, nb):
    """Width 96 runs its own row-oriented kernel: the pack is wbig itself (out = g (x wbig) + the low-rank term). With
    nb = 100 the 37 items (frequency, 128-row block) are odd in number, so one CTA's second pipeline has no item."""
    from ffnoml_gb300.executor import mix_pack
    nat = _nat()
    F = 37
    if layout == "horizontal":
        sf, sb, s_im = C, 2 * F * C, F * C        # [b][2][F][C]
    else:
        sf, sb, s_im = nb * C, C, F * nb * C      # [2][F][b][C]
    x = _rand(nb * 2 * F * C, seed=1)
    wr, wi = _rand(C, C, seed=2, scale=C ** -0.5), _rand(C, C, seed=3, scale=C ** -0.5)
    wbig = torch.cat([torch.cat([wr, wi], 1), torch.cat([-wi, wr], 1)], 0).contiguous()
    gg = _rand(F, 2, seed=4)
    U = _rand(F, C, max(rank, 1), seed=5) if rank else None
    Vm = _rand(F, max(rank, 1), C, seed=6) if rank else None
    ptr = lambda t: None if t is None else t.data_ptr()
    a, b = torch.zeros_like(x), torch.zeros_like(x)
    err = torch.zeros(1, dtype=torch.int32, device="cuda")
    nat.call("ffno_spectral_mix", x.data_ptr(), a.data_ptr(), F, nb, sf, sb, s_im, C, wbig.data_ptr(), gg.data_ptr(),
             ptr(U), ptr(Vm), rank, _s())
    pack = _pack(wbig).data_ptr() if C == 96 else _hold(mix_pack(torch.device("cuda"), wbig.t().cpu()))
    nat.call("ffno_spectral_mix_tc", x.data_ptr(), b.data_ptr(), F, nb, sf, sb, s_im, C, pack, gg.data_ptr(), ptr(U),
             ptr(Vm), rank, err.data_ptr(), _s())
    torch.cuda.synchronize()
    assert int(err.item()) == 0
    _close(b, a)


def test_spectral_mix_tc96_large():
    """The width-96 mixing on a height-layout spectrum larger than L2 ([2][64][16384][96] FP32, 0.8 GB each way),
    rank 8: every CTA runs many items on both pipelines; against the FP32 kernel."""
    nat = _nat()
    C, F, nb, rank = 96, 64, 16384, 8
    sf, sb, s_im = nb * C, C, F * nb * C
    x = torch.randn(nb * 2 * F * C, generator=torch.Generator("cuda").manual_seed(1), device="cuda")
    wr, wi = _rand(C, C, seed=2, scale=C ** -0.5), _rand(C, C, seed=3, scale=C ** -0.5)
    wbig = torch.cat([torch.cat([wr, wi], 1), torch.cat([-wi, wr], 1)], 0).contiguous()
    gg, U, Vm = _rand(F, 2, seed=4), _rand(F, C, rank, seed=5), _rand(F, rank, C, seed=6)
    a, b = torch.empty_like(x), torch.empty_like(x)
    err = torch.zeros(1, dtype=torch.int32, device="cuda")
    nat.call("ffno_spectral_mix", x.data_ptr(), a.data_ptr(), F, nb, sf, sb, s_im, C, wbig.data_ptr(), gg.data_ptr(),
             U.data_ptr(), Vm.data_ptr(), rank, _s())
    pack = _pack(wbig)
    nat.call("ffno_spectral_mix_tc", x.data_ptr(), b.data_ptr(), F, nb, sf, sb, s_im, C, pack.data_ptr(),
             gg.data_ptr(), U.data_ptr(), Vm.data_ptr(), rank, err.data_ptr(), _s())
    torch.cuda.synchronize()
    assert int(err.item()) == 0
    _close(b, a)


@pytest.mark.parametrize("name", ["hca_stretched", "w32_m16", "w64_m32"])
@pytest.mark.parametrize("math32", [0, 1])
def test_head_tc(name, math32):
    """ffno_head_fwd_tc / ffno_head_bwd_tc against the FP32 head kernels (LTE math in FP64) on a golden model's head
    and normalised inputs, tiled to a ragged voxel count; output compared in log10 n."""
    from golden_io import load, model_config
    from ffnoml_gb300 import FFNO3D
    from ffnoml_gb300.executor import Packed
    nat = _nat()
    meta, state, a = load(name)
    model = FFNO3D(**model_config(meta))
    model.load_state_dict({k: v.float() for k, v in state.items()}, strict=True)
    C, L = model.width, model.out_channels
    pk = Packed(model, torch.device("cuda"))
    hp = nat.HeadParams.from_buffer_copy(pk.head)
    hp.math32 = math32
    xin0 = a["x"][0].reshape(6, -1).float()
    Vn = 5 * 128 + 77
    xin = xin0.repeat(1, (Vn + xin0.shape[1] - 1) // xin0.shape[1])[:, :Vn].cuda().contiguous()
    x, ybar = _rand(Vn, C, seed=11), _rand(L, Vn, seed=12)
    err = torch.zeros(1, dtype=torch.int32, device="cuda")
    s = _s()
    ref, out = torch.empty(L, Vn, device="cuda"), torch.empty(L, Vn, device="cuda")
    nat.call("ffno_head_fwd", x.data_ptr(), xin.data_ptr(), Vn, C, pk.p1.data_ptr(), pk.p2.data_ptr(),
             pk.b2.data_ptr(), pk.nh, pk.nhp, pk.head, ref.data_ptr(), None, s)
    nat.call("ffno_head_fwd_tc", x.data_ptr(), xin.data_ptr(), Vn, C, pk.tc_head.data_ptr(), pk.b2.data_ptr(),
             pk.nh, pk.nhp, hp, out.data_ptr(), None, err.data_ptr(), s)
    std_y = model.std_Y.detach().float().cuda()[:, None]
    dlog = ((out - ref) * std_y).abs().max().item()
    assert dlog < 1e-4, dlog
    xb_ref, xib_ref = torch.empty(Vn, C, device="cuda"), torch.empty(6, Vn, device="cuda")
    xb, xib = torch.empty(Vn, C, device="cuda"), torch.empty(6, Vn, device="cuda")
    nat.call("ffno_head_bwd", x.data_ptr(), xin.data_ptr(), ybar.data_ptr(), Vn, C, pk.p1.data_ptr(),
             pk.p2.data_ptr(), pk.b2.data_ptr(), pk.p2t.data_ptr(), pk.p1t.data_ptr(), pk.nhp, pk.head,
             xb_ref.data_ptr(), xib_ref.data_ptr(), s)
    nat.call("ffno_head_bwd_tc", x.data_ptr(), xin.data_ptr(), ybar.data_ptr(), Vn, C, pk.tcb_head.data_ptr(),
             pk.b2.data_ptr(), pk.nhp, hp, xb.data_ptr(), xib.data_ptr(), err.data_ptr(), s)
    torch.cuda.synchronize()
    assert err.item() == 0
    _close(xb, xb_ref, 2e-4)
    _close(xib, xib_ref, 1e-3 if math32 else 2e-4)


@pytest.mark.parametrize("Ma,Mb,N,nsplit", [(12, 8, 1000, 3), (256, 64, 65536 + 196, 152), (64, 256, 65536 + 196, 152),
                                           (300, 40, 8192, 7), (496, 64, 4096, 5), (16, 16, 256, 9)])
def test_outer_tc(Ma, Mb, N, nsplit):
    """ffno_outer_tc against a float64 product and against ffno_outer: tile counts 1-4 (one stage at 4), the longer
    operand on either side, ragged rows and chunks, and more splits than chunks (splits with no work)."""
    nat = _nat()
    A, B = _rand(Ma, N, seed=21), _rand(Mb, N, seed=22)
    ref = A.double() @ B.double().t()
    part = torch.empty(nsplit * Ma * Mb, device="cuda")
    err = torch.zeros(1, dtype=torch.int32, device="cuda")
    out = torch.full((Ma, Mb), 0.5, dtype=torch.float64, device="cuda")
    nat.call("ffno_outer_tc", A.data_ptr(), N, Ma, B.data_ptr(), N, Mb, N, part.data_ptr(), nsplit, out.data_ptr(),
             1, err.data_ptr(), _s())
    out32 = torch.empty(Ma, Mb, dtype=torch.float64, device="cuda")
    part32 = torch.empty(nat.lib().ffno_outer_parts(Ma, Mb, N) * Ma * Mb, device="cuda")
    nat.call("ffno_outer", A.data_ptr(), N, Ma, B.data_ptr(), N, Mb, N, part32.data_ptr(),
             nat.lib().ffno_outer_parts(Ma, Mb, N), out32.data_ptr(), 0, _s())
    torch.cuda.synchronize()
    assert err.item() == 0
    _close(out - 0.5, ref, 2e-5)
    _close(out32, ref, 2e-5)


@pytest.mark.parametrize("ma,mb,calls", [(256, 680, 3), (680, 256, 3), (64, 1300, 2), (200, 200, 1)])
def test_outer_tc_in_slices(ma, mb, calls):
    """The executor's height-table gradient product at production sizes (2 M' = 680 rows at D = 256): sliced calls of
    ffno_outer_tc_ld along the longer side, into rows of out (ma longer) or into columns at row stride mb (mb longer),
    accumulated onto what out holds, against a float64 product; and the unsliced single call at (200, 200)."""
    from ffnoml_gb300.executor import Executor, _outer_tc_slices

    class _WS:
        err = torch.zeros(1, dtype=torch.int32, device="cuda")

    class _Model:
        precision = "bf16"

    ex = Executor.__new__(Executor)
    ex.model = _Model()
    import threading
    ex._tls = threading.local()
    N = 16384 * 4 + 96
    a, b = _rand(ma, N, seed=31), _rand(mb, N, seed=32)
    ref = a.double() @ b.double().t()
    plan = _outer_tc_slices(ma, mb)
    assert plan is not None and len(plan) == calls
    part = torch.empty(152 * max(r for _, r in plan) * min(ma, mb), device="cuda")
    out = torch.full((ma, mb), 0.25, dtype=torch.float64, device="cuda")
    ex._outer(_WS, a, ma, b, mb, N, part, 64, out)      # 64 splits for the single call (the sliced ones pick theirs)
    torch.cuda.synchronize()
    assert _WS.err.item() == 0
    _close(out - 0.25, ref, 2e-5)


@pytest.mark.parametrize("V", [V, 152 * 128 * 3 + 77, 600_000])
def test_fuse_tc96(V):
    """The branch fusion at width 96 on tensor cores (gates, hidden pre-activation, output; backward in three
    kernels that read their transposed weights out of the forward's packs) against the FP32 fusion kernels."""
    nat = _nat()
    C = 96
    x, sp, vp = _rand(V, C, seed=1), _rand(V, C, seed=2), _rand(V, C, seed=3)
    sc, vc = _coefs(C, 4), _coefs(C, 5)
    fb, base = _rand(V, C, seed=6), _rand(V, C, seed=7)
    bg0, bg2, bb, f0, f2 = _fuse_weights(C)
    dw = (1 + 0.1 * _rand(V, seed=8)).contiguous()
    err = torch.zeros(1, dtype=torch.int32, device="cuda")
    T = lambda m: _hold(m.t().contiguous())
    Nn = lambda m: _hold(m.contiguous())
    # forward
    P0, P1 = nat.lib().ffno_stats_parts(V), nat.lib().ffno_tc_parts(V)
    part0 = torch.empty(P0 * G * 3, dtype=torch.float64, device="cuda")
    part1 = torch.empty(P1 * G * 3, dtype=torch.float64, device="cuda")
    a, b = torch.empty(V, C, device="cuda"), torch.empty(V, C, device="cuda")
    nat.call("ffno_fuse_fwd", x.data_ptr(), sp.data_ptr(), sc.data_ptr(), vp.data_ptr(), vc.data_ptr(), V, C, T(bg0),
             T(bg2), bb.data_ptr(), T(f0), T(f2), dw.data_ptr(), a.data_ptr(), part0.data_ptr(), P0, G, _s())
    gates, hg, hf = (torch.empty(V, 2 * C, device="cuda"), torch.empty(V, C, device="cuda"),
                     torch.empty(V, 2 * C, device="cuda"))
    g_pack, f1_pack, f2_pack = _pack(bg0, bg2), _pack(f0), _pack(f2)
    nat.call("ffno_fuse1_tc", x.data_ptr(), sp.data_ptr(), sc.data_ptr(), vp.data_ptr(), vc.data_ptr(), V, C,
             g_pack.data_ptr(), bb.data_ptr(), gates.data_ptr(), hg.data_ptr(), err.data_ptr(), _s())
    nat.call("ffno_fuse_hidden_tc", sp.data_ptr(), sc.data_ptr(), vp.data_ptr(), vc.data_ptr(), gates.data_ptr(), V,
             C, f1_pack.data_ptr(), hf.data_ptr(), err.data_ptr(), _s())
    nat.call("ffno_fuse_out_tc", sp.data_ptr(), sc.data_ptr(), vp.data_ptr(), vc.data_ptr(), gates.data_ptr(),
             hf.data_ptr(), V, C, f2_pack.data_ptr(), dw.data_ptr(), b.data_ptr(), part1.data_ptr(), P1, G,
             err.data_ptr(), _s())
    ones, zeros = torch.ones(C, device="cuda"), torch.zeros(C, device="cuda")
    st = []
    for part, P in ((part0, P0), (part1, P1)):
        coefs, gst = torch.empty(3 * C, device="cuda"), torch.empty(G * 3, dtype=torch.float64, device="cuda")
        nat.call("ffno_gn_finalize", part.data_ptr(), P, C, G, ones.data_ptr(), zeros.data_ptr(), 1e-5,
                 coefs.data_ptr(), gst.data_ptr(), _s())
        st.append(gst)
    # backward
    o = [torch.empty(V, C, device="cuda") for _ in range(6)]
    nat.call("ffno_fuse_bwd", x.data_ptr(), sp.data_ptr(), sc.data_ptr(), vp.data_ptr(), vc.data_ptr(), fb.data_ptr(),
             base.data_ptr(), V, C, T(bg0), T(bg2), bb.data_ptr(), T(f0), Nn(f2), Nn(f0), Nn(bg2), Nn(bg0),
             o[0].data_ptr(), o[1].data_ptr(), o[2].data_ptr(), _s())
    hfb = torch.empty(V, 2 * C, device="cuda")
    nat.call("ffno_fuse_bwd_h_tc", fb.data_ptr(), hf.data_ptr(), V, C, f2_pack.data_ptr(), hfb.data_ptr(),
             err.data_ptr(), _s())
    nat.call("ffno_fuse_bwd_q_tc", sp.data_ptr(), sc.data_ptr(), vp.data_ptr(), vc.data_ptr(), gates.data_ptr(),
             fb.data_ptr(), hfb.data_ptr(), V, C, f1_pack.data_ptr(), o[4].data_ptr(), o[5].data_ptr(),
             hfb.data_ptr(), err.data_ptr(), _s())
    nat.call("ffno_fuse_bwd_x_tc", hfb.data_ptr(), hg.data_ptr(), base.data_ptr(), V, C, g_pack.data_ptr(),
             o[3].data_ptr(), o[4].data_ptr(), o[5].data_ptr(), err.data_ptr(), _s())
    torch.cuda.synchronize()
    assert int(err.item()) == 0
    _close(b, a)
    assert torch.allclose(st[1], st[0], rtol=1e-4, atol=1e-6)
    for i in range(3):
        _close(o[3 + i], o[i])


@pytest.mark.parametrize("math32", [0, 1])
@pytest.mark.parametrize("atoms", [["H"], ["H", "CA"]])
def test_head_tc96(math32, atoms):
    """The head at width 96 (one pipeline, the hidden layer in K-slices, the backward reading the transposes out of
    the forward's pack) against the FP32 head kernels, for the one- and two-species heads (7 and 14 head channels,
    padded to 16), at a ragged voxel count."""
    import bench
    from ffnoml_gb300 import create_ffno3d
    from ffnoml_gb300.executor import Packed
    nat = _nat()
    torch.manual_seed(4)
    L = 6 * len(atoms)
    model = create_ffno3d(6, L, atoms=atoms, n_layers=1)
    with torch.no_grad():
        model.proj2.weight.normal_(0.0, 0.3)
        model.proj2.bias.normal_(0.0, 0.3)
    model.set_normalization(bench.MEAN_X, bench.STD_X, np.zeros(L), np.ones(L))
    C = model.width
    assert C == 96
    pk = Packed(model.eval(), torch.device("cuda"))
    hp = nat.HeadParams.from_buffer_copy(pk.head)
    hp.math32 = math32
    Vn = 5 * 128 + 77
    f, z = bench.synthetic_si((Vn, 1, 1), seed=13)
    xn, _ = bench.normalised(f, z)
    xin = torch.from_numpy(xn.reshape(6, Vn)).cuda().contiguous()
    x, ybar = _rand(Vn, C, seed=11), _rand(L, Vn, seed=12)
    err = torch.zeros(1, dtype=torch.int32, device="cuda")
    s = _s()
    ref, out = torch.empty(L, Vn, device="cuda"), torch.empty(L, Vn, device="cuda")
    nat.call("ffno_head_fwd", x.data_ptr(), xin.data_ptr(), Vn, C, pk.p1.data_ptr(), pk.p2.data_ptr(),
             pk.b2.data_ptr(), pk.nh, pk.nhp, pk.head, ref.data_ptr(), None, s)
    nat.call("ffno_head_fwd_tc", x.data_ptr(), xin.data_ptr(), Vn, C, pk.tc_head.data_ptr(), pk.b2.data_ptr(),
             pk.nh, pk.nhp, hp, out.data_ptr(), None, err.data_ptr(), s)
    assert (out - ref).abs().max().item() < 1e-4
    xb_ref, xib_ref = torch.empty(Vn, C, device="cuda"), torch.empty(6, Vn, device="cuda")
    xb, xib = torch.empty(Vn, C, device="cuda"), torch.empty(6, Vn, device="cuda")
    nat.call("ffno_head_bwd", x.data_ptr(), xin.data_ptr(), ybar.data_ptr(), Vn, C, pk.p1.data_ptr(),
             pk.p2.data_ptr(), pk.b2.data_ptr(), pk.p2t.data_ptr(), pk.p1t.data_ptr(), pk.nhp, pk.head,
             xb_ref.data_ptr(), xib_ref.data_ptr(), s)
    nat.call("ffno_head_bwd_tc", x.data_ptr(), xin.data_ptr(), ybar.data_ptr(), Vn, C, pk.tcb_head.data_ptr(),
             pk.b2.data_ptr(), pk.nhp, hp, xb.data_ptr(), xib.data_ptr(), err.data_ptr(), s)
    torch.cuda.synchronize()
    assert err.item() == 0
    _close(xb, xb_ref, 2e-4)
    _close(xib, xib_ref, 1e-3 if math32 else 2e-4)
