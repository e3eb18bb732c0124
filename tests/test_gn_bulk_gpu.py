"""The bulk-copy GroupNorm-backward kernels (ffno_gn_bwd_stats_bulk / ffno_gn_bwd_apply_bulk) against the register
versions (ffno_gn_bwd_stats / ffno_gn_bwd_apply), through the C ABI, at every width, both modes and ragged voxel
counts (a last tile shorter than the others, fewer tiles than CTAs)."""
import pytest
import torch

pytestmark = pytest.mark.gpu


def _rand(*shape, seed=0, scale=1.0):
    g = torch.Generator().manual_seed(seed)
    return (torch.randn(*shape, generator=g) * scale).cuda().contiguous()


@pytest.mark.parametrize("C", [16, 32, 64, 96])
@pytest.mark.parametrize("mode", [0, 1])
@pytest.mark.parametrize("V", [1000, 152 * 64 * 7 + 33, 40])
def test_gn_bwd_bulk_matches(C, mode, V):
    from ffnoml_gb300 import _native as nat
    G, eps = 8, 1e-5
    s = torch.cuda.current_stream().cuda_stream
    u, pre = _rand(V, C, seed=1), _rand(V, C, seed=2, scale=2.0)
    gamma, beta = 1 + 0.1 * _rand(C, seed=3), 0.1 * _rand(C, seed=4)
    dw = (1 + 0.2 * _rand(V, seed=5)).abs().contiguous()
    gst = torch.stack([0.1 * torch.randn(G, dtype=torch.float64), 0.5 + torch.rand(G, dtype=torch.float64),
                       torch.full((G,), float(V), dtype=torch.float64)], 1).reshape(-1).cuda().contiguous()
    nparts = nat.lib().ffno_stats_parts(V)
    err = torch.zeros(1, dtype=torch.int32, device="cuda")
    res = []
    for bulk in (False, True):
        part = torch.empty(nparts * G * 2, dtype=torch.float64, device="cuda")
        sums = torch.empty(G * 2, dtype=torch.float64, device="cuda")
        pbar = torch.empty(V, C, device="cuda")
        wbar = torch.full((V,), 0.25, device="cuda")
        if bulk:
            nat.call("ffno_gn_bwd_stats_bulk", mode, u.data_ptr(), 0.7, pre.data_ptr(), gamma.data_ptr(),
                     beta.data_ptr(), gst.data_ptr(), V, C, G, part.data_ptr(), nparts, err.data_ptr(), s)
        else:
            nat.call("ffno_gn_bwd_stats", mode, u.data_ptr(), 0.7, pre.data_ptr(), gamma.data_ptr(),
                     beta.data_ptr(), gst.data_ptr(), V, C, G, part.data_ptr(), nparts, s)
        nat.call("ffno_gn_bwd_final", part.data_ptr(), nparts, G, sums.data_ptr(), s)
        if bulk:
            nat.call("ffno_gn_bwd_apply_bulk", mode, u.data_ptr(), 0.7, pre.data_ptr(), gamma.data_ptr(),
                     beta.data_ptr(), gst.data_ptr(), sums.data_ptr(), dw.data_ptr(), V, C, G, eps, pbar.data_ptr(),
                     wbar.data_ptr(), err.data_ptr(), s)
        else:
            nat.call("ffno_gn_bwd_apply", mode, u.data_ptr(), 0.7, pre.data_ptr(), gamma.data_ptr(),
                     beta.data_ptr(), gst.data_ptr(), sums.data_ptr(), dw.data_ptr(), V, C, G, eps, pbar.data_ptr(),
                     wbar.data_ptr(), s)
        torch.cuda.synchronize()
        res.append((sums.clone(), pbar, wbar))
    assert err.item() == 0
    (s0, p0, w0), (s1, p1, w1) = res
    assert ((s1 - s0).abs().max() / s0.abs().max()).item() < 1e-6   # float partials summed in another order
    assert ((p1 - p0).abs().max() / p0.abs().max()).item() < 1e-5
    assert ((w1 - w0).abs().max() / (w0 - 0.25).abs().max()).item() < 1e-5
