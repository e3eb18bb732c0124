"""ffno_outer_noalloc, the non-allocating twin of ffno_outer, through the C ABI: two calls in a row (different
shapes, so the shared scratch is reused with other contents in it) against ffno_outer with caller scratch, and the
refusal of a product beyond its fixed capacity. It serves hosts that bind the C ABI but cannot allocate device memory
for the library on each call. Collected last so that a run stopping at the first failure has run every other test."""
import pytest
import torch

pytestmark = pytest.mark.gpu


CAPACITY = 4 << 20      # floats of the library's fixed partial-sum array


def _outer_pair(Ma, Mb, N, seed, accumulate=0):
    from ffnoml_gb300 import _native as nat
    g = torch.Generator().manual_seed(seed)
    A = torch.randn(Ma, N, generator=g).cuda()
    B = torch.randn(Mb, N, generator=g).cuda()
    s = torch.cuda.current_stream().cuda_stream
    nsplit = nat.lib().ffno_outer_parts(Ma, Mb, N)
    part = torch.empty(nsplit * Ma * Mb, device="cuda")
    start = torch.randn(Ma, Mb, generator=g, dtype=torch.float64).cuda() if accumulate else None
    ref = start.clone() if accumulate else torch.empty(Ma, Mb, dtype=torch.float64, device="cuda")
    got = start.clone() if accumulate else torch.full((Ma, Mb), float("nan"), dtype=torch.float64, device="cuda")
    nat.call("ffno_outer", A.data_ptr(), N, Ma, B.data_ptr(), N, Mb, N, part.data_ptr(), nsplit, ref.data_ptr(),
             accumulate, s)
    nat.call("ffno_outer_noalloc", A.data_ptr(), N, Ma, B.data_ptr(), N, Mb, N, got.data_ptr(), accumulate, s)
    torch.cuda.synchronize()
    exact = A.double() @ B.double().t() + (start if accumulate else 0.0)
    return ref, got, exact, nsplit


def test_noalloc_outer_matches_outer_on_two_calls():
    for Ma, Mb, N, seed in ((256, 64, 200_000, 1), (72, 130, 50_000, 2)):
        ref, got, exact, nsplit = _outer_pair(Ma, Mb, N, seed)
        assert Ma * Mb * nsplit <= CAPACITY
        scale = exact.abs().max()
        # the same split count as ffno_outer: the same partial sums in the same order
        assert torch.equal(got, ref)
        assert ((got - exact).abs().max() / scale).item() < 1e-5


def test_noalloc_outer_accumulates_like_outer():
    ref, got, exact, _ = _outer_pair(96, 40, 80_000, 3, accumulate=1)
    assert torch.equal(got, ref)
    assert ((got - exact).abs().max() / exact.abs().max()).item() < 1e-5


@pytest.mark.parametrize("Ma,Mb,N", [(1500, 1500, 50_000), (2048, 2048, 4096)], ids=["clamped", "at_capacity"])
def test_noalloc_outer_with_fewer_splits_than_outer(Ma, Mb, N):
    """Where Ma * Mb * ffno_outer_parts exceeds the array, the entry point runs fewer splits (one split of Ma * Mb =
    4 Mi floats at the capacity itself): the same sums to rounding."""
    ref, got, exact, nsplit = _outer_pair(Ma, Mb, N, 4)
    assert Ma * Mb <= CAPACITY
    scale = exact.abs().max()
    # both are float32 sums over N terms per split (fewer, longer splits here): each within float32 summation error
    # of the float64 product, so within twice that of each other
    e_got = ((got - exact).abs().max() / scale).item()
    e_ref = ((ref - exact).abs().max() / scale).item()
    assert e_got < 5e-5 and e_ref < 5e-5
    assert ((got - ref).abs().max() / scale).item() < 1e-4


def test_noalloc_outer_refuses_oversized_products():
    from ffnoml_gb300 import _native as nat
    A = torch.zeros(16, device="cuda")
    out = torch.zeros(1, dtype=torch.float64, device="cuda")
    status = nat.lib().ffno_outer_noalloc(A.data_ptr(), 1, 4096, A.data_ptr(), 1, 2048, 1, out.data_ptr(), 0,
                                          torch.cuda.current_stream().cuda_stream)
    assert status == 5
