"""The tcgen05 primitives (canonical K-major BF16 operands, FP32 accumulation in tensor memory) against torch."""
import pytest
import torch

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("b_mn", [0, 1])
@pytest.mark.parametrize("K,N", [(16, 16), (64, 128), (128, 64), (192, 64), (64, 192), (256, 256)])
def test_tc_gemm_matches_torch(K, N, b_mn):
    from ffnoml_gb300 import _native as nat
    g = torch.Generator().manual_seed(K * 1000 + N)
    A = torch.randn(128, K, generator=g).cuda()
    B = torch.randn(N, K, generator=g).cuda()
    D = torch.full((128, N), float("nan"), device="cuda")
    st = torch.zeros(1, dtype=torch.int32, device="cuda")
    nat.call("ffno_tc_selftest", A.data_ptr(), B.data_ptr(), K, N, b_mn, D.data_ptr(), st.data_ptr(),
             torch.cuda.current_stream().cuda_stream)
    torch.cuda.synchronize()
    assert int(st.item()) == 0
    ref = A.bfloat16().float() @ B.bfloat16().float().t()
    assert torch.allclose(D, ref, rtol=1e-4, atol=1e-3), (D - ref).abs().max().item()
