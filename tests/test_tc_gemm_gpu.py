"""The tcgen05 BF16 GEMM building block against torch (FP32 math on the same BF16 inputs)."""
import pytest

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("M,N,K", [(128, 16, 16), (128, 128, 64), (256, 128, 128), (128, 256, 96), (512, 16, 128),
                                   (128, 128, 4096)])
def test_tc_gemm_matches_torch(pkg, M, N, K):
    torch = pytest.importorskip("torch")
    g = torch.Generator(device="cpu").manual_seed(M + N + K)
    A = torch.randn(M, K, generator=g).to(torch.bfloat16).cuda()
    B = torch.randn(N, K, generator=g).to(torch.bfloat16).cuda()
    D = torch.full((M, N), float("nan"), dtype=torch.float32, device="cuda")
    pkg.get_context().tc_gemm_bf16(M, N, K, A.data_ptr(), B.data_ptr(), D.data_ptr(),
                                   stream=torch.cuda.current_stream().cuda_stream)
    ref = A.float() @ B.float().t()
    err = (D - ref).abs().max().item()
    assert err <= 1e-3 * ref.abs().max().item() + 1e-3, err
