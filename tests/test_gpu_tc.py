"""GPU: the tcgen05 GEMM against an FP32 matmul of the same (BF16 / TF32-representable) operands."""
import pytest

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")


@pytest.fixture(scope="module")
def lib():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from pibronic_gb300 import build, _native
    return _native.load(build.build())


def _run(lib, fmt, M, N, K, seed=0):
    from pibronic_gb300 import _native
    g = torch.Generator(device="cpu").manual_seed(seed)
    A = torch.randn((M, K), generator=g)
    B = torch.randn((N, K), generator=g)
    if fmt == 1:
        A, B = A.to(torch.bfloat16), B.to(torch.bfloat16)
        ref = A.float() @ B.float().T
    else:
        # values exactly representable in TF32 (10-bit mantissa)
        A = (A * 1024).round() / 1024
        B = (B * 1024).round() / 1024
        ref = A.double() @ B.double().T
    A, B = A.cuda().contiguous(), B.cuda().contiguous()
    C = torch.full((M, N), float("nan"), device="cuda")
    st = torch.zeros(1, dtype=torch.int32, device="cuda")
    _native.check(lib.pbr_tc_gemm(fmt, _native.ptr(A), _native.ptr(B), _native.ptr(C), M, N, K,
                                  _native.ptr(st), _native.stream_handle()), "pbr_tc_gemm")
    torch.cuda.synchronize()
    assert int(st.item()) == 0
    return C.cpu().double(), ref.double()


@pytest.mark.parametrize("fmt,M,N,K", [(1, 128, 64, 64), (1, 256, 256, 256), (1, 384, 48, 128),
                                       (2, 128, 32, 32), (2, 256, 144, 96)])
def test_tc_gemm_matches_fp32(lib, fmt, M, N, K):
    C, ref = _run(lib, fmt, M, N, K)
    assert torch.allclose(C, ref, rtol=1e-4, atol=1e-3 * ref.abs().max().item())
