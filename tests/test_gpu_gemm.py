"""The tcgen05 BF16 GEMM of the learned density estimator against a PyTorch FP32 matmul of the
same BF16 operands: FP32 accumulation, so only the summation order differs (relative tolerance
stated per check); M, N and K tails, N over several tiles, bias + ReLU + BF16 epilogue, split-K
atomic accumulation."""
import pytest
import torch

pytestmark = pytest.mark.gpu


def _ops(M, N, K, seed, pad=0):
    g = torch.Generator(device="cuda").manual_seed(seed)
    a = torch.randn(M, K + pad, device="cuda", generator=g).to(torch.bfloat16)[:, :K]
    b = torch.randn(N, K + pad, device="cuda", generator=g).to(torch.bfloat16)[:, :K]
    return a, b


def _ref(a, b):
    return a.float() @ b.float().t()


@pytest.mark.parametrize("M,N,K", [(128, 64, 64), (128, 16, 8), (256, 48, 72), (300, 96, 1440), (1000, 256, 320),
                                   (128, 300, 64), (77, 130, 200), (4096, 32, 288)])
def test_store_f32(rk, M, N, K):
    a, b = _ops(M, N, K, M * 7 + N)
    c = torch.full((M, N), float("nan"), device="cuda")
    rk.gemm_bf16(a, b, c)
    ref = _ref(a, b)
    # FP32 accumulation of BF16 products: |err| <= ~K * 2^-24 * sum|a||b|
    tol = 1e-5 * (a.float().abs() @ b.float().abs().t()) + 1e-6
    assert torch.all((c - ref).abs() <= tol), float((c - ref).abs().max())


def test_strided_operands(rk):
    a, b = _ops(200, 40, 96, 5, pad=40)  # row strides 136 != K
    c = torch.zeros(200, 48, device="cuda")[:, :40]
    rk.gemm_bf16(a, b, c)
    assert torch.allclose(c, _ref(a, b), rtol=1e-5, atol=1e-4)


@pytest.mark.parametrize("relu", [False, True])
def test_bias_relu_bf16(rk, relu):
    M, N, K = 515, 96, 864
    a, b = _ops(M, N, K, 11)
    bias = torch.randn(N, device="cuda")
    c = torch.zeros(M, N, device="cuda", dtype=torch.bfloat16)
    rk.gemm_bf16(a, b, c, mode=rk.GEMM_STORE_BF16, bias=bias, relu=relu)
    ref = _ref(a, b) + bias
    if relu:
        ref = ref.clamp_min(0)
    # one BF16 rounding of the FP32 result
    assert torch.allclose(c.float(), ref, rtol=2 ** -8, atol=1e-3)


@pytest.mark.parametrize("splits", [1, 3, 16])
def test_split_k_atomic(rk, splits):
    M, N, K = 96, 200, 8192
    a, b = _ops(M, N, K, 3)
    c = torch.ones(M, N, device="cuda")
    rk.gemm_bf16(a, b, c, mode=rk.GEMM_ATOMIC_F32, splits=splits)
    assert torch.allclose(c, 1.0 + _ref(a, b), rtol=1e-4, atol=2e-3)


def test_bad_arguments_rejected(rk):
    a, b = _ops(128, 64, 64, 1)
    c = torch.zeros(128, 64, device="cuda")
    with pytest.raises(rk.RefraktError):
        rk.gemm_bf16(a[:, :60], b[:, :60], c)  # K not a multiple of 8
    with pytest.raises(rk.RefraktError):
        rk.gemm_bf16(a, b, c, splits=2)  # split K without atomic accumulation
