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


# ---- implicit 3x3 convolution (rf_conv3x3_bf16) against PyTorch's FP32 conv2d of the same BF16
# operands: zero padding at every border, nearest-neighbour upsampling of the first input,
# channel concatenation, M tails, N over several tiles, every epilogue

def _conv_ops(n, h, w, ca, cb, N, up, seed):
    g = torch.Generator(device="cuda").manual_seed(seed)
    ha, wa = (h // 2, w // 2) if up else (h, w)
    xa = torch.randn(n, ha, wa, ca, device="cuda", generator=g).to(torch.bfloat16)
    xb = torch.randn(n, h, w, cb, device="cuda", generator=g).to(torch.bfloat16) if cb else None
    wt = torch.randn(N, 9 * (ca + cb), device="cuda", generator=g).to(torch.bfloat16)
    return xa, xb, wt


def _conv_ref(xa, xb, wt, up, absolute=False):
    import torch.nn.functional as F
    f = (lambda t: t.float().abs()) if absolute else (lambda t: t.float())
    x = f(xa).permute(0, 3, 1, 2)
    if up:
        x = x.repeat_interleave(2, dim=2).repeat_interleave(2, dim=3)
    if xb is not None:
        x = torch.cat([x, f(xb).permute(0, 3, 1, 2)], dim=1)
    C = x.shape[1]
    k = f(wt).view(-1, 9, C).permute(0, 2, 1).reshape(-1, C, 3, 3)
    y = F.conv2d(x, k, padding=1)
    return y.permute(0, 2, 3, 1).reshape(-1, wt.shape[0])


@pytest.mark.parametrize("n,h,w,ca,cb,N,up", [(2, 16, 24, 8, 0, 32, False), (1, 37, 53, 48, 0, 48, False),
                                              (2, 32, 48, 64, 48, 48, True), (1, 20, 20, 96, 64, 64, True),
                                              (3, 9, 130, 32, 0, 96, False), (1, 40, 24, 16, 8, 200, False),
                                              (1, 12, 20, 16, 0, 16, False), (2, 16, 300, 32, 32, 48, True),
                                              (1, 8, 8, 96, 96, 96, False)])
def test_conv3x3_store_f32(rk, n, h, w, ca, cb, N, up):
    xa, xb, wt = _conv_ops(n, h, w, ca, cb, N, up, n * 1000 + h * 10 + N)
    c = torch.full((n * h * w, N), float("nan"), device="cuda")
    rk.conv3x3_bf16(xa, wt, c, xb=xb, up=up)
    ref = _conv_ref(xa, xb, wt, up)
    # FP32 accumulation of BF16 products: |err| <= ~K * 2^-24 * sum|x||w|
    tol = 1e-5 * _conv_ref(xa, xb, wt, up, absolute=True) + 1e-6
    assert torch.all((c - ref).abs() <= tol), float((c - ref).abs().max())


@pytest.mark.parametrize("relu", [False, True])
def test_conv3x3_bias_relu_bf16(rk, relu):
    n, h, w, ca, cb, N = 2, 24, 40, 64, 48, 48
    xa, xb, wt = _conv_ops(n, h, w, ca, cb, N, True, 17)
    bias = torch.randn(N, device="cuda")
    c = torch.zeros(n * h * w, N, device="cuda", dtype=torch.bfloat16)
    rk.conv3x3_bf16(xa, wt, c, xb=xb, up=True, mode=rk.GEMM_STORE_BF16, bias=bias, relu=relu)
    ref = _conv_ref(xa, xb, wt, True) + bias
    if relu:
        ref = ref.clamp_min(0)
    # one BF16 rounding of the FP32 result
    assert torch.allclose(c.float(), ref, rtol=2 ** -8, atol=2e-3)


def test_conv3x3_atomic_and_strided_output(rk):
    n, h, w, ca, N = 1, 33, 17, 32, 40
    xa, _, wt = _conv_ops(n, h, w, ca, 0, N, False, 23)
    c = torch.ones(n * h * w, 48, device="cuda")[:, :N]
    rk.conv3x3_bf16(xa, wt, c, mode=rk.GEMM_ATOMIC_F32)
    assert torch.allclose(c, 1.0 + _conv_ref(xa, None, wt, False), rtol=1e-4, atol=1e-3)


def test_conv3x3_bad_arguments_rejected(rk):
    xa, _, wt = _conv_ops(1, 8, 8, 12, 0, 16, False, 1)  # 12 channels: not a multiple of 8
    c = torch.zeros(64, 16, device="cuda")
    with pytest.raises(rk.RefraktError):
        rk.conv3x3_bf16(xa, wt, c)
    xa, _, wt = _conv_ops(1, 8, 8, 16, 0, 16, False, 1)
    with pytest.raises(rk.RefraktError):
        rk.conv3x3_bf16(xa, wt, torch.zeros(64, 8, device="cuda"))  # output rows narrower than N
    with pytest.raises(ValueError):
        rk.conv3x3_bf16(xa, wt[:, :96], c)  # weights narrower than 9 (ca + cb)


# ---- the persistent TMA pipeline: shapes with more than two rounds of tiles (152 SMs, one CTA
# each), so every CTA walks several tiles and both tensor-memory accumulators alternate

@pytest.mark.parametrize("M,N,K", [(16384, 768, 192), (65536, 48, 72), (40000, 100, 136)])
def test_persistent_many_tiles(rk, M, N, K):
    a, b = _ops(M, N, K, M + N + K)
    c = torch.full((M, N), float("nan"), device="cuda")
    rk.gemm_bf16(a, b, c)
    ref = _ref(a, b)
    tol = 1e-5 * (a.float().abs() @ b.float().abs().t()) + 1e-6
    assert torch.all((c - ref).abs() <= tol), float((c - ref).abs().max())


def test_persistent_split_k_many_tiles(rk):
    M, N, K, splits = 96, 2048, 65536, 64  # 8 column tiles x 64 splits = 512 tiles
    a, b = _ops(M, N, K, 9)
    c = torch.ones(M, N, device="cuda")
    rk.gemm_bf16(a, b, c, mode=rk.GEMM_ATOMIC_F32, splits=splits)
    ref = 1.0 + _ref(a, b)
    tol = 1e-5 * (a.float().abs() @ b.float().abs().t()) + 1e-4
    assert torch.all((c - ref).abs() <= tol), float((c - ref).abs().max())


def test_persistent_bias_relu_bf16(rk):
    M, N, K = 50000, 96, 200
    a, b = _ops(M, N, K, 13)
    bias = torch.randn(N, device="cuda")
    c = torch.zeros(M, N, device="cuda", dtype=torch.bfloat16)
    rk.gemm_bf16(a, b, c, mode=rk.GEMM_STORE_BF16, bias=bias, relu=True)
    ref = (_ref(a, b) + bias).clamp_min(0)
    assert torch.allclose(c.float(), ref, rtol=2 ** -8, atol=1e-3)
