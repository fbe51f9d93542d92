"""GPU: the tcgen05 TF32 GEMM (C = alpha A Bᵀ + beta C) against an FP32
reference of the same operation."""

import pytest
import torch

from lineax_gb300 import _blas

pytestmark = pytest.mark.gpu


def ref(a, b, c, alpha, beta):
    torch.backends.cuda.matmul.allow_tf32 = False
    out = alpha * (a.double() @ b.double().T)
    if c is not None:
        out = out + beta * c.double()
    return out


@pytest.mark.parametrize("m,n,k", [(128, 128, 32), (128, 128, 8), (256, 384, 200), (1000, 700, 64),
                                   (130, 260, 96), (512, 512, 512), (64, 128, 300)])
def test_tf32_gemm_matches_fp32_reference(dev, m, n, k):
    g = torch.Generator(device=dev).manual_seed(m * 131 + n * 7 + k)
    a = torch.randn(m, k, device=dev, generator=g)
    b = torch.randn(n, k, device=dev, generator=g)
    c = torch.randn(m, n, device=dev, generator=g)
    c0 = c.clone()
    out = _blas.gemm_tf32_nt(a, b, c, alpha=-1.0, beta=1.0)
    r = ref(a, b, c0, -1.0, 1.0)
    # TF32 keeps 10 mantissa bits: per-product relative error <= 2^-10; the
    # sum of k products is bounded by k * 2^-10 * max|a||b| (stated bound).
    bound = (k * 2.0 ** -10) * float(a.abs().max() * b.abs().max()) + 1e-5
    assert float((out.double() - r).abs().max()) <= bound
    # and the typical error is that of TF32 rounding, far below the bound
    rel = float((out.double() - r).norm() / r.norm())
    assert rel < 5e-3, rel


def test_tf32_gemm_beta_zero_and_k_zero(dev):
    a = torch.randn(200, 0, device=dev)
    b = torch.randn(150, 0, device=dev)
    c = torch.full((200, 150), 3.0, device=dev)
    _blas.gemm_tf32_nt(a, b, c, alpha=1.0, beta=0.5)
    assert torch.allclose(c, torch.full_like(c, 1.5))


@pytest.mark.parametrize("m,n,k", [(128, 128, 32), (300, 260, 64), (512, 512, 512)])
def test_3xtf32_gemm_reaches_fp32_accuracy(dev, m, n, k):
    g = torch.Generator(device=dev).manual_seed(m + n + k)
    a = torch.randn(m, k, device=dev, generator=g)
    b = torch.randn(n, k, device=dev, generator=g)
    out = _blas.gemm_3xtf32_nt(a, b)
    r = ref(a, b, None, 1.0, 0.0)
    rel = float((out.double() - r).norm() / r.norm())
    # FP32-level: sqrt(k) 2^-24 accumulation plus the dropped lo*lo term
    # (plain TF32 products give ~1e-3 here)
    assert rel < 1e-5, rel


@pytest.mark.parametrize("layout", ["aligned", "odd_ld", "offset", "beta0"])
def test_tf32_gemm_epilogue_layouts(dev, layout):
    """C updated through the TMA epilogue (16-byte base and row stride) and
    through the direct-store epilogue (any other C) gives the same values."""
    m, n, k = 300, 200, 64
    g = torch.Generator(device=dev).manual_seed(17)
    a = torch.randn(m, k, device=dev, generator=g)
    b = torch.randn(n, k, device=dev, generator=g)
    big = torch.randn(m + 1, n + 5, device=dev, generator=g)
    if layout == "odd_ld":
        c = big[:m, :n]            # row stride n + 5: not a multiple of 4
    elif layout == "offset":
        c = big[1:, 1:n + 1]       # base 4 bytes past a 16-byte boundary
    else:
        c = torch.randn(m, n, device=dev, generator=g)
    beta = 0.0 if layout == "beta0" else 1.0
    c0 = c.clone()
    outside = big.clone()
    _blas.gemm_tf32_nt(a, b, c, alpha=-1.0, beta=beta)
    r = ref(a, b, c0, -1.0, beta)
    bound = (k * 2.0 ** -10) * float(a.abs().max() * b.abs().max()) + 1e-5
    assert float((c.double() - r).abs().max()) <= bound
    if layout in ("odd_ld", "offset"):   # nothing outside the C view was written
        mask = torch.ones_like(big, dtype=torch.bool)
        if layout == "odd_ld":
            mask[:m, :n] = False
        else:
            mask[1:, 1:n + 1] = False
        assert torch.equal(big[mask], outside[mask])


@pytest.mark.parametrize("m,n,k", [(128, 128, 64), (128, 128, 16), (256, 384, 200),
                                   (1000, 700, 64), (130, 260, 96), (512, 512, 512)])
def test_bf16_gemm_matches_reference(dev, m, n, k):
    """lxgb_gemm_bf16_nt (tcgen05 kind::f16, BF16 operands, FP32 accumulation):
    products of BF16 values are exact in FP32, so against the product of the
    BF16-rounded operands the error is the FP32 accumulation's, k 2^-24."""
    from lineax_gb300 import _ffi

    g = torch.Generator(device=dev).manual_seed(m * 17 + n * 3 + k)
    a = torch.randn(m, k, device=dev, generator=g).to(torch.bfloat16)
    b = torch.randn(n, k, device=dev, generator=g).to(torch.bfloat16)
    ka = (k + 7) // 8 * 8  # row strides: multiples of 8 elements (16 bytes)
    ap = torch.zeros(m, ka, dtype=torch.bfloat16, device=dev)
    bp = torch.zeros(n, ka, dtype=torch.bfloat16, device=dev)
    ap[:, :k] = a
    bp[:, :k] = b
    c = torch.randn(m, n, device=dev, generator=g)
    c0 = c.clone()
    err = torch.zeros(1, dtype=torch.int32, device=dev)
    _ffi.call("lxgb_gemm_bf16_nt", m, n, k, _ffi.ptr(ap), ka, _ffi.ptr(bp), ka, _ffi.ptr(c), n,
              -1.0, 1.0, _ffi.ptr(err), _ffi.stream_handle(dev))
    torch.cuda.synchronize()
    assert int(err.item()) == 0
    r = c0.double() - a.double() @ b.double().T
    scale = (a.double().abs() @ b.double().abs().T) + c0.double().abs()
    assert float(((c.double() - r).abs() / scale).max()) <= (k + 2) * 2.0 ** -23


def _run_mode(mode, a, b, c, alpha, beta):
    from lineax_gb300 import _ffi

    if mode == "tf32":
        return _blas.gemm_tf32_nt(a, b, c, alpha=alpha, beta=beta)
    if mode == "3xtf32":
        return _blas.gemm_3xtf32_nt(a, b, c, alpha=alpha, beta=beta)
    m, k = a.shape
    n = b.shape[0]
    ah, bh = a.to(torch.bfloat16).contiguous(), b.to(torch.bfloat16).contiguous()
    err = torch.zeros(1, dtype=torch.int32, device=a.device)
    _ffi.call("lxgb_gemm_bf16_nt", m, n, k, _ffi.ptr(ah), k, _ffi.ptr(bh), k, _ffi.ptr(c),
              c.stride(0), float(alpha), float(beta), _ffi.ptr(err), _ffi.stream_handle(a.device))
    torch.cuda.synchronize()
    assert int(err.item()) == 0
    return c


@pytest.mark.parametrize("mode", ["tf32", "3xtf32", "bf16"])
@pytest.mark.parametrize("m,n,k,beta", [(4096, 4096, 64, 1.0), (2000, 3000, 96, 1.0),
                                        (1100, 700, 304, 0.0), (4500, 520, 64, 0.5),
                                        (129, 257, 40, 1.0)])
def test_persistent_kernel_matches_tile_kernel(dev, mode, m, n, k, beta):
    """The persistent GEMM (one CTA per SM, two tensor-memory accumulators,
    several tiles per CTA at these sizes, ragged right and bottom tiles) gives
    the values of the one-tile-per-CTA kernel: the same products accumulated
    in the same K order, the same epilogue."""
    from lineax_gb300 import _ffi

    g = torch.Generator(device=dev).manual_seed(m + 3 * n + 7 * k)
    a = torch.randn(m, k, device=dev, generator=g)
    b = torch.randn(n, k, device=dev, generator=g)
    c0 = torch.randn(m, n, device=dev, generator=g)
    try:
        _ffi.call("lxgb_gemm_set_persistent", 0)
        tile = _run_mode(mode, a, b, c0.clone(), -1.0, beta)
    finally:
        _ffi.call("lxgb_gemm_set_persistent", 1)
    pers = _run_mode(mode, a, b, c0.clone(), -1.0, beta)
    torch.cuda.synchronize()
    diff = float((pers.double() - tile.double()).abs().max())
    scale = float(((a.double().abs() @ b.double().abs().T) + c0.double().abs()).max())
    assert diff <= (k + 2) * 2.0 ** -23 * scale, (diff, scale)
    print(f"{mode} {m}x{n}x{k} beta={beta}: max |persistent - tile| = {diff:.3e}"
          f" ({'bit-identical' if diff == 0 else 'differs'})")
