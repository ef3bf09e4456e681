"""The surrogate's tensor-core kernels (tcgen05, BF16 in, FP32 accumulate)
against CPU products of the same BF16 values.  Bar: rel 1e-5 of the product
scale (FP32 accumulation of exact BF16 products)."""
import numpy as np
import pytest

from swap_gb300 import abi

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("K", [16, 64, 256])
def test_tc_gemm_matches_cpu(K):
    import torch

    lib = abi.load()
    g = torch.Generator().manual_seed(K)
    A = torch.randn(128, K, generator=g).to(torch.bfloat16)
    B = torch.randn(32, K, generator=g).to(torch.bfloat16)
    want = A.double() @ B.double().T
    dA, dB = A.cuda(), B.cuda()
    D = torch.zeros(128, 32, dtype=torch.float32, device="cuda")
    r = lib.swap_tc_gemm_check(dA.data_ptr(), dB.data_ptr(), D.data_ptr(), K)
    assert r == 0
    got = D.cpu().double()
    err = (got - want).abs().max().item() / want.abs().max().item()
    assert err < 1e-5, err


def conv3_ref(X, W, bias, dims):
    """Periodic 3x3x3 convolution in float64 on the CPU: X [V][cin], W
    [27][cout][cin] with tap = (dz+1)*9 + (dy+1)*3 + (dx+1)."""
    import torch
    import torch.nn.functional as F

    nx, ny, nz = dims
    cin, cout = X.shape[1], W.shape[1]
    x = X.double().T.reshape(1, cin, nz, ny, nx)
    w = W.double().reshape(3, 3, 3, cout, cin).permute(3, 4, 0, 1, 2)  # (cout, cin, kz, ky, kx)
    y = F.conv3d(F.pad(x, (1, 1, 1, 1, 1, 1), mode="circular"), w)
    y = y.reshape(cout, -1).T
    return y + (bias.double() if bias is not None else 0.0)


@pytest.mark.parametrize("cin,cout,dims", [(16, 32, (8, 8, 4)), (32, 32, (16, 8, 8)), (32, 16, (8, 4, 8)),
                                           (16, 16, (32, 4, 2))])
def test_conv3_matches_cpu(cin, cout, dims):
    import torch

    lib = abi.load()
    V = dims[0] * dims[1] * dims[2]
    g = torch.Generator().manual_seed(cin * 100 + cout)
    X = torch.randn(V, cin, generator=g).to(torch.bfloat16)
    W = (0.1 * torch.randn(27, cout, cin, generator=g)).to(torch.bfloat16)
    b = torch.randn(cout, generator=g).float()
    want = conv3_ref(X, W, b, dims)
    Yf = torch.zeros(V, cout, dtype=torch.float32, device="cuda")
    Y = torch.zeros(V, cout, dtype=torch.bfloat16, device="cuda")
    dX, dW, db = X.cuda(), W.cuda(), b.cuda()
    r = lib.swap_conv3_check(*dims, cin, cout, dX.data_ptr(), dW.data_ptr(), db.data_ptr(), Y.data_ptr(),
                             Yf.data_ptr(), 1)
    assert r == 0
    got = Yf.cpu().double()
    assert (got - want).abs().max().item() / want.abs().max().item() < 1e-5
    gelu = torch.nn.functional.gelu(want)  # exact (erf) GELU, then bf16
    assert (Y.cpu().double() - gelu).abs().max().item() <= 1e-2 * gelu.abs().max().item()
