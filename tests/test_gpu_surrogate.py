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
