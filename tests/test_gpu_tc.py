"""Tensor-core GEMM (tcgen05.mma kind::f16, BF16 operands, FP32 accumulation in TMEM) against an
FP64 product of the same BF16 inputs.  FP32 accumulation over K terms bounds the error by about
K * 2^-24 relative to sum |a_k b_k|; the test allows 1e-5 of that scale."""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def bf16_bits(x):
    """Round-to-nearest-even BF16 bit patterns (uint16) and their float64 values."""
    f = np.ascontiguousarray(x, np.float32)
    u = f.view(np.uint32).astype(np.uint64)
    r = ((u + 0x7FFF + ((u >> 16) & 1)) >> 16).astype(np.uint16)
    back = (r.astype(np.uint32) << 16).view(np.float32).astype(np.float64)
    return r, back


@pytest.mark.parametrize("m,n,k", [(128, 16, 64), (256, 48, 192), (384, 256, 320), (128, 128, 1024)])
def test_tc_gemm_matches_fp64(agb, m, n, k):
    import torch
    from aurora_gb300 import _abi
    rng = np.random.default_rng(m + n + k)
    a, a64 = bf16_bits(rng.normal(0, 1, (m, k)))
    b, b64 = bf16_bits(rng.normal(0, 1, (n, k)))
    ad = torch.from_numpy(a.view(np.int16)).cuda()
    bd = torch.from_numpy(b.view(np.int16)).cuda()
    dd = torch.zeros((m, n), dtype=torch.float32, device="cuda")
    _abi.check(agb.agb_tc_gemm_bf16(ad.data_ptr(), bd.data_ptr(), dd.data_ptr(), m, n, k, None))
    d = dd.cpu().numpy()
    ref = a64 @ b64.T
    scale = np.abs(a64) @ np.abs(b64).T
    err = np.abs(d - ref) / scale
    print(f"{m}x{n}x{k}: max error / sum|ab| = {err.max():.3g}")
    assert err.max() < 1e-5
