"""Kernel-level GPU tests: the tcgen05 BF16x3 GEMM against a PyTorch FP32
reference of the same operation (and its exact BF16-split emulation), from
one tile to more tiles than SMs (persistent CTAs, both TMEM accumulators)."""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _lib():
    from wavebem_gb300.bem_problem import load_library
    L = load_library()
    L.wbem_test_gemm_bf16x3.argtypes = [ctypes.c_int] * 3 + [ctypes.c_void_p] * 3
    return L


@pytest.mark.parametrize("M,Nc,K", [(128, 256, 64), (300, 520, 128), (1000, 777, 128), (256, 512, 256),
                                    (64, 40, 32), (2048, 1000, 512), (4096, 4096, 128)])
def test_gemm_bf16x3_matches_torch(M, Nc, K):
    torch = pytest.importorskip("torch")
    g = torch.Generator(device="cpu").manual_seed(M + Nc + K)
    A = torch.randn(M, K, generator=g).cuda()
    B = torch.randn(Nc, K, generator=g).cuda()
    C = torch.randn(M, Nc, generator=g).cuda()
    C0 = C.clone()
    st = _lib().wbem_test_gemm_bf16x3(M, Nc, K, A.data_ptr(), B.data_ptr(), C.data_ptr())
    assert st == 0
    ref = (C0.double() - A.double() @ B.double().T)
    # BF16x3 keeps ~16 significant bits per operand: tolerance 1e-4 of |A||B^T|
    scale = (A.double().abs() @ B.double().abs().T)
    err = ((C.double() - ref).abs() / scale).max().item()
    assert err < 1e-4, err
    # exact emulation of the three BF16 products (FP32 accumulation order aside)
    Ah = A.bfloat16().float(); Al = (A - Ah).bfloat16().float()
    Bh = B.bfloat16().float(); Bl = (B - Bh).bfloat16().float()
    emu = C0.double() - (Ah.double() @ Bh.double().T + Ah.double() @ Bl.double().T + Al.double() @ Bh.double().T)
    err2 = ((C.double() - emu).abs() / scale).max().item()
    assert err2 < 2e-6, err2


def _tf32(x, mode):
    """FP32 -> TF32 (10 mantissa bits) by truncation or round-to-nearest-even."""
    torch = pytest.importorskip("torch")
    u = x.contiguous().view(torch.int32).to(torch.int64) & 0xFFFFFFFF
    if mode == "rn":
        u = u + 0xFFF + ((u >> 13) & 1)
    u = (u & 0xFFFFE000)
    u = torch.where(u >= 2 ** 31, u - 2 ** 32, u).to(torch.int32)
    return u.view(torch.float32)


@pytest.mark.parametrize("M,Nc,K", [(128, 256, 64), (300, 520, 128), (1000, 777, 512), (64, 40, 32),
                                    (2048, 1000, 512), (4096, 4096, 128)])
def test_gemm_tf32_matches_torch(M, Nc, K):
    """The factorisation's trailing update: one TF32 product, against FP64
    (TF32 keeps 11 significant bits per operand: 2e-3 of |A||B^T|) and against
    the exact TF32 emulation, which must match to FP32 accumulation order."""
    torch = pytest.importorskip("torch")
    L = _lib()
    L.wbem_test_gemm_tf32.argtypes = [ctypes.c_int] * 3 + [ctypes.c_void_p] * 3
    g = torch.Generator(device="cpu").manual_seed(7 * M + Nc + K)
    A = torch.randn(M, K, generator=g).cuda()
    B = torch.randn(Nc, K, generator=g).cuda()
    C = torch.randn(M, Nc, generator=g).cuda()
    C0 = C.clone()
    assert L.wbem_test_gemm_tf32(M, Nc, K, A.data_ptr(), B.data_ptr(), C.data_ptr()) == 0
    scale = A.double().abs() @ B.double().abs().T
    ref = C0.double() - A.double() @ B.double().T
    assert ((C.double() - ref).abs() / scale).max().item() < 2e-3
    errs = {}
    for mode in ("trunc", "rn"):
        emu = C0.double() - _tf32(A, mode).double() @ _tf32(B, mode).double().T
        errs[mode] = ((C.double() - emu).abs() / scale).max().item()
    assert min(errs.values()) < 2e-6, errs
