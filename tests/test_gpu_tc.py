"""The tcgen05 tensor-core GEMM (3xTF32 split) against an FP64 torch product.

C = beta*C + alpha*A*B^T with A (M x K) and B (N x K) K-major, split into
TF32 heads and FP32 remainders.  Tolerances: 3-term split 1e-5 (FP32-level),
head-only product 5e-3 (TF32-level), relative Frobenius.
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _split(x):
    import torch
    h = (x.view(torch.int32) & ~0x1FFF).view(torch.float32)
    return h.contiguous(), (x - h).contiguous()


def _lib():
    from openmeeg_gb300 import _lib
    lib = _lib.load()
    f = lib.omg_internal_gemm_tf32x3
    f.restype = ctypes.c_int
    f.argtypes = [ctypes.c_int64, ctypes.c_int64, ctypes.c_int64, ctypes.c_float, ctypes.c_void_p, ctypes.c_void_p,
                  ctypes.c_int64, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int64, ctypes.c_float, ctypes.c_void_p,
                  ctypes.c_int64, ctypes.c_int, ctypes.c_void_p]
    return f


def _run(M, N, K, alpha, beta, lower, three, seed=0):
    import torch
    f = _lib()
    g = torch.Generator(device="cuda").manual_seed(seed)
    A = torch.randn(M, K, device="cuda", generator=g, dtype=torch.float32)
    B = A if lower else torch.randn(N, K, device="cuda", generator=g, dtype=torch.float32)
    Ah, Al = _split(A)
    Bh, Bl = _split(B)
    C0 = torch.randn(N, M, device="cuda", generator=g, dtype=torch.float32)   # column-major M x N
    C = C0.clone()
    err = torch.zeros(1, dtype=torch.int32, device="cuda")
    p = lambda t: ctypes.c_void_p(t.data_ptr()) if t is not None else ctypes.c_void_p(0)
    rc = f(M, N, K, alpha, p(Ah), p(Al if three else None), K, p(Bh), p(Bl if three else None), K, beta, p(C), M,
           1 if lower else 0, p(err))
    assert rc == 0 and int(err.item()) == 0
    ref = (beta * C0.double().T + alpha * (A.double() @ B.double().T))
    got = C.double().T
    if lower:
        mask = torch.tril(torch.ones(M, N, dtype=torch.bool, device="cuda"))
        # entries above the diagonal are untouched
        assert torch.equal(got[~mask], C0.double().T[~mask])
        ref, got = ref[mask], got[mask]
    return float(torch.linalg.norm(got - ref) / torch.linalg.norm(ref))


@pytest.mark.parametrize("M,N,K", [(128, 128, 32), (300, 200, 128), (1000, 215, 96)])
def test_tc_gemm_3xtf32_general(cuda, M, N, K):
    assert _run(M, N, K, 1.0, 0.0, False, True) < 1e-5
    assert _run(M, N, K, -1.0, 1.0, False, True) < 1e-5


def test_tc_gemm_head_only_is_tf32_accurate(cuda):
    e = _run(256, 256, 128, 1.0, 0.0, False, False)
    assert 1e-6 < e < 5e-3


def test_tc_gemm_lower_update(cuda):
    assert _run(640, 640, 128, -1.0, 1.0, True, True) < 1e-5


@pytest.mark.parametrize("M,N,K,lower", [(5000, 1000, 64, False), (4100, 4100, 128, True)])
def test_tc_gemm_many_tiles_per_cta(cuda, M, N, K, lower):
    # more tiles than SMs: every CTA walks several tiles through both TMEM accumulators
    assert _run(M, N, K, -1.0, 1.0, lower, True) < 1e-5
