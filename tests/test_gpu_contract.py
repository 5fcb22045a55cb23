"""The split-TF32 tensor-core contraction (fd2d_contract_f32) against FP64 torch."""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ctx(fd2d_lib):
    import torch
    from fd2d_noise_gb300 import _lib
    c = _lib.Context(0, _lib.PREC_FP32)
    c.set_memspace(_lib.MEM_DEVICE)
    s = torch.cuda.Stream()
    c.set_stream(s.cuda_stream)
    c.torch_stream = s
    yield c
    c.close()


@pytest.mark.parametrize("M,N,Kd", [(128, 256, 32), (1000, 300, 70), (4096, 600, 600), (300, 17, 5)])
def test_contract_matches_fp64(ctx, M, N, Kd):
    import torch
    from fd2d_noise_gb300 import _lib
    g = torch.Generator(device="cpu").manual_seed(M + N + Kd)
    A = torch.randn(Kd, M, generator=g, dtype=torch.float64)
    B = torch.randn(Kd, N, generator=g, dtype=torch.float64)
    A32, B32 = A.float().cuda(), B.float().cuda()
    R = torch.full((N, M), float("nan"), dtype=torch.float32, device="cuda")
    torch.cuda.synchronize()
    st = ctx.L.fd2d_contract_f32(ctx.h, ctypes.c_void_p(A32.data_ptr()), ctypes.c_int64(M),
                                 ctypes.c_void_p(B32.data_ptr()), ctypes.c_int64(N), M, N, Kd,
                                 ctypes.c_void_p(R.data_ptr()), ctypes.c_int64(M))
    _lib.check(st, ctx.h)
    ctx.synchronize()
    ref = (B32.double().T @ A32.double())  # exact products of the FP32 inputs
    err = (R.double() - ref).norm() / ref.norm()
    assert torch.isfinite(R).all()
    # FP32 accumulation in tensor memory: error grows with depth (about 5e-6 at Kd = 600)
    assert err < 1e-5, float(err)
