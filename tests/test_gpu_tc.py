"""tcgen05 GEMM (BF16 operands, FP32 accumulation in tensor memory) against
the FP32 product of the same BF16 values.  Tolerance: relative error of the
whole matrix <= 1e-5 (only the summation order differs)."""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("M,N,K", [(128, 16, 64), (256, 256, 128), (300, 208, 1856), (1000, 256, 256),
                                   (130, 512, 64)])
@pytest.mark.parametrize("act", [0, 1])
def test_tc_gemm(gpu_lib, M, N, K, act):
    torch = pytest.importorskip("torch")
    L = gpu_lib.lib()
    g = torch.Generator(device="cpu").manual_seed(M + N + K)
    A = torch.randn(M, K, generator=g).to(torch.bfloat16).cuda()
    B = torch.randn(N, K, generator=g).to(torch.bfloat16).cuda()
    bias = torch.randn(N, generator=g).cuda()
    C = torch.zeros(M, N, device="cuda")
    Cb = torch.zeros(M, N, device="cuda", dtype=torch.bfloat16)
    P = lambda t: ctypes.c_void_p(t.data_ptr())
    rc = L.moloch_tc_gemm(P(A), K, P(B), K, P(C), N, P(Cb), N, P(bias), M, N, K, act, None)
    assert rc == 0, L.moloch_gpu_last_error()
    assert L.moloch_tc_status() == 0
    ref = A.float() @ B.float().T + bias
    err = (C - ref).norm() / ref.norm()
    assert err.item() <= 1e-5, err.item()
    refb = torch.nn.functional.silu(ref) if act == 1 else ref
    errb = (Cb.float() - refb).norm() / refb.norm()
    assert errb.item() <= 1e-2, errb.item()


def test_tc_gemm_surrogate_layer1(gpu_lib):
    """The first surrogate layer at 256 x 256 x 40: 65536 columns x 1856
    features -> 256 (BF16 out with SiLU), many tiles per persistent CTA."""
    torch = pytest.importorskip("torch")
    L = gpu_lib.lib()
    M, N, K = 65536, 256, 1856
    g = torch.Generator(device="cpu").manual_seed(7)
    A = torch.randn(M, K, generator=g).to(torch.bfloat16).cuda()
    B = (torch.randn(N, K, generator=g) / K ** 0.5).to(torch.bfloat16).cuda()
    bias = torch.randn(N, generator=g).cuda()
    Cb = torch.zeros(M, N, device="cuda", dtype=torch.bfloat16)
    P = lambda t: ctypes.c_void_p(t.data_ptr())
    rc = L.moloch_tc_gemm(P(A), K, P(B), K, None, 0, P(Cb), N, P(bias), M, N, K, 1, None)
    assert rc == 0, L.moloch_gpu_last_error()
    assert L.moloch_tc_status() == 0
    for r0 in (0, 30000, M - 512):
        ref = torch.nn.functional.silu(A[r0:r0 + 512].float() @ B.float().T + bias)
        err = (Cb[r0:r0 + 512].float() - ref).norm() / ref.norm()
        assert err.item() <= 1e-2, (r0, err.item())


def test_tc_gemm_rejects_bad_shapes(gpu_lib):
    L = gpu_lib.lib()
    dummy = ctypes.c_void_p(16)
    assert L.moloch_tc_gemm(dummy, 72, dummy, 72, dummy, 24, None, 0, None, 128, 24, 72, 0, None) == 1


def test_tc_gemm_wait_runs_out(gpu_lib):
    """CTA 0's loader leaves its second K chunk unarmed and unissued (test
    hook), with the wait limit at 2e6 SM cycles: the MMA issuer's wait for
    that chunk, then the loader's wait for the stage it never frees, the
    epilogue's wait for the accumulator and the final drain's wait for the
    unissued chunk all run out.  moloch_tc_status reports MOLOCH_ERR_TIMEOUT,
    and the next GEMM, with the hook off, is correct (the kernel drained its
    loads in flight and freed its tensor memory)."""
    torch = pytest.importorskip("torch")
    L = gpu_lib.lib()
    M, N, K = 256, 64, 512
    g = torch.Generator(device="cpu").manual_seed(3)
    A = torch.randn(M, K, generator=g).to(torch.bfloat16).cuda()
    B = torch.randn(N, K, generator=g).to(torch.bfloat16).cuda()
    C = torch.zeros(M, N, device="cuda")
    P = lambda t: ctypes.c_void_p(t.data_ptr())
    assert L.moloch_tc_set_wait_limit(2_000_000, 0, 1) == 0
    try:
        assert L.moloch_tc_gemm(P(A), K, P(B), K, P(C), N, None, 0, None, M, N, K, 0, None) == 0
        assert L.moloch_tc_status() == 6  # MOLOCH_ERR_TIMEOUT
    finally:
        assert L.moloch_tc_set_wait_limit(0, -1, -1) == 0
    C.zero_()
    assert L.moloch_tc_gemm(P(A), K, P(B), K, P(C), N, None, 0, None, M, N, K, 0, None) == 0
    assert L.moloch_tc_status() == 0
    ref = A.float() @ B.float().T
    err = (C - ref).norm() / ref.norm()
    assert err.item() <= 1e-5, err.item()
