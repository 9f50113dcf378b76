"""The tcgen05 BF16 GEMM (dpg_gemm_bf16) against the CUDA-core reference
kernel and an FP64 numpy product of the same bf16 inputs.

Tolerance: |C - C_ref| <= 1e-3 * sum_k |A_mk B_nk| + 1e-5 (FP32 accumulation
in a different order; inputs are exact bf16)."""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _run(lib, torch, M, N, K, impl, split=1, seed=0):
    g = torch.Generator().manual_seed(seed)
    A = torch.randn(M, K, generator=g).to(torch.bfloat16)
    B = torch.randn(N, K, generator=g).to(torch.bfloat16)
    Ad, Bd = A.cuda(), B.cuda()
    Cd = torch.empty(M, N, dtype=torch.float32, device="cuda")
    rc = lib.dpg_gemm_bf16(C.c_void_p(Ad.data_ptr()), C.c_void_p(Bd.data_ptr()), C.c_void_p(Cd.data_ptr()),
                           M, N, K, impl, split)
    assert rc == 0, rc
    a, b = A.float().numpy().astype(np.float64), B.float().numpy().astype(np.float64)
    return Cd.cpu().numpy(), a @ b.T, np.abs(a) @ np.abs(b).T


@pytest.mark.parametrize("M,N,K", [(128, 16, 64), (128, 256, 256), (300, 96, 128), (1024, 256, 256),
                                   (256, 48, 640)])
def test_tcgen05_gemm_matches_reference(dpg_lib, M, N, K):
    torch = pytest.importorskip("torch")
    dpg_lib.dpg_gemm_bf16.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_int, C.c_int, C.c_int, C.c_int,
                                      C.c_int]
    c_tc, exact, mag = _run(dpg_lib, torch, M, N, K, 0)
    c_ref, _, _ = _run(dpg_lib, torch, M, N, K, 1)
    tol = 1e-3 * mag + 1e-5
    assert (np.abs(c_ref - exact) <= tol).all()
    bad = np.abs(c_tc - exact) > tol
    assert not bad.any(), f"{bad.sum()} of {bad.size} differ; first {np.argwhere(bad)[:4].tolist()}"


@pytest.mark.parametrize("split", [2, 8])
def test_tcgen05_gemm_split_k(dpg_lib, split):
    torch = pytest.importorskip("torch")
    dpg_lib.dpg_gemm_bf16.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_int, C.c_int, C.c_int, C.c_int,
                                      C.c_int]
    c_tc, exact, mag = _run(dpg_lib, torch, 256, 256, 4096, 0, split=split)
    assert (np.abs(c_tc - exact) <= 1e-3 * mag + 1e-5).all()


@pytest.mark.parametrize("M,N,K,split", [(128, 16, 64, 1), (128, 256, 256, 1), (300, 96, 128, 1),
                                         (1024, 256, 256, 1), (256, 48, 640, 1), (16, 256, 1024, 4),
                                         (256, 128, 4096, 8), (4096, 144, 320, 1)])
def test_tma_gemm_matches_reference(dpg_lib, M, N, K, split):
    """impl 2: the TMA-fed, warp-specialised kernel (multi-stage ring; rows
    beyond M and tiles taller than the matrix load as zeros)."""
    torch = pytest.importorskip("torch")
    dpg_lib.dpg_gemm_bf16.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_int, C.c_int, C.c_int, C.c_int,
                                      C.c_int]
    c_tc, exact, mag = _run(dpg_lib, torch, M, N, K, 2, split=split)
    bad = np.abs(c_tc - exact) > 1e-3 * mag + 1e-5
    assert not bad.any(), f"{bad.sum()} of {bad.size} differ; first {np.argwhere(bad)[:4].tolist()}"


def test_bounded_wait_gives_up_and_device_stays_usable(dpg_lib):
    """The bounded mbarrier wait of the tensor-core kernels, made to run out:
    nothing completes the barrier (no copy or MMA is issued), the wait gives
    up after its polls, the kernel records the timeout, frees its tensor
    memory and returns DPG_ERR_TIMEOUT; the next tensor-core GEMM runs."""
    torch = pytest.importorskip("torch")
    from dynoplan_gb300 import _lib
    for _ in range(2):
        assert dpg_lib.dpg_mlp_wait_selftest(0, 4096) == _lib.DPG_ERR_TIMEOUT
    got, ref, mag = _run(dpg_lib, torch, 256, 64, 128, 2)
    assert (np.abs(got - ref) <= 1e-3 * mag + 1e-5).all()
