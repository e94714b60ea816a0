"""tcgen05 3xTF32 GEMM (the tensor-core form of the spectral products) vs FP64."""
import pytest
import torch

pytestmark = pytest.mark.gpu


def tc_gemm(A, B):
    from pyaxisymflow_gb300 import _native as N
    M, K = A.shape
    Nn = B.shape[0]
    C = torch.empty((M, Nn), dtype=torch.float32, device=A.device)
    work = torch.empty(N.lib().axi_tf32x3_gemm_work_bytes(M, Nn, K), dtype=torch.uint8,
                       device=A.device)
    N.call("axi_tf32x3_gemm", N.ptr(C), N.ptr(A), N.ptr(B), M, Nn, K, N.ptr(work),
           N.stream_of(A))
    return C


@pytest.mark.parametrize("M,N,K", [(128, 128, 32), (128, 128, 256), (256, 512, 512),
                                   (512, 256, 1024), (200, 136, 72), (1024, 512, 512)])
def test_tf32x3_gemm_matches_fp64(M, N, K):
    g = torch.Generator(device="cpu").manual_seed(M * 7 + N + K)
    A = torch.randn((M, K), generator=g, dtype=torch.float64)
    B = torch.randn((N, K), generator=g, dtype=torch.float64)
    ref = A @ B.T
    C = tc_gemm(A.float().cuda(), B.float().cuda()).double().cpu()
    # FP32-rounded inputs: compare with the exact product of the rounded
    # inputs. 3xTF32 with FP32 accumulation lands at the FP32 level (~1e-6 for
    # K in the hundreds); a single TF32 product would be ~1e-3.
    ref32 = A.float().double() @ B.float().double().T
    err = ((C - ref32).norm() / ref32.norm()).item()
    assert err < 1e-5, err
    assert ((C - ref).norm() / ref.norm()).item() < 1e-5
