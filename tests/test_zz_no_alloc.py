"""The allocation-free spectral transform against the scratch-taking one.

axi_fd_transform_static_f64 serves callers that may not call cudaMalloc (a
host whose device memory is owned by another allocator): its intermediate
products live in a fixed device array inside the library. Both entry points are called through the C ABI on
the same operands; the results must agree to the spectral-solve tolerance of
the other GPU tests, on two calls in a row (the second call reuses the array
the first one left behind). Named so that pytest collects it last.
"""
import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu

SOLVE_RTOL = 1e-12


def rel_l2(a, b):
    return float(torch.linalg.norm(a - b) / torch.linalg.norm(b))


def test_static_scratch_transform_matches_scratch_taking_transform():
    from pyaxisymflow_gb300 import _native as N
    from pyaxisymflow_gb300.kernels.FastDiagonalisationStokesSolver import \
        FastDiagonalisationStokesSolver
    lib = N.lib()
    assert lib.axi_fd_transform_static_max_cells() >= 512 * 1024
    nr, nz = 256, 512
    solver = FastDiagonalisationStokesSolver(nr, nz, 1.0 / nz, device="cuda")
    d = solver.engine.dev
    stream = torch.cuda.current_stream()
    s = N._c.c_void_p(stream.cuda_stream)
    work = torch.empty(2 * nr * nz, dtype=torch.float64, device="cuda")
    g = torch.Generator(device="cpu").manual_seed(5)
    for call in range(2):
        rhs = torch.randn((nr, nz), generator=g, dtype=torch.float64).cuda()
        ref = torch.empty_like(rhs)
        out = torch.full_like(rhs, float("nan"))
        N.check(lib.axi_fd_transform_f64(N.ptr(ref), nz, N.ptr(rhs), nz, N.ptr(d["Er_inv_w"]),
                                         N.ptr(d["EzinvT"]), N.ptr(d["inv_eig"]), N.ptr(d["Er"]),
                                         N.ptr(d["EzT"]), N.ptr(work), nr, nz, s))
        torch.cuda.synchronize()
        free_before = torch.cuda.mem_get_info()[0]
        N.check(lib.axi_fd_transform_static_f64(N.ptr(out), nz, N.ptr(rhs), nz,
                                                N.ptr(d["Er_inv_w"]), N.ptr(d["EzinvT"]),
                                                N.ptr(d["inv_eig"]), N.ptr(d["Er"]),
                                                N.ptr(d["EzT"]), nr, nz, s))
        torch.cuda.synchronize()
        if call == 1:
            # the second call (the module is loaded by the first): no device
            # memory taken or given back
            assert torch.cuda.mem_get_info()[0] == free_before
        assert torch.isfinite(out).all()
        assert rel_l2(out, ref) < SOLVE_RTOL, (call, rel_l2(out, ref))


def test_static_scratch_transform_rejects_oversize_grids():
    from pyaxisymflow_gb300 import _native as N
    lib = N.lib()
    big = lib.axi_fd_transform_static_max_cells() + 1
    dummy = torch.zeros(8, dtype=torch.float64, device="cuda")
    p = N.ptr(dummy)
    st = lib.axi_fd_transform_static_f64(p, big, p, big, p, p, p, p, p, 1, big,
                                         N._c.c_void_p(torch.cuda.current_stream().cuda_stream))
    assert st == N.AXI_ERR_INVALID
    assert b"static scratch" in lib.axi_last_error()
