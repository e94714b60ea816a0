"""FP32 spectral solves on the tcgen05 tensor cores (3xTF32) with one step of
iterative refinement (FP64 residual), against the FP64 oracle.

The isolated Poisson configuration: periodic z, Neumann r, a seeded
sum of 32 axisymmetric Gaussian vortex rings as right-hand side; errors of psi
and of the velocity derived from it are relative L2 against FP64.
"""
import numpy as np
import pytest
import torch

from oracle import kernels as K

pytestmark = pytest.mark.gpu


def rel_l2(a, b):
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


def vortex_rings(nr, nz, dx, seed=3, n=32):
    rng = np.random.default_rng(seed)
    z = (np.arange(nz) + 0.5) * dx
    r = (np.arange(nr) + 0.5) * dx
    Z, R = np.meshgrid(z, r)
    Lz, Lr = nz * dx, nr * dx
    w = np.zeros((nr, nz))
    for _ in range(n):
        zc, rc = rng.uniform(0, Lz), rng.uniform(0.1, 0.9) * Lr
        rad, s = rng.uniform(0.02, 0.2), rng.standard_normal()
        w += s * np.exp(-((Z - zc) ** 2 + (R - rc) ** 2) / rad ** 2)
    return w, Z, R


@pytest.mark.parametrize("bc,nr,nz", [(K.NEUMANN_ZR, 128, 256), (K.NEUMANN_R_PERIODIC_Z, 256, 512),
                                      (K.NEUMANN_R_PERIODIC_Z, 512, 1024)])
def test_tensor_core_stokes_solve_with_refinement(bc, nr, nz):
    from pyaxisymflow_gb300.kernels.FastDiagonalisationStokesSolver import \
        FastDiagonalisationStokesSolver
    dx = 1.0 / nr
    w, Z, R = vortex_rings(nr, nz, dx)
    ref = np.zeros_like(w)
    K.FastDiagonalisationStokesSolver(nr, nz, dx, bc_type=bc).solve(ref, w)
    uz_ref, ur_ref = np.zeros_like(w), np.zeros_like(w)
    K.compute_velocity_from_psi_unb(uz_ref, ur_ref, ref, R, dx)
    tw = torch.tensor(w, dtype=torch.float64, device="cuda")
    errs = {}
    for refine in (0, 1):
        s = FastDiagonalisationStokesSolver(nr, nz, dx, real_dtype=np.float32, bc_type=bc,
                                            refine=refine)
        psi = torch.zeros_like(tw)
        s.solve(psi, tw)
        torch.cuda.synchronize()
        assert s.engine.tc_status() == 0
        p = psi.cpu().numpy()
        uz, ur = np.zeros_like(w), np.zeros_like(w)
        K.compute_velocity_from_psi_unb(uz, ur, p, R, dx)
        errs[refine] = (rel_l2(p, ref), rel_l2(uz, uz_ref), rel_l2(ur, ur_ref))
    print(bc, nr, nz, "rel L2 (psi, u_z, u_r) without / with refinement:", errs)
    # One FP64-residual refinement step squares the relative error of the
    # 3xTF32 transform (~1e-5 on velocity at these sizes).
    assert max(errs[0]) < 2e-4, errs
    assert max(errs[1]) < 1e-8, errs


def test_tensor_core_solve_float32_fields_and_potential():
    from pyaxisymflow_gb300.kernels.FastDiagonalisationStokesSolver import \
        FastDiagonalisationStokesSolver
    from pyaxisymflow_gb300.kernels.implicit_diffusion_solver import \
        ImplicitEulerDiffusionStepper
    nr, nz = 128, 256
    dx = 1.0 / nz
    w, _, _ = vortex_rings(nr, nz, dx, seed=9, n=8)
    ref = np.zeros_like(w)
    K.FastDiagonalisationStokesSolver(nr, nz, dx).solve(ref, w)
    s = FastDiagonalisationStokesSolver(nr, nz, dx, real_dtype=np.float32)
    t32 = torch.tensor(w, dtype=torch.float32, device="cuda")
    psi32 = torch.zeros_like(t32)
    s.solve(psi32, t32)
    ref32 = np.zeros_like(w)
    K.FastDiagonalisationStokesSolver(nr, nz, dx).solve(ref32, w.astype(np.float32).astype(np.float64))
    assert rel_l2(psi32.double().cpu().numpy(), ref32) < 5e-7
    dt = 0.5 * dx * dx / 1e-2
    st = ImplicitEulerDiffusionStepper(dt, 1e-2, nr, nz, dx, real_dtype=np.float32)
    x = torch.tensor(w, dtype=torch.float64, device="cuda")
    st.step(x, dt)
    refd = w.copy()
    K.ImplicitEulerDiffusionStepper(dt, 1e-2, nr, nz, dx).step(refd, dt)
    assert rel_l2(x.cpu().numpy(), refd) < 1e-8
