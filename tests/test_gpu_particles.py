"""Particle remeshing on the GPU (MP4 particle-to-mesh, vorticity advection by
remeshed particles) against the reference's outputs and the oracle: bit-exact."""
import numpy as np
import pytest
import torch

from oracle import kernels as K

pytestmark = pytest.mark.gpu


def cuda(a):
    return torch.tensor(np.ascontiguousarray(a), dtype=torch.float64, device="cuda")


@pytest.mark.parametrize("tag", ["a", "b"])
def test_particles_to_mesh_matches_reference(golden, tag):
    from pyaxisymflow_gb300.core import particles_to_mesh as p2m
    g = golden("p2m")
    px, py, v, dx = cuda(g[f"{tag}/px"]), cuda(g[f"{tag}/py"]), cuda(g[f"{tag}/v"]), float(
        g[f"{tag}/dx"])
    for name, fn in (("periodic", p2m.particles_to_mesh_2D_mp4),
                     ("unbounded", p2m.particles_to_mesh_2D_unbounded_mp4)):
        out = torch.empty_like(v)
        fn(px, py, v, out, dx, dx)
        np.testing.assert_array_equal(out.cpu().numpy(), g[f"{tag}/{name}"])


def test_particles_far_from_their_mesh_point_are_rejected(golden):
    from pyaxisymflow_gb300.core import particles_to_mesh as p2m
    g = golden("p2m")
    px, py, v = cuda(g["c/px"]), cuda(g["c/py"]), cuda(g["c/v"])
    with pytest.raises(ValueError, match="cell or more"):
        p2m.particles_to_mesh_2D_unbounded_mp4(px, py, v, torch.empty_like(v), float(g["c/dx"]),
                                               float(g["c/dx"]))


def test_advect_vorticity_via_particles_matches_reference(golden):
    from pyaxisymflow_gb300.kernels import advect_particle as ap
    g = golden("p2m")
    nr, dx, dt = int(g["adv/nr"]), float(g["adv/dx"]), float(g["adv/dt"])
    nz = g["adv/w0"].shape[1]
    Zd, Rd = np.meshgrid((np.arange(nz) + 0.5) * dx, (np.arange(2 * nr) + 0.5) * dx)
    for name, fn in (("unbounded", ap.advect_vorticity_via_particles),
                     ("periodic", ap.advect_vorticity_via_particles_periodic)):
        w = cuda(g["adv/w0"])
        zp, rp, vp = cuda(Zd), cuda(Rd), torch.zeros_like(cuda(Zd))
        Zt, Rt = cuda(Zd), cuda(Rd)
        for _ in range(2):
            fn(zp, rp, vp, w, Zt, Rt, nr, cuda(g["adv/u_z"]), cuda(g["adv/u_r"]), dx, dt)
        np.testing.assert_array_equal(w.cpu().numpy(), g[f"adv/{name}"])
        assert torch.equal(zp, Zt) and torch.equal(rp, Rt)


@pytest.mark.parametrize("nr,nz", [(128, 256), (96, 200)])
def test_advect_vorticity_via_particles_matches_oracle_larger(nr, nz):
    from pyaxisymflow_gb300.kernels import advect_particle as ap
    rng = np.random.default_rng(nr + nz)
    dx = 1.0 / nz
    Zd, Rd = np.meshgrid((np.arange(nz) + 0.5) * dx, (np.arange(2 * nr) + 0.5) * dx)
    w0 = rng.standard_normal((nr, nz))
    uz, ur = rng.uniform(-2, 2, (nr, nz)), rng.uniform(-2, 2, (nr, nz))
    dt = 0.45 * dx / 2
    for ref_fn, fn in ((K.advect_vorticity_via_particles, ap.advect_vorticity_via_particles),
                       (K.advect_vorticity_via_particles_periodic,
                        ap.advect_vorticity_via_particles_periodic)):
        w_ref = w0.copy()
        zp, rp, vp = Zd.copy(), Rd.copy(), np.zeros_like(Zd)
        w = cuda(w0)
        zt, rt, vt, Zt, Rt = cuda(Zd), cuda(Rd), torch.zeros_like(cuda(Zd)), cuda(Zd), cuda(Rd)
        ut, vr = cuda(uz), cuda(ur)
        for _ in range(3):
            ref_fn(zp, rp, vp, w_ref, Zd, Rd, nr, uz, ur, dx, dt)
            fn(zt, rt, vt, w, Zt, Rt, nr, ut, vr, dx, dt)
        np.testing.assert_array_equal(w.cpu().numpy(), w_ref)


@pytest.mark.parametrize("tag", ["a", "b", "c"])
def test_mesh_to_particles_matches_reference_golden(golden, tag):
    """Mesh-to-particle MP4 (periodic and unbounded) on the device against
    the reference's C++ results, bit for bit: particles in and around the
    mesh, particle arrays shaped differently from the mesh."""
    from pyaxisymflow_gb300.core.mesh_to_particles import (mesh_to_particles_2D_mp4,
                                                           mesh_to_particles_2D_unbounded_mp4)
    g = golden("m2p")
    fx, fy, px, py = (torch.tensor(g[f"{tag}/{k}"], device="cuda")
                      for k in ("fx", "fy", "px", "py"))
    dx = float(g[f"{tag}/dx"])
    for name, fn in (("periodic", mesh_to_particles_2D_mp4),
                     ("unbounded", mesh_to_particles_2D_unbounded_mp4)):
        ox, oy = torch.zeros_like(px), torch.zeros_like(px)
        fn(fx, fy, px, py, ox, oy, dx, dx)
        assert np.array_equal(ox.cpu().numpy(), g[f"{tag}/{name}_x"]), name
        assert np.array_equal(oy.cpu().numpy(), g[f"{tag}/{name}_y"]), name


def test_mesh_to_particles_matches_oracle_at_size():
    from oracle import kernels as K
    from pyaxisymflow_gb300.core.mesh_to_particles import mesh_to_particles_2D_unbounded_mp4
    rng = np.random.default_rng(21)
    n0, n1, dx = 256, 384, 1.0 / 256
    fx, fy = rng.standard_normal((n0, n1)), rng.standard_normal((n0, n1))
    px = rng.uniform(-1, n1 + 1, (300, 200)) * dx
    py = rng.uniform(-1, n0 + 1, (300, 200)) * dx
    ox, oy = np.zeros(px.shape), np.zeros(px.shape)
    K.mesh_to_particles_2D_unbounded_mp4(fx, fy, px, py, ox, oy, dx, dx)
    t = [torch.tensor(a, device="cuda") for a in (fx, fy, px, py)]
    gx, gy = torch.zeros_like(t[2]), torch.zeros_like(t[2])
    mesh_to_particles_2D_unbounded_mp4(*t, gx, gy, dx, dx)
    assert np.array_equal(gx.cpu().numpy(), ox) and np.array_equal(gy.cpu().numpy(), oy)
