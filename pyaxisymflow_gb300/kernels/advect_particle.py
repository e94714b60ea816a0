"""Vorticity advection by remeshed particles (kernels/advect_particle.py:5-68)
on the GPU: particles on the axis-mirrored (2 nr, nz) domain move by u dt,
their vorticity is interpolated back onto the mesh with the MP4 kernel, and
the particles are reset to the mesh. Same arguments and in-place semantics
as the reference; float64 CUDA tensors."""
import torch

from .. import _native as N
from ..core.particles_to_mesh import particles_to_mesh_2D_mp4, particles_to_mesh_2D_unbounded_mp4


def _advect(z_particles, r_particles, vort_particles, vorticity, Z_double, R_double, grid_size_r,
            u_z, u_r, dx, dt, p2m):
    nr = int(grid_size_r)
    nz = vorticity.shape[1]
    N.require(z_particles, r_particles, vort_particles, Z_double, R_double, shape=(2 * nr, nz),
              dtype=torch.float64,
              names=("z_particles", "r_particles", "vort_particles", "Z_double", "R_double"))
    N.require(vorticity, u_z, u_r, shape=(nr, nz), dtype=torch.float64,
              names=("vorticity", "u_z", "u_r"))
    N.call("axi_advect_particles_prepare_f64", N.ptr(z_particles), N.ptr(r_particles),
           N.ptr(vort_particles), N.ptr(vorticity), N.ptr(u_z), N.ptr(u_r), nr, nz, float(dt),
           N.stream_of(vorticity))
    vort_double = torch.empty_like(Z_double)
    p2m(z_particles, r_particles, vort_particles, vort_double, dx, dx)
    z_particles.copy_(Z_double)
    r_particles.copy_(R_double)
    vorticity.copy_(vort_double[nr:, :])


def advect_vorticity_via_particles(z_particles, r_particles, vort_particles, vorticity, Z_double,
                                   R_double, grid_size_r, u_z, u_r, dx, dt):
    """kernels/advect_particle.py:5-35 (unbounded remeshing)."""
    _advect(z_particles, r_particles, vort_particles, vorticity, Z_double, R_double, grid_size_r,
            u_z, u_r, dx, dt, particles_to_mesh_2D_unbounded_mp4)


def advect_vorticity_via_particles_periodic(z_particles, r_particles, vort_particles, vorticity,
                                            Z_double, R_double, grid_size_r, u_z, u_r, dx, dt):
    """kernels/advect_particle.py:38-68 (periodic remeshing)."""
    _advect(z_particles, r_particles, vort_particles, vorticity, Z_double, R_double, grid_size_r,
            u_z, u_r, dx, dt, particles_to_mesh_2D_mp4)
