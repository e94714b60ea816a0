"""Drop-in for the compiled module pyaxisymflow.core.particles_to_mesh, the
2-D MP4 functions the reference calls (kernels/advect_particle.py:30, 63;
core/src/particles_to_mesh_bind.cpp): particle values interpolated onto the
cell-centred mesh, bit-identical to the reference's sequential sum.

Particle (j, i) must lie less than one cell from mesh point (j, i) along each
axis (the remeshing step resets the particles to the mesh every step);
otherwise ValueError is raised (check=True, which synchronises) because the
gather that makes the sum deterministic would miss contributions.
"""
import torch

from .. import _native as N

_work = {}


def _scratch(n0, n1, device):
    key = (n0, n1, device)
    if key not in _work:
        _work[key] = torch.empty(int(N.lib().axi_p2m_mp4_work_bytes(n0, n1)), dtype=torch.uint8,
                                 device=device)
    return _work[key]


def _p2m(px, py, vin, out, delta_x, delta_y, periodic, check):
    N.require(px, py, vin, out, shape=out.shape, dtype=torch.float64,
              names=("particle_positions_x", "particle_positions_y",
                     "input_field_at_particle_positions", "output_field_at_mesh"))
    n0, n1 = out.shape
    work = _scratch(n0, n1, out.device)
    N.call("axi_particles_to_mesh_2d_mp4_f64", N.ptr(px), N.ptr(py), N.ptr(vin), N.ptr(out), n0,
           n1, float(delta_x), float(delta_y), int(periodic), N.ptr(work), N.stream_of(out))
    if check:
        flag = N._c.c_int(0)
        N.call("axi_p2m_status", N.ptr(work), n0, n1, N._c.byref(flag), N.stream_of(out))
        if flag.value:
            raise ValueError("particles_to_mesh: a particle moved a cell or more from its mesh "
                             "point (|u| dt must stay below dx along each axis)")


def particles_to_mesh_2D_mp4(particle_positions_x, particle_positions_y,
                             input_field_at_particle_positions, output_field_at_mesh, delta_x,
                             delta_y, check=True):
    """Periodic in both directions (core/src/particles_to_mesh.hpp:69-91)."""
    _p2m(particle_positions_x, particle_positions_y, input_field_at_particle_positions,
         output_field_at_mesh, delta_x, delta_y, True, check)


def particles_to_mesh_2D_unbounded_mp4(particle_positions_x, particle_positions_y,
                                       input_field_at_particle_positions, output_field_at_mesh,
                                       delta_x, delta_y, check=True):
    """Unbounded: stencil points off the mesh are dropped
    (core/src/particles_to_mesh.hpp:163-184)."""
    _p2m(particle_positions_x, particle_positions_y, input_field_at_particle_positions,
         output_field_at_mesh, delta_x, delta_y, False, check)
