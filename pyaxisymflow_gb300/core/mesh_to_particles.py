"""Drop-in for the 2-D MP4 functions of the compiled module
pyaxisymflow.core.mesh_to_particles (core/src/mesh_to_particles.hpp,
core/src/interpolation/mesh_to_particles_2D.hpp, bound by
core/src/mesh_to_particles_bind.cpp): two mesh fields interpolated at the
particle positions, one thread per particle, bit-identical to the
reference's sums. Arguments are float64 CUDA tensors; the particle arrays
may be shaped differently from the mesh.
"""
import torch

from .. import _native as N


def _m2p(input_field_x, input_field_y, particle_positions_x, particle_positions_y,
         output_field_x, output_field_y, delta_x, delta_y, periodic):
    N.require(input_field_x, input_field_y, shape=input_field_x.shape, dtype=torch.float64,
              names=("input_field_x", "input_field_y"))
    N.require(particle_positions_x, particle_positions_y, output_field_x, output_field_y,
              shape=particle_positions_x.shape, dtype=torch.float64,
              names=("particle_positions_x", "particle_positions_y", "output_field_x",
                     "output_field_y"))
    if input_field_x.dim() != 2 or particle_positions_x.dim() != 2:
        raise ValueError("mesh and particle arrays must be 2-D")
    n0, n1 = input_field_x.shape
    p0, p1 = particle_positions_x.shape
    N.call("axi_mesh_to_particles_2d_mp4_f64", N.ptr(input_field_x), N.ptr(input_field_y), n0,
           n1, N.ptr(particle_positions_x), N.ptr(particle_positions_y), N.ptr(output_field_x),
           N.ptr(output_field_y), p0, p1, float(delta_x), float(delta_y), int(periodic),
           N.stream_of(output_field_x))


def mesh_to_particles_2D_mp4(input_field_x, input_field_y, particle_positions_x,
                             particle_positions_y, output_field_x, output_field_y, delta_x,
                             delta_y):
    """MP4 mesh-to-particle interpolation in a 2-D periodic domain."""
    _m2p(input_field_x, input_field_y, particle_positions_x, particle_positions_y,
         output_field_x, output_field_y, delta_x, delta_y, True)


def mesh_to_particles_2D_unbounded_mp4(input_field_x, input_field_y, particle_positions_x,
                                       particle_positions_y, output_field_x, output_field_y,
                                       delta_x, delta_y):
    """MP4 mesh-to-particle interpolation in a 2-D unbounded domain (one-sided
    at the mesh edges)."""
    _m2p(input_field_x, input_field_y, particle_positions_x, particle_positions_y,
         output_field_x, output_field_y, delta_x, delta_y, False)
