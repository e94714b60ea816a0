"""Drop-in for pyaxisymflow/kernels/kill_boundary_vorticity_sine.py:4-27.

The reference's literal ``1 - Z`` and ``1 - R`` (a unit domain length) are
kept, so results match it on any domain."""
from .. import _native as N


def kill_boundary_vorticity_sine_z(vorticity, Z, width, dx):
    """kills vorticity on the boundaries in a sine wave fashion
    in the given width in Z direction"""
    s = N.require(vorticity, Z, shape=vorticity.shape, names=("vorticity", "Z"))
    nr, nz = vorticity.shape
    N.call(f"axi_kill_boundary_vorticity_sine_z_{s}", N.ptr(vorticity), N.ptr(Z), nr, nz,
           int(width), N.real(s, dx), N.stream_of(vorticity))


def kill_boundary_vorticity_sine_r(vorticity, R, width, dx):
    """kills vorticity on the boundaries in a sine wave fashion in the given
    width in R direction (only on maxR); on axis, set vorticity = 0"""
    s = N.require(vorticity, R, shape=vorticity.shape, names=("vorticity", "R"))
    nr, nz = vorticity.shape
    N.call(f"axi_kill_boundary_vorticity_sine_r_{s}", N.ptr(vorticity), N.ptr(R), nr, nz,
           int(width), N.real(s, dx), N.stream_of(vorticity))
