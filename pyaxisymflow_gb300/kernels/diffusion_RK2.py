"""Drop-in for pyaxisymflow/kernels/diffusion_RK2.py:4-89."""
from .. import _native as N
from .periodic_boundary_ghost_comm import native_ghost_size


def diffusion_RK2_unb(vorticity, temp_vorticity, R, nu, dt, dx):
    """update field due to diffusion using a RK2 time stepper"""
    s = N.require(vorticity, temp_vorticity, R, shape=vorticity.shape,
                  names=("vorticity", "temp_vorticity", "R"))
    nr, nz = vorticity.shape
    N.call(f"axi_diffusion_rk2_unb_{s}", N.ptr(vorticity), N.ptr(temp_vorticity), N.ptr(R), nr,
           nz, N.real(s, nu), N.real(s, dt), N.real(s, dx), N.stream_of(vorticity))


def diffusion_RK2_periodic(vorticity, temp_vorticity, R, nu, dt, dx, per_communicator):
    """update field due to diffusion using a RK2 time stepper, with periodic
    ghost exchange of vorticity and of the intermediate stage"""
    s = N.require(vorticity, temp_vorticity, R, shape=vorticity.shape,
                  names=("vorticity", "temp_vorticity", "R"))
    nr, nz = vorticity.shape
    g = native_ghost_size(per_communicator)
    if g is None:
        raise TypeError("diffusion_RK2_periodic needs a communicator from "
                        "gen_periodic_boundary_ghost_comm")
    N.call(f"axi_diffusion_rk2_periodic_{s}", N.ptr(vorticity), N.ptr(temp_vorticity), N.ptr(R),
           nr, nz, N.real(s, nu), N.real(s, dt), N.real(s, dx), g, N.stream_of(vorticity))
