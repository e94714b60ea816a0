"""Drop-in for pyaxisymflow/kernels/compute_vorticity_from_velocity.py:4-28."""
from .. import _native as N
from .periodic_boundary_ghost_comm import native_ghost_size


def compute_vorticity_from_velocity_unb(vort, u_z, u_r, dx):
    """compute vorticity from velocity field on the interior [1:-1, 1:-1]
    (boundaries untouched)."""
    s = N.require(vort, u_z, u_r, shape=vort.shape, names=("vort", "u_z", "u_r"))
    nr, nz = vort.shape
    N.call(f"axi_vorticity_from_velocity_unb_{s}", N.ptr(vort), N.ptr(u_z), N.ptr(u_r), nr, nz,
           N.real(s, dx), N.stream_of(vort))


def compute_vorticity_from_velocity_periodic(vort, u_z, u_r, dx, per_communicator):
    """compute vorticity from velocity field after exchanging the ghosts of
    u_r and u_z."""
    s = N.require(vort, u_z, u_r, shape=vort.shape, names=("vort", "u_z", "u_r"))
    nr, nz = vort.shape
    g = native_ghost_size(per_communicator)
    if g is None:
        per_communicator(u_r)
        per_communicator(u_z)
        compute_vorticity_from_velocity_unb(vort, u_z, u_r, dx)
        return
    N.call(f"axi_vorticity_from_velocity_periodic_{s}", N.ptr(vort), N.ptr(u_z), N.ptr(u_r), nr,
           nz, N.real(s, dx), g, N.stream_of(vort))
