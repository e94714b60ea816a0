"""Drop-in for pyaxisymflow/kernels/compute_velocity_from_psi.py:4-34."""
from .. import _native as N
from .periodic_boundary_ghost_comm import native_ghost_size


def compute_velocity_from_psi_unb(u_z, u_r, psi, R, dx):
    """computes velocity from the Stokes stream function
    (u_z = d_psi/dr / r, u_r = -d_psi/dz / r)."""
    s = N.require(u_z, u_r, psi, R, shape=psi.shape, names=("u_z", "u_r", "psi", "R"))
    nr, nz = psi.shape
    N.call(f"axi_velocity_from_psi_unb_{s}", N.ptr(u_z), N.ptr(u_r), N.ptr(psi), N.ptr(R), nr, nz,
           N.real(s, dx), N.stream_of(psi))


def compute_velocity_from_psi_periodic(u_z, u_r, psi, R, dx, per_communicator):
    """computes velocity from the Stokes stream function; psi ghosts are
    exchanged first with per_communicator."""
    s = N.require(u_z, u_r, psi, R, shape=psi.shape, names=("u_z", "u_r", "psi", "R"))
    nr, nz = psi.shape
    g = native_ghost_size(per_communicator)
    if g is None:
        per_communicator(psi)
        compute_velocity_from_psi_unb(u_z, u_r, psi, R, dx)
        return
    N.call(f"axi_velocity_from_psi_periodic_{s}", N.ptr(u_z), N.ptr(u_r), N.ptr(psi), N.ptr(R),
           nr, nz, N.real(s, dx), g, N.stream_of(psi))
