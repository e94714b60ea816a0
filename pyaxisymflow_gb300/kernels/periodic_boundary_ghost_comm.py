"""Drop-in for pyaxisymflow/kernels/periodic_boundary_ghost_comm.py:4-33."""
from .. import _native as N


class _PeriodicGhostComm:
    """Callable exchanging `ghost_size` periodic z-ghost columns in place."""

    def __init__(self, ghost_size, eta_shift=None):
        self.ghost_size = ghost_size
        self.eta_shift = eta_shift  # (Z_max, dx) for the reference-map variant

    def __call__(self, field):
        s = N.require(field, names=("field",))
        nr, nz = field.shape
        if self.eta_shift is None:
            N.call(f"axi_periodic_ghost_comm_{s}", N.ptr(field), nr, nz, self.ghost_size,
                   N.stream_of(field))
        else:
            z_max, dx = self.eta_shift
            N.call(f"axi_periodic_ghost_comm_eta_{s}", N.ptr(field), nr, nz, self.ghost_size,
                   N.real(s, z_max), N.real(s, dx), N.stream_of(field))


def gen_periodic_boundary_ghost_comm(ghost_size):
    """Generates kernel that will communicate the ghosts at the periodic boundary."""
    assert ghost_size > 0 and isinstance(ghost_size, int), "invalid ghost size"
    return _PeriodicGhostComm(ghost_size)


def gen_periodic_boundary_ghost_comm_eta(ghost_size, Z_max, dx):
    """Generates kernel that will communicate the ghosts at the periodic
    boundary, shifting the reference map by the period."""
    assert ghost_size > 0 and isinstance(ghost_size, int), "invalid ghost size"
    return _PeriodicGhostComm(ghost_size, eta_shift=(Z_max, dx))


def native_ghost_size(per_communicator):
    """Ghost width of a plain communicator made here, else None (then the
    caller invokes the user's communicator itself)."""
    if isinstance(per_communicator, _PeriodicGhostComm) and per_communicator.eta_shift is None:
        return per_communicator.ghost_size
    return None
