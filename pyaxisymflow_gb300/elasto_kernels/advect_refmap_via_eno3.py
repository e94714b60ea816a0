"""Drop-in for pyaxisymflow/elasto_kernels/advect_refmap_via_eno3.py:8-115.

Non-conservative ENO3 step of the reference map: eta1 mirrored even, eta2
odd, velocity u_z even, u_r odd (index reflection, no doubled buffers)."""
import numpy as np

from .. import _native as N
from ..kernels.advect_vorticity_via_eno3 import _Scratch
from ..kernels.periodic_boundary_ghost_comm import _PeriodicGhostComm, native_ghost_size


def gen_advect_refmap_via_eno3(dx, grid_size_r, grid_size_z, real_t=np.float64,
                               num_threads=False):
    """Returns advect_refmap_via_eno3(eta1, eta2, u_z, u_r, dt), in place."""
    nr, nz = grid_size_r, grid_size_z
    scratch = _Scratch(nr, nz, 2)

    def advect_refmap_via_eno3(eta1, eta2, u_z, u_r, dt):
        s = N.require(eta1, eta2, u_z, u_r, shape=(nr, nz), names=("eta1", "eta2", "u_z", "u_r"))
        N.call(f"axi_advect_refmap_eno3_{s}", N.ptr(eta1), N.ptr(eta2), N.ptr(u_z), N.ptr(u_r),
               N.ptr(scratch.get(eta1)), nr, nz, N.real(s, dt / dx), N.stream_of(eta1))

    return advect_refmap_via_eno3


def gen_advect_refmap_via_eno3_periodic(dx, grid_size_r, grid_size_z, per_communicator1,
                                        per_communicator2, real_t=np.float64,
                                        num_threads=False):
    """Periodic-z variant: per_communicator1 (plain) exchanges u_z, u_r, eta2;
    per_communicator2 (eta-shifted) exchanges eta1."""
    nr, nz = grid_size_r, grid_size_z
    scratch = _Scratch(nr, nz, 2)
    g = native_ghost_size(per_communicator1)
    if (g is None or not isinstance(per_communicator2, _PeriodicGhostComm)
            or per_communicator2.eta_shift is None or per_communicator2.ghost_size != g):
        raise TypeError("gen_advect_refmap_via_eno3_periodic needs communicators from "
                        "gen_periodic_boundary_ghost_comm(_eta) with one ghost size")
    z_max, cdx = per_communicator2.eta_shift

    def advect_refmap_via_eno3_periodic(eta1, eta2, u_z, u_r, dt):
        s = N.require(eta1, eta2, u_z, u_r, shape=(nr, nz), names=("eta1", "eta2", "u_z", "u_r"))
        N.call(f"axi_advect_refmap_eno3_periodic_{s}", N.ptr(eta1), N.ptr(eta2), N.ptr(u_z),
               N.ptr(u_r), N.ptr(scratch.get(eta1)), nr, nz, N.real(s, dt / dx), g,
               N.real(s, z_max), N.real(s, cdx), N.stream_of(eta1))

    return advect_refmap_via_eno3_periodic
