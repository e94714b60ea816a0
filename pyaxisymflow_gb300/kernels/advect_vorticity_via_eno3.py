"""Drop-in for pyaxisymflow/kernels/advect_vorticity_via_eno3.py:8-91.

The reference mirrors vorticity (odd), u_z (even) and u_r (odd) into
(2 nr, nz) float64 buffers, runs the pystencils ENO3 step and copies the upper
half back. The CUDA kernel reads the mirror by index reflection instead, so the
closure owns one (nr, nz) scratch field (the pre-step copy of vorticity).
"""
import numpy as np
import torch

from .. import _native as N
from .periodic_boundary_ghost_comm import native_ghost_size


class _Scratch:
    def __init__(self, nr, nz, count):
        self.shape = (count * nr, nz)
        self.buf = None

    def get(self, like):
        if (self.buf is None or self.buf.dtype != like.dtype or self.buf.device != like.device):
            self.buf = torch.empty(self.shape, dtype=like.dtype, device=like.device)
        return self.buf


def gen_advect_vorticity_via_eno3(dx, grid_size_r, grid_size_z, real_t=np.float64,
                                  num_threads=False):
    """Returns advect_vorticity_via_eno3(vorticity, u_z, u_r, dt): one
    conservative ENO3 Euler-forward step of vorticity, in place."""
    nr, nz = grid_size_r, grid_size_z
    scratch = _Scratch(nr, nz, 1)

    def advect_vorticity_via_eno3(vorticity, u_z, u_r, dt):
        s = N.require(vorticity, u_z, u_r, shape=(nr, nz), names=("vorticity", "u_z", "u_r"))
        N.call(f"axi_advect_vorticity_eno3_{s}", N.ptr(vorticity), N.ptr(u_z), N.ptr(u_r),
               N.ptr(scratch.get(vorticity)), nr, nz, N.real(s, dt / dx),
               N.stream_of(vorticity))

    return advect_vorticity_via_eno3


def gen_advect_vorticity_via_eno3_periodic(dx, grid_size_r, grid_size_z, per_communicator,
                                           real_t=np.float64, num_threads=False):
    """Periodic-z variant: exchanges the ghosts of u_z, u_r and vorticity first."""
    nr, nz = grid_size_r, grid_size_z
    scratch = _Scratch(nr, nz, 1)
    g = native_ghost_size(per_communicator)
    if g is None:
        raise TypeError("gen_advect_vorticity_via_eno3_periodic needs a communicator from "
                        "gen_periodic_boundary_ghost_comm")

    def advect_vorticity_via_eno3_periodic(vorticity, u_z, u_r, dt):
        s = N.require(vorticity, u_z, u_r, shape=(nr, nz), names=("vorticity", "u_z", "u_r"))
        N.call(f"axi_advect_vorticity_eno3_periodic_{s}", N.ptr(vorticity), N.ptr(u_z),
               N.ptr(u_r), N.ptr(scratch.get(vorticity)), nr, nz, N.real(s, dt / dx), g,
               N.stream_of(vorticity))

    return advect_vorticity_via_eno3_periodic
