"""Drop-in for pyaxisymflow/elasto_kernels/extrapolate_eta_using_least_squares_unb.py:7-30."""
import torch

from .. import _native as N
from ..core.extrapolate_using_least_squares import MAX_SWEEPS


def extrapolate_eta_with_least_squares(inside_solid, ball_phi, eta1, eta2, ball_phi_double,
                                       eta1_double, eta2_double, extrap_zone, grid_size_r, z):
    """Mirror phi and the masked reference map about the axis into the
    (2 nr, nz) buffers, extrapolate eta into phi < extrap_zone, copy back."""
    nr = int(grid_size_r)
    N.require(ball_phi, eta1, eta2, shape=ball_phi.shape, dtype=torch.float64,
              names=("ball_phi", "eta1", "eta2"))
    nz = ball_phi.shape[1]
    N.require(ball_phi_double, eta1_double, eta2_double, shape=(2 * nr, nz),
              dtype=torch.float64, names=("ball_phi_double", "eta1_double", "eta2_double"))
    N.require(z, dtype=torch.float64, names=("z",))
    if z.numel() < max(2 * nr, nz):
        raise ValueError("z must hold at least max(2 * grid_size_r, nz) coordinates")
    inside = inside_solid.to(torch.uint8).contiguous()
    N.require(inside, shape=ball_phi.shape, dtype=torch.uint8, names=("inside_solid",))
    dev = ball_phi.device
    flags = torch.empty((2, 2 * nr, nz), dtype=torch.int16, device=dev)
    work = torch.empty(N.lib().axi_lsq_work_bytes(2 * nr, nz), dtype=torch.uint8, device=dev)
    sweeps = N._c.c_int(0)
    N.call("axi_extrapolate_eta_with_least_squares_f64", N.ptr(inside), N.ptr(ball_phi),
           N.ptr(eta1), N.ptr(eta2), N.ptr(ball_phi_double), N.ptr(eta1_double),
           N.ptr(eta2_double), N.ptr(flags[0]), N.ptr(flags[1]), float(extrap_zone), nr, nz,
           N.ptr(z), N.ptr(z), MAX_SWEEPS, N.ptr(work), N._c.byref(sweeps), N.stream_of(eta1))
