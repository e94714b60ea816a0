"""Drop-in for the compiled module pyaxisymflow.core.extrapolate_using_least_squares
(core/src/extrapolate_using_least_squares_bind.cpp:88-91, first order)."""
import torch

from .. import _native as N

# Front marching converges in about extrap_zone / dx sweeps; the cap only
# guards against inputs on which the reference itself would loop forever.
MAX_SWEEPS = 100000


def extrapolate_using_least_squares_till_first_order(current_flag, target_flag, eta_x, eta_y,
                                                     grid_x, grid_y, max_sweeps=MAX_SWEEPS):
    """Extrapolate eta_x, eta_y from cells with current_flag == 1 into cells
    with target_flag == 1, in place (current_flag is updated). int16 flags and
    float64 fields, like the reference binding's noconvert arguments.
    Synchronises the stream; returns the number of sweeps."""
    N.require(current_flag, target_flag, shape=current_flag.shape, dtype=torch.int16,
              names=("current_flag", "target_flag"))
    N.require(eta_x, eta_y, shape=current_flag.shape, dtype=torch.float64,
              names=("eta_x", "eta_y"))
    N.require(grid_x, grid_y, dtype=torch.float64, names=("grid_x", "grid_y"))
    n0, n1 = current_flag.shape
    if grid_x.numel() < n1 or grid_y.numel() < n0:
        raise ValueError("grid_x / grid_y shorter than the flag array")
    work = torch.empty(N.lib().axi_lsq_work_bytes(n0, n1), dtype=torch.uint8,
                       device=current_flag.device)
    sweeps = N._c.c_int(0)
    N.call("axi_extrapolate_lsq_first_order_f64", N.ptr(current_flag), N.ptr(target_flag),
           N.ptr(eta_x), N.ptr(eta_y), N.ptr(grid_x), N.ptr(grid_y), n0, n1, int(max_sweeps),
           N.ptr(work), N._c.byref(sweeps), N.stream_of(eta_x))
    return sweeps.value
