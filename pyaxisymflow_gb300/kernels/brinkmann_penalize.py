"""Drop-in for pyaxisymflow/kernels/brinkmann_penalize.py:4-16."""
from .. import _native as N


def brinkmann_penalize(lam, dt, char_func, U_z, U_r, grid_u_z, grid_u_r, penalized_u_z,
                       penalized_u_r):
    """implicit Brinkmann penalization for velocity:
    penalized = (grid_u + lam dt chi U) / (1 + lam dt chi), in place."""
    s = N.require(char_func, grid_u_z, grid_u_r, penalized_u_z, penalized_u_r,
                  shape=char_func.shape,
                  names=("char_func", "grid_u_z", "grid_u_r", "penalized_u_z", "penalized_u_r"))
    N.call(f"axi_brinkmann_penalize_{s}", N.real(s, lam), N.real(s, dt), N.ptr(char_func),
           N.real(s, U_z), N.real(s, U_r), N.ptr(grid_u_z), N.ptr(grid_u_r),
           N.ptr(penalized_u_z), N.ptr(penalized_u_r), char_func.numel(), N.stream_of(char_func))
