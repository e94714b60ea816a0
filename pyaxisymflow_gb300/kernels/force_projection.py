"""Drop-in for pyaxisymflow/kernels/force_projection.py:5-15 (FP64 accumulation)."""
from .. import _native as N
from .compute_forces import _scratch


def force_projection(rho_s, char_func, u_z, u_r, R):
    """computes projected momentum on floating bodies from the fluid; returns
    (U_z, U_r) as Python floats (synchronises the stream)."""
    s = N.require(char_func, u_z, u_r, R, shape=R.shape, names=("char_func", "u_z", "u_r", "R"))
    buf = _scratch(R.device)
    out = buf[-2:]
    N.call(f"axi_force_projection_{s}", float(rho_s), N.ptr(char_func), N.ptr(u_z), N.ptr(u_r),
           N.ptr(R), R.numel(), N.ptr(buf), N.ptr(out), N.stream_of(R))
    U_z, U_r = out.tolist()
    return U_z, U_r
