"""Drop-in for pyaxisymflow/kernels/compute_forces.py:4-17 (FP64 accumulation)."""
import torch

from .. import _native as N


def _scratch(device):
    n = N.lib().axi_reduction_scratch_doubles(0)
    return torch.empty(n + 2, dtype=torch.float64, device=device)


def compute_force_on_body(R, part_char_func, rho_f, brink_lam, u_z, U_z_cm_part, part_vol, dt,
                          diff):
    """computes brinkman penalization force and unsteady force; returns
    (F_pen, F_un) as Python floats (synchronises the stream)."""
    s = N.require(R, part_char_func, u_z, shape=R.shape, names=("R", "part_char_func", "u_z"))
    buf = _scratch(R.device)
    out = buf[-2:]
    N.call(f"axi_compute_force_on_body_{s}", N.ptr(R), N.ptr(part_char_func), float(rho_f),
           float(brink_lam), N.ptr(u_z), float(U_z_cm_part), float(part_vol), float(dt),
           float(diff), R.numel(), N.ptr(buf), N.ptr(out), N.stream_of(R))
    F_pen, F_un = out.tolist()
    return F_pen, F_un
