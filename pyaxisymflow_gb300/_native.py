"""ctypes binding of the CUDA library (include/axisym_gb300.h).

The library is built in-tree (``pyaxisymflow_gb300/_build``) by
``pyaxisymflow_gb300.build``. There is no CPU fallback: importing a kernel
module without the built library, or calling it with tensors that are not on
a CUDA device, raises.
"""
import ctypes
import os

import torch

from . import build as _build

_c = ctypes
P = _c.c_void_p
I = _c.c_int
I64 = _c.c_int64
D = _c.c_double
F = _c.c_float

AXI_OK = 0
AXI_ERR_INVALID = 1
AXI_ERR_CUDA = 2
AXI_ERR_NOT_CONVERGED = 3
AXI_ERR_NONFINITE = 4
AXI_ERR_RANGE = 5


class AxiError(RuntimeError):
    """A failing status from the CUDA library."""

    def __init__(self, status, message):
        super().__init__(message)
        self.status = status


def _real(suffix):
    return D if suffix == "f64" else F


def _signatures():
    sig = {
        "axi_version": (I, []),
        "axi_last_error": (_c.c_char_p, []),
        "axi_reduction_scratch_doubles": (I64, [I64]),
        "axi_lsq_work_bytes": (I64, [I, I]),
        "axi_p2m_mp4_work_bytes": (I64, [I, I]),
        "axi_particles_to_mesh_2d_mp4_f64": (I, [P, P, P, P, I, I, D, D, I, P, P]),
        "axi_p2m_status": (I, [P, I, I, P, P]),
        "axi_mesh_to_particles_2d_mp4_f64": (I, [P, P, I, I, P, P, P, P, I, I, D, D, I, P]),
        "axi_level_set_work_bytes": (I64, [I, I]),
        "axi_level_set_distance_f64": (I, [P, P, I, I, D, D, P, P, P]),
        "axi_advect_particles_prepare_f64": (I, [P, P, P, P, P, P, I, I, D, P]),
        "axi_extrapolate_lsq_first_order_f64": (I, [P, P, P, P, P, P, I, I, I, P, P, P]),
        "axi_extrapolate_eta_with_least_squares_f64": (
            I, [P, P, P, P, P, P, P, P, P, D, I, I, P, P, I, P, P, P]),
        "axi_fd_transform_f64": (I, [P, I, P, I, P, P, P, P, P, P, I, I, P]),
        "axi_fd_transform_static_max_cells": (I64, []),
        "axi_fd_transform_static_f64": (I, [P, I, P, I, P, P, P, P, P, I, I, P]),
        "axi_dgemm_f64": (I, [P, I, P, I, P, I, P, I, I, I, P]),
        "axi_tf32x3_gemm_work_bytes": (I64, [I, I, I]),
        "axi_tc_transform_plan": (I, [P, I, P, P, P]),
        "axi_tc_transform_run": (I, [P, P, P]),
        "axi_tc_transform_status": (I, [P, P, P, P]),
        "axi_tc_split_f32": (I, [P, P, P, I64, P]),
        "axi_tc_split_f64": (I, [P, P, P, I64, P]),
        "axi_fd_residual_f64": (I, [P, P, P, P, P, P, I, I, D, D, P]),
        "axi_add_f32_to_f64": (I, [P, P, I64, P]),
        "axi_widen_f32_to_f64": (I, [P, P, I64, P]),
        "axi_tf32x3_gemm": (I, [P, P, P, I, I, I, P, P]),
        "axi_plan_init": (I, [P, I, I, I, P]),
        "axi_plan_tc_status": (I, [P, P, P, P]),
        "axi_rigid_refresh_operands": (I, [P, P, P]),
        "axi_plan_upload": (I, [P, P, P, P]),
        "axi_rigid_step_f64": (I, [P, P, I, P]),
        "axi_rigid_step_f32": (I, [P, P, I, P]),
        "axi_rigid_phase_f64": (I, [P, P, I, P]),
        "axi_rigid_phase_f32": (I, [P, P, I, P]),
        # the soft-sphere loop with dt and t on the device
        "axi_soft_dt_f64": (I, [P, P, I64, P, D, D, D, D, P]),
        "axi_soft_advect_eno3_f64": (I, [P, P, I, P, P, P, I, I, D, P, P]),
        "axi_soft_pin_level_set_f64": (I, [P, P, P, I64, D, D, D, P]),
        "axi_soft_mask_f64": (I, [P, P, P, I64, D, P]),
        "axi_soft_extrapolate_eta_f64": (
            I, [P, P, P, P, P, P, P, P, P, D, I, I, P, P, I, P, P, P]),
        "axi_soft_stress_mask_f64": (I, [P, P, P, P, I64, P]),
        "axi_soft_update_vorticity_from_solid_stress_f64": (
            I, [P, P, P, P, P, P, P, I, I, D, P, P]),
        "axi_soft_tether_f64": (I, [P, P, P, I64, P, D, D, D, D, D, P]),
        "axi_soft_penalise_f64": (I, [P, P, P, P, P, P, I, I, D, D, D, D, P, P]),
        "axi_soft_diffusion_rk2_f64": (I, [P, P, P, I, I, D, D, P, P]),
        "axi_soft_advance_f64": (I, [P, P]),
        "axi_dct64_plan_bytes": (I64, [I, I]),
        "axi_dct64_plan_f64": (I, [P, P, I, I, P, I, P, P]),
        "axi_dct64_run_f64": (I, [P, I, I, I, P]),
    }
    for s in ("f64", "f32"):
        T = _real(s)
        sig.update({
            f"axi_velocity_from_psi_unb_{s}": (I, [P, P, P, P, I, I, T, P]),
            f"axi_velocity_from_psi_periodic_{s}": (I, [P, P, P, P, I, I, T, I, P]),
            f"axi_vorticity_from_velocity_unb_{s}": (I, [P, P, P, I, I, T, P]),
            f"axi_vorticity_from_velocity_periodic_{s}": (I, [P, P, P, I, I, T, I, P]),
            f"axi_brinkmann_penalize_{s}": (I, [T, T, P, T, T, P, P, P, P, I64, P]),
            f"axi_smooth_heaviside_{s}": (I, [P, P, T, I64, P]),
            f"axi_kill_boundary_vorticity_sine_z_{s}": (I, [P, P, I, I, I, T, P]),
            f"axi_kill_boundary_vorticity_sine_r_{s}": (I, [P, P, I, I, I, T, P]),
            f"axi_diffusion_rk2_unb_{s}": (I, [P, P, P, I, I, T, T, T, P]),
            f"axi_diffusion_rk2_periodic_{s}": (I, [P, P, P, I, I, T, T, T, I, P]),
            f"axi_periodic_ghost_comm_{s}": (I, [P, I, I, I, P]),
            f"axi_periodic_ghost_comm_eta_{s}": (I, [P, I, I, I, T, T, P]),
            f"axi_compute_force_on_body_{s}": (I, [P, P, D, D, P, D, D, D, D, I64, P, P, P]),
            f"axi_force_projection_{s}": (I, [D, P, P, P, P, I64, P, P, P]),
            f"axi_advect_vorticity_eno3_{s}": (I, [P, P, P, P, I, I, T, P]),
            f"axi_advect_vorticity_eno3_periodic_{s}": (I, [P, P, P, P, I, I, T, I, P]),
            f"axi_advect_refmap_eno3_{s}": (I, [P, P, P, P, P, I, I, T, P]),
            f"axi_advect_refmap_eno3_periodic_{s}": (I, [P, P, P, P, P, I, I, T, I, T, T, P]),
            f"axi_solid_sigma_{s}": (I, [P, P, P, T, T, P, P, P, P, P, P, I, I, P]),
            f"axi_update_vorticity_from_solid_stress_{s}": (
                I, [P, P, P, P, P, P, P, I, I, T, T, P]),
        })
    return sig


SIGNATURES = _signatures()

_lib = None


def library_path():
    return _build.lib_path()


def lib():
    """The loaded library; raises if it has not been built."""
    global _lib
    if _lib is None:
        path = library_path()
        if not os.path.exists(path):
            raise ImportError(
                f"CUDA library not built ({path} missing); run "
                "`python -c 'import __graft_entry__ as g; g.build()'`")
        handle = _c.CDLL(path)
        for name, (res, args) in SIGNATURES.items():
            fn = getattr(handle, name)
            fn.restype = res
            fn.argtypes = args
        _lib = handle
    return _lib


def check(status, what=""):
    if status != AXI_OK:
        msg = lib().axi_last_error().decode(errors="replace")
        raise AxiError(status, f"{what}: {msg}" if what else msg)


def call(name, *args):
    """Call an entry point and raise AxiError on a failing status."""
    check(getattr(lib(), name)(*args), name)


def suffix(t):
    if t.dtype == torch.float64:
        return "f64"
    if t.dtype == torch.float32:
        return "f32"
    raise TypeError(f"unsupported dtype {t.dtype}; expected float64 or float32")


def ptr(t):
    return _c.c_void_p(t.data_ptr())


def stream_of(t):
    """Handle of torch's current stream on the tensor's device."""
    return _c.c_void_p(torch.cuda.current_stream(t.device).cuda_stream)


def require(*tensors, shape=None, dtype=None, names=None):
    """Check the drop-in contract: CUDA, contiguous, same dtype/shape/device."""
    first = tensors[0]
    for k, t in enumerate(tensors):
        name = names[k] if names else f"argument {k}"
        if not isinstance(t, torch.Tensor):
            raise TypeError(f"{name} must be a torch.Tensor on a CUDA device")
        if not t.is_cuda:
            raise ValueError(f"{name} must be on a CUDA device (there is no CPU path)")
        if not t.is_contiguous():
            raise ValueError(f"{name} must be contiguous (row-major (nr, nz))")
        if t.dtype != (dtype or first.dtype):
            raise TypeError(f"{name} has dtype {t.dtype}, expected {dtype or first.dtype}")
        if t.device != first.device:
            raise ValueError(f"{name} is on {t.device}, expected {first.device}")
        if shape is not None and tuple(t.shape) != tuple(shape):
            raise ValueError(f"{name} has shape {tuple(t.shape)}, expected {tuple(shape)}")
    return suffix(first) if first.dtype in (torch.float32, torch.float64) else None


def real(sfx, x):
    return (D if sfx == "f64" else F)(float(x))
