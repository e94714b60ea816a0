"""The oracle's rigid and sedimenting sphere loops with their per-step grid
kernels in C + OpenMP (oracle/cstep.c). TEST / MEASUREMENT INFRASTRUCTURE
ONLY: this is the timed CPU baseline (the reference runs these kernels as
numba-compiled loops and its ENO3 advection as pystencils-generated C with
OpenMP); tests check it against the numpy oracle bit for bit.

What stays in numpy, as in the reference: the boundary-vorticity taper, the
spectral solve (BLAS, kernels/FastDiagonalisationStokesSolver.py:130-156) and
the drag and force sums (np.sum). The sedimenting body's mask rebuild
(numba smooth_Heaviside in the reference) runs in C.
"""
import ctypes
import os

import numpy as np

from . import build
from . import kernels as K
from . import simulation as sim

_LIB = None


def lib():
    """The compiled restatement (built on first use when missing)."""
    global _LIB
    if _LIB is None:
        path = build.cstep_path()
        if not os.path.exists(path):
            build.build_cstep()
        L = ctypes.CDLL(path)
        vp, ci, cd = ctypes.c_void_p, ctypes.c_int, ctypes.c_double
        L.ora_velocity_from_psi.restype = cd
        L.ora_velocity_from_psi.argtypes = [vp, vp, vp, vp, ci, ci, cd, ci, cd]
        L.ora_penalise.restype = None
        L.ora_penalise.argtypes = [vp, vp, vp, vp, ci, ci, cd, cd, cd, vp, vp]
        L.ora_advect_eno3.restype = None
        L.ora_advect_eno3.argtypes = [vp, vp, vp, ci, ci, cd, vp]
        L.ora_diffusion_rk2.restype = None
        L.ora_diffusion_rk2.argtypes = [vp, vp, vp, vp, ci, ci, cd, cd, cd]
        L.ora_sphere_mask.restype = None
        L.ora_sphere_mask.argtypes = [vp, vp, vp, ci, ci, cd, cd, cd]
        L.ora_set_threads.restype = None
        L.ora_set_threads.argtypes = [ci]
        L.ora_max_threads.restype = ci
        _LIB = L
    return _LIB


def set_threads(n):
    lib().ora_set_threads(int(n))


def threads():
    return int(lib().ora_max_threads())


def _p(a):
    assert a.dtype == np.float64 and a.flags.c_contiguous
    return a.ctypes.data


class CStepScratch:
    """Per-case arrays of the C kernels: r^-2 (as the oracle forms it) and
    three (nr, nz) scratch fields."""

    def __init__(self, R):
        self.Rm2 = np.ascontiguousarray(R ** -2)
        self.a = np.zeros_like(R)
        self.b = np.zeros_like(R)
        self.c = np.zeros_like(R)


def rigid_sphere_step(case, st, coords, solver, ex):
    """sim.rigid_sphere_step (examples/FlowPastSphere/flow_past_sphere.py:107-188)
    with the grid kernels in C; `ex` is the case's CStepScratch."""
    L = lib()
    z, r, Z, R = coords
    dx = case.dx
    nr, nz = case.nr, case.nz
    w = st.vorticity
    K.kill_boundary_vorticity_sine_z(w, Z, case.kill_width, dx)
    K.kill_boundary_vorticity_sine_r(w, R, case.kill_width, dx)
    solver.solve(solution_field=st.psi, rhs_field=w)
    prefac = 1.0
    if case.ramp and st.t < case.t_ramp:
        prefac = np.sin(0.5 * np.pi * st.t / case.t_ramp)
    vmax = L.ora_velocity_from_psi(_p(st.u_z), _p(st.u_r), _p(st.psi), _p(R), nr, nz, dx, 1,
                                   case.U0 * prefac)
    dt = min(0.9 * dx ** 2 / 4 / case.nu, case.cfl * dx / (vmax + sim.EPS))
    L.ora_penalise(_p(w), _p(st.u_z), _p(st.u_r), _p(st.char_func), nr, nz, case.lam * dt, 0.0,
                   dx, _p(ex.a), _p(ex.b))
    st.Cd = (2 * 2 * np.pi * dx * dx * case.lam * np.sum(R * st.char_func * st.u_z)
             / (np.pi * case.r_sphere ** 2))
    L.ora_advect_eno3(_p(w), _p(st.u_z), _p(st.u_r), nr, nz, dt / dx, _p(ex.a))
    L.ora_diffusion_rk2(_p(w), _p(ex.b), _p(R), _p(ex.Rm2), nr, nz, case.nu, dt, dx)
    st.dt = dt
    st.t += dt
    st.it += 1
    return st


def sedimenting_step(case, st, coords, solver, ex):
    """sim.sedimenting_step (examples/SedimentingRigidSphere/falling_rigid_sphere.py:96-187)
    with the grid kernels in C."""
    L = lib()
    z, r, Z, R = coords
    dx = case.dx
    nr, nz = case.nr, case.nz
    g = (case.rho_s - case.rho_f) * case.gravity
    w = st.vorticity
    K.kill_boundary_vorticity_sine_z(w, Z, case.kill_width, dx)
    K.kill_boundary_vorticity_sine_r(w, R, case.kill_width, dx)
    solver.solve(solution_field=st.psi, rhs_field=w)
    vmax = L.ora_velocity_from_psi(_p(st.u_z), _p(st.u_r), _p(st.psi), _p(R), nr, nz, dx, 0,
                                   0.0)
    dt = min(0.9 * dx ** 2 / 4 / case.nu, case.cfl * dx / (vmax + sim.EPS))
    L.ora_penalise(_p(w), _p(st.u_z), _p(st.u_r), _p(st.char_func), nr, nz, case.lam * dt,
                   st.U_z_cm_part, dx, _p(ex.a), _p(ex.b))
    F_pen, F_un = K.compute_force_on_body(R, st.char_func, case.rho_f, case.lam, st.u_z,
                                          st.U_z_cm_part, st.part_vol, dt, st.diff)
    F_total = 2 * np.pi * dx * dx * F_pen + F_un
    L.ora_sphere_mask(_p(st.char_func), _p(Z), _p(R), nr, nz, st.part_Z_cm, case.r_sphere,
                      case.moll_zone)
    L.ora_advect_eno3(_p(w), _p(st.u_z), _p(st.u_r), nr, nz, dt / dx, _p(ex.a))
    L.ora_diffusion_rk2(_p(w), _p(ex.b), _p(R), _p(ex.Rm2), nr, nz, case.nu, dt, dx)
    st.Cd = (2 * 2 * np.pi * dx * dx * case.lam * np.sum(R * st.char_func * st.u_z)
             / (np.pi * case.r_sphere ** 2))
    U_old = st.U_z_cm_part
    st.U_z_cm_part += dt * ((-g + (F_total / st.part_mass)))
    st.diff = dt * (-g / case.rho_s + (F_total / st.part_mass))
    st.part_Z_cm += U_old * dt + (0.5 * dt * dt * (-g / case.rho_s + (F_total / st.part_mass)))
    st.F_total = F_total
    st.dt = dt
    st.t += dt
    st.it += 1
    return st
