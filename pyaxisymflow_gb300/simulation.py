"""Per-timestep drivers of the reference examples on the GPU.

RigidSphereSimulation runs the loop body of
examples/FlowPastSphere/flow_past_sphere.py:107-188 (kill boundary vorticity,
stream-function solve, velocity, free stream, CFL time step, Brinkman
penalisation and its vorticity, drag, ENO3 advection, RK2 diffusion) with all
fields resident on one GPU.
"""
import math

import numpy as np
import torch

from .kernels.advect_vorticity_via_eno3 import gen_advect_vorticity_via_eno3
from .kernels.brinkmann_penalize import brinkmann_penalize
from .kernels.compute_velocity_from_psi import compute_velocity_from_psi_unb
from .kernels.compute_vorticity_from_velocity import compute_vorticity_from_velocity_unb
from .kernels.diffusion_RK2 import diffusion_RK2_unb
from .kernels.FastDiagonalisationStokesSolver import FastDiagonalisationStokesSolver
from .kernels.kill_boundary_vorticity_sine import (kill_boundary_vorticity_sine_r,
                                                   kill_boundary_vorticity_sine_z)
from .kernels.smooth_Heaviside import smooth_Heaviside

EPS = float(np.finfo(float).eps)


def grid(nz, nr, dx):
    """Cell-centred coordinates (examples/FlowPastSphere/flow_past_sphere.py:58-60)."""
    z = np.linspace(dx / 2, nz * dx - dx / 2, nz)
    r = np.linspace(dx / 2, nr * dx - dx / 2, nr)
    Z, R = np.meshgrid(z, r)
    return z, r, Z, R


class RigidSphereSimulation:
    """Flow past a fixed rigid sphere, FP64, through the drop-in kernels.

    `case` carries nz, nr, dx, z_cm, r_sphere, U0, nu, lam, cfl, kill_width,
    ramp, t_ramp, moll_zone, noise and seed (the names of
    examples/FlowPastSphere/flow_past_sphere.py:39-55).
    """

    def __init__(self, case, device="cuda", vorticity=None):
        self.case = case
        dev = torch.device(device)
        self.device = dev
        c = case
        z, r, Z, R = grid(c.nz, c.nr, c.dx)
        f64 = dict(dtype=torch.float64, device=dev)
        self.Z = torch.tensor(Z, **f64)
        self.R = torch.tensor(R, **f64)
        if vorticity is None:
            rng = np.random.default_rng(c.seed)
            vorticity = c.noise * rng.standard_normal((c.nr, c.nz))
        self.vorticity = torch.tensor(np.asarray(vorticity), **f64)
        phi0 = -np.sqrt((Z - c.z_cm) ** 2 + R ** 2) + c.r_sphere
        self.char_func = torch.zeros((c.nr, c.nz), **f64)
        smooth_Heaviside(self.char_func, torch.tensor(phi0, **f64), c.moll_zone)
        self.psi = torch.zeros((c.nr, c.nz), **f64)
        self.u_z = torch.zeros_like(self.psi)
        self.u_r = torch.zeros_like(self.psi)
        self.u_z_upen = torch.zeros_like(self.psi)
        self.u_r_upen = torch.zeros_like(self.psi)
        self.penal = torch.zeros_like(self.psi)
        self.tmp = torch.zeros_like(self.psi)
        self.solver = FastDiagonalisationStokesSolver(c.nr, c.nz, c.dx, device=dev)
        self.advect = gen_advect_vorticity_via_eno3(c.dx, c.nr, c.nz)
        self.t = 0.0
        self.it = 0
        self.dt = 0.0
        self.Cd = 0.0

    def step(self):
        c = self.case
        dx = c.dx
        w = self.vorticity
        kill_boundary_vorticity_sine_z(w, self.Z, c.kill_width, dx)
        kill_boundary_vorticity_sine_r(w, self.R, c.kill_width, dx)
        self.solver.solve(self.psi, w)
        compute_velocity_from_psi_unb(self.u_z, self.u_r, self.psi, self.R, dx)
        prefac = 1.0
        if c.ramp and self.t < c.t_ramp:
            prefac = math.sin(0.5 * math.pi * self.t / c.t_ramp)
        self.u_z += c.U0 * prefac
        umax = float(torch.amax(torch.abs(self.u_z) + torch.abs(self.u_r)))
        dt = min(0.9 * dx ** 2 / 4 / c.nu, c.cfl * dx / (umax + EPS))
        self.u_z_upen.copy_(self.u_z)
        self.u_r_upen.copy_(self.u_r)
        brinkmann_penalize(c.lam, dt, self.char_func, 0.0, 0.0, self.u_z_upen, self.u_r_upen,
                           self.u_z, self.u_r)
        compute_vorticity_from_velocity_unb(self.penal, self.u_z - self.u_z_upen,
                                            self.u_r - self.u_r_upen, dx)
        w += self.penal
        self.Cd = (2 * 2 * math.pi * dx * dx * c.lam
                   * float(torch.sum(self.R * self.char_func * self.u_z))
                   / (math.pi * c.r_sphere ** 2))
        self.advect(w, self.u_z, self.u_r, dt)
        diffusion_RK2_unb(w, self.tmp, self.R, c.nu, dt, dx)
        self.dt = dt
        self.t += dt
        self.it += 1

    def run(self, n):
        for _ in range(n):
            self.step()


class SoftSphereSimulation:
    """Soft neo-Hookean sphere driven by an oscillating penalised tether, FP64,
    through the drop-in kernels: the loop body of
    examples/SoftSphereStreaming/soft_sphere_streaming.py:129-272 without
    plotting / averaging and without the scikit-fmm narrow-band
    reinitialisation (:196-199): the level set is the analytic pinned one in
    the band (:191-193) and keeps its previous value elsewhere.

    `case` carries nz, nr, dx, z_cm, r_ball, rho_f, omega, U0, nu, G, lam, cfl,
    kill_width, zeta, moll_zone and extrap_zone (names of the example).
    """

    def __init__(self, case, device="cuda"):
        from .elasto_kernels.advect_refmap_via_eno3 import gen_advect_refmap_via_eno3
        self.case = c = case
        dev = torch.device(device)
        f64 = dict(dtype=torch.float64, device=dev)
        z, r, Z, R = grid(c.nz, c.nr, c.dx)
        nzd = 2 * c.nr
        zd = np.linspace(c.dx / 2, nzd * c.dx - c.dx / 2, nzd) if nzd > c.nz else z
        self.z = torch.tensor(zd, **f64)
        self.Z = torch.tensor(Z, **f64)
        self.R = torch.tensor(R, **f64)
        phi = -np.sqrt((Z - c.z_cm) ** 2 + R ** 2) + c.r_ball
        self.ball_phi = torch.tensor(phi, **f64)
        self.ball_char_func = torch.zeros_like(self.ball_phi)
        smooth_Heaviside(self.ball_char_func, self.ball_phi, c.moll_zone)
        self.tether_char_func = torch.zeros_like(self.ball_phi)
        tphi = -np.sqrt((Z - c.z_cm) ** 2 + R ** 2) + c.zeta * c.r_ball
        smooth_Heaviside(self.tether_char_func, torch.tensor(tphi, **f64), c.moll_zone)
        zeros = lambda: torch.zeros((c.nr, c.nz), **f64)  # noqa: E731
        self.vorticity, self.psi, self.u_z, self.u_r = zeros(), zeros(), zeros(), zeros()
        self.u_z_upen, self.u_r_upen, self.penal, self.tmp = zeros(), zeros(), zeros(), zeros()
        self.eta1 = self.Z.clone()
        self.eta2 = self.R.clone()
        self.s11, self.s12, self.s22 = zeros(), zeros(), zeros()
        self.e1z, self.e1r, self.e2z, self.e2r = zeros(), zeros(), zeros(), zeros()
        self.tau_z, self.tau_r = zeros(), zeros()
        self.phi_d = torch.zeros((2 * c.nr, c.nz), **f64)
        self.e1_d = torch.zeros_like(self.phi_d)
        self.e2_d = torch.zeros_like(self.phi_d)
        self.solver = FastDiagonalisationStokesSolver(c.nr, c.nz, c.dx, device=dev)
        self.advect_w = gen_advect_vorticity_via_eno3(c.dx, c.nr, c.nz)
        self.advect_eta = gen_advect_refmap_via_eno3(c.dx, c.nr, c.nz)
        self.t = 0.0
        self.it = 0
        self.dt = 0.0

    def step(self):
        from .elasto_kernels.div_tau import update_vorticity_from_solid_stress
        from .elasto_kernels.extrapolate_eta_using_least_squares_unb import \
            extrapolate_eta_with_least_squares
        from .elasto_kernels.solid_sigma import solid_sigma
        c = self.case
        dx = c.dx
        w = self.vorticity
        kill_boundary_vorticity_sine_z(w, self.Z, c.kill_width, dx)
        kill_boundary_vorticity_sine_r(w, self.R, c.kill_width, dx)
        self.solver.solve(self.psi, w)
        compute_velocity_from_psi_unb(self.u_z, self.u_r, self.psi, self.R, dx)
        umax = float(torch.amax(torch.abs(self.u_z) + torch.abs(self.u_r)))
        dt = min(c.cfl * dx / math.sqrt(c.G / c.rho_f), c.cfl * dx / (umax + EPS),
                 0.9 * dx ** 2 / 4 / c.nu)
        self.advect_eta(self.eta1, self.eta2, self.u_z, self.u_r, dt)
        # pin the level set to the advected reference map in the band (:191-193)
        phi_orig = -torch.sqrt((self.eta1 - c.z_cm) ** 2 + self.eta2 ** 2) + c.r_ball
        band = self.ball_phi > -3 * dx
        self.ball_phi = torch.where(band, phi_orig, self.ball_phi)
        self.advect_w(w, self.u_z, self.u_r, dt)
        smooth_Heaviside(self.ball_char_func, self.ball_phi, c.moll_zone)
        inside_solid = self.ball_char_func > 0.5
        extrapolate_eta_with_least_squares(inside_solid, self.ball_phi, self.eta1, self.eta2,
                                           self.phi_d, self.e1_d, self.e2_d, c.extrap_zone,
                                           c.nr, self.z)
        solid_sigma(self.s11, self.s12, self.s22, c.G, dx, self.eta1, self.eta2, self.e1z,
                    self.e1r, self.e2z, self.e2r)
        self.s11 *= self.ball_char_func
        self.s12 *= self.ball_char_func
        self.s22 *= self.ball_char_func
        update_vorticity_from_solid_stress(w, self.tau_z, self.tau_r, self.s11, self.s12,
                                           self.s22, self.R, dt, dx)
        z_cm_t = c.z_cm + c.e * c.r_ball * math.sin(c.omega * self.t)
        tphi = -torch.sqrt((self.Z - z_cm_t) ** 2 + self.R ** 2) + c.zeta * c.r_ball
        smooth_Heaviside(self.tether_char_func, tphi.contiguous(), c.moll_zone)
        self.u_z_upen.copy_(self.u_z)
        self.u_r_upen.copy_(self.u_r)
        brinkmann_penalize(c.lam, dt, self.tether_char_func, c.U0 * math.cos(c.omega * self.t),
                           0.0, self.u_z_upen, self.u_r_upen, self.u_z, self.u_r)
        compute_vorticity_from_velocity_unb(self.penal, self.u_z - self.u_z_upen,
                                            self.u_r - self.u_r_upen, dx)
        w += self.penal
        diffusion_RK2_unb(w, self.tmp, self.R, c.nu, dt, dx)
        self.dt = dt
        self.t += dt
        self.it += 1

    def run(self, n):
        for _ in range(n):
            self.step()
