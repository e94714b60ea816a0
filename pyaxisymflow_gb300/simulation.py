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
