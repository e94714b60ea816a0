"""Per-timestep drivers of the reference examples on the GPU.

RigidSphereSimulation runs the loop body of
examples/FlowPastSphere/flow_past_sphere.py:107-188 (kill boundary vorticity,
stream-function solve, velocity, free stream, CFL time step, Brinkman
penalisation and its vorticity, drag, ENO3 advection, RK2 diffusion) with all
fields resident on one GPU. SoftSphereSimulation runs the soft-sphere
streaming loop through the drop-in kernels (dt formed on the host each
step); SoftSphereEngine runs the same loop with dt and t on the device.
"""
import ctypes
import math
from dataclasses import dataclass

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


@dataclass
class SoftCase:
    """Parameters of the soft-sphere streaming loop, named as in
    examples/SoftSphereStreaming/soft_sphere_streaming.py:31-63 (defaults:
    that example on its 256 x 128 grid); derived quantities follow its
    formulas."""
    nz: int = 256
    nr: int = 128
    dx: float = 1.0 / 256
    z_cm: float = 0.5
    r_ball: float = 0.15
    rho_f: float = 1.0
    freq: float = 16.0
    nond_AC: float = 0.125
    e: float = 0.1
    cauchy: float = 0.1
    zeta: float = 0.25
    lam: float = 1e8
    cfl: float = 0.1
    kill_width: int = 3

    @property
    def omega(self):
        return 2 * np.pi * self.freq

    @property
    def U0(self):
        return self.e * self.r_ball * self.omega

    @property
    def nu(self):
        Rs = (self.e / self.nond_AC) ** 2
        return self.e * self.U0 * self.r_ball / Rs

    @property
    def G(self):
        return self.e * self.rho_f * (self.r_ball * self.omega) ** 2 / self.cauchy

    @property
    def moll_zone(self):
        return self.dx * 2

    @property
    def extrap_zone(self):
        return self.moll_zone + 4 * self.dx


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


# state words of the device-resident soft loop (include/axisym_gb300.h AXI_SOFT_*)
SOFT_T, SOFT_DT, SOFT_STEPS, SOFT_STATUS, SOFT_SWEEPS, SOFT_WORDS = 0, 1, 2, 3, 4, 8


class SoftSphereEngine:
    """The soft-sphere loop of SoftSphereSimulation with the time step and
    the simulated time resident on the device: a kernel reduces
    max(|u_z| + |u_r|) into dt, the dt- and t-dependent kernels read it
    there, and no step reads anything back to the host, so a run of steps can
    be captured in a CUDA graph (capture / replay). The arithmetic is that of
    the drop-in kernels, with sin and cos of omega t taken on the device.
    Extrapolation failures set bits of status() instead of raising."""

    def __init__(self, case, device="cuda", dct=False):
        from . import _native as N
        from .core.extrapolate_using_least_squares import MAX_SWEEPS
        self._N = N
        self.max_sweeps = MAX_SWEEPS
        self.sim = s = SoftSphereSimulation(case, device=device)
        self.case = c = case
        self.device = torch.device(device)
        self.dct = bool(dct)
        nr, nz = c.nr, c.nz
        f64 = dict(dtype=torch.float64, device=self.device)
        self.state = torch.zeros(SOFT_WORDS, **f64)
        self.inside = torch.zeros((nr, nz), dtype=torch.uint8, device=self.device)
        self.flags = torch.zeros((2, 2 * nr, nz), dtype=torch.int16, device=self.device)
        self.lsq_work = torch.zeros(int(N.lib().axi_lsq_work_bytes(2 * nr, nz)),
                                    dtype=torch.uint8, device=self.device)
        self.scratch2 = torch.zeros(2 * nr * nz, **f64)
        if self.dct:
            self._setup_dct()
        dx = c.dx
        self.dt_elastic = c.cfl * dx / math.sqrt(c.G / c.rho_f)
        self.cfl_dx = c.cfl * dx
        self.dt_diffusive = 0.9 * dx ** 2 / 4 / c.nu
        self.graph = None

    def _setup_dct(self):
        """The spectral solve with the z products as FP64 DCT-II / DCT-III row
        transforms (the Neumann z operator is diagonal in the cosine basis;
        psi does not depend on which eigenbasis diagonalises it): E_z^-1 and
        E_z become O(nz log nz) per row, the radial products stay dense. psi
        differs from the dense eigenvector products by ~1e-12 of a solve."""
        from .engine import dct_ok, dct_table
        N, s, c = self._N, self.sim, self.case
        nr, nz, dx = c.nr, c.nz, c.dx
        if not dct_ok(nz, "f64"):
            raise ValueError(f"nz = {nz} has no FP64 DCT plan (even, factors 2 and 3 only, "
                             "<= 2048)")
        eng = s.solver.engine
        f64 = dict(dtype=torch.float64, device=self.device)
        lam_z = (2.0 - 2.0 * np.cos(np.pi * np.arange(nz) / nz)) / (dx * dx)
        self.inv_eig_dct = torch.tensor(1.0 / (eng.eig_vals_r.reshape(nr, 1)
                                               + lam_z.reshape(1, nz)), **f64)
        self.dct_tab = torch.tensor(dct_table(nz, np.float64), **f64)
        self.w1 = torch.zeros((nr, nz), **f64)
        self.w2 = torch.zeros((nr, nz), **f64)
        nb = int(N.lib().axi_dct64_plan_bytes(nr, nz))
        self.plan_fwd = torch.zeros(nb, dtype=torch.uint8, device=self.device)
        self.plan_inv = torch.zeros(nb, dtype=torch.uint8, device=self.device)
        st = N.stream_of(self.w1)
        N.call("axi_dct64_plan_f64", N.ptr(s.vorticity), N.ptr(self.w1), nr, nz,
               N.ptr(self.dct_tab), 1, N.ptr(self.plan_fwd), st)
        N.call("axi_dct64_plan_f64", N.ptr(self.w2), N.ptr(self.w1), nr, nz,
               N.ptr(self.dct_tab), 0, N.ptr(self.plan_inv), st)

    def _solve(self, st):
        N, s, c = self._N, self.sim, self.case
        if not self.dct:
            s.solver.solve(s.psi, s.vorticity)
            return
        p = N.ptr
        nr, nz = c.nr, c.nz
        d = s.solver.engine.dev
        N.call("axi_dct64_run_f64", p(self.plan_fwd), nr, nz, 1, st)
        N.call("axi_dgemm_f64", p(self.w2), nz, p(d["Er_inv_w"]), nr, p(self.w1), nz,
               p(self.inv_eig_dct), nr, nz, nr, st)
        N.call("axi_dct64_run_f64", p(self.plan_inv), nr, nz, 0, st)
        N.call("axi_dgemm_f64", p(s.psi), nz, p(d["Er"]), nr, p(self.w1), nz, None, nr, nz,
               nr, st)

    # the launch groups of one step, in order (timed one at a time by phase())
    PARTS = ("solve_velocity_dt", "advect_pin_mask", "extrapolate", "solid_stress",
             "tether_penalise_diffuse")

    def _part(self, k, st):
        N, s, c = self._N, self.sim, self.case
        p = N.ptr
        nr, nz, dx = c.nr, c.nz, c.dx
        n = nr * nz
        w = s.vorticity
        if k == 0:
            N.call("axi_kill_boundary_vorticity_sine_z_f64", p(w), p(s.Z), nr, nz, c.kill_width,
                   dx, st)
            N.call("axi_kill_boundary_vorticity_sine_r_f64", p(w), p(s.R), nr, nz, c.kill_width,
                   dx, st)
            self._solve(st)
            N.call("axi_velocity_from_psi_unb_f64", p(s.u_z), p(s.u_r), p(s.psi), p(s.R), nr, nz,
                   dx, st)
            N.call("axi_soft_dt_f64", p(s.u_z), p(s.u_r), n, p(self.state), self.dt_elastic,
                   self.cfl_dx, self.dt_diffusive, EPS, st)
        elif k == 1:
            N.call("axi_soft_advect_eno3_f64", p(s.eta1), p(s.eta2), 1, p(s.u_z), p(s.u_r),
                   p(self.scratch2), nr, nz, dx, p(self.state), st)
            N.call("axi_soft_pin_level_set_f64", p(s.ball_phi), p(s.eta1), p(s.eta2), n, c.z_cm,
                   c.r_ball, -3 * dx, st)
            N.call("axi_soft_advect_eno3_f64", p(w), None, 0, p(s.u_z), p(s.u_r),
                   p(self.scratch2), nr, nz, dx, p(self.state), st)
            N.call("axi_soft_mask_f64", p(s.ball_char_func), p(self.inside), p(s.ball_phi), n,
                   c.moll_zone, st)
        elif k == 2:
            N.call("axi_soft_extrapolate_eta_f64", p(self.inside), p(s.ball_phi), p(s.eta1),
                   p(s.eta2), p(s.phi_d), p(s.e1_d), p(s.e2_d), p(self.flags[0]),
                   p(self.flags[1]), float(c.extrap_zone), nr, nz, p(s.z), p(s.z),
                   self.max_sweeps, p(self.lsq_work), p(self.state), st)
        elif k == 3:
            N.call("axi_solid_sigma_f64", p(s.s11), p(s.s12), p(s.s22), c.G, dx, p(s.eta1),
                   p(s.eta2), p(s.e1z), p(s.e1r), p(s.e2z), p(s.e2r), nr, nz, st)
            N.call("axi_soft_stress_mask_f64", p(s.s11), p(s.s12), p(s.s22),
                   p(s.ball_char_func), n, st)
            N.call("axi_soft_update_vorticity_from_solid_stress_f64", p(w), p(s.tau_z),
                   p(s.tau_r), p(s.s11), p(s.s12), p(s.s22), p(s.R), nr, nz, dx, p(self.state),
                   st)
        else:
            N.call("axi_soft_tether_f64", p(s.tether_char_func), p(s.Z), p(s.R), n,
                   p(self.state), c.z_cm, c.e * c.r_ball, c.omega, c.zeta * c.r_ball,
                   c.moll_zone, st)
            N.call("axi_soft_penalise_f64", p(w), p(s.u_z), p(s.u_r), p(s.tether_char_func),
                   p(s.u_z_upen), p(s.u_r_upen), nr, nz, dx, c.lam, c.U0, c.omega,
                   p(self.state), st)
            N.call("axi_soft_diffusion_rk2_f64", p(w), p(s.tmp), p(s.R), nr, nz, c.nu, dx,
                   p(self.state), st)
            N.call("axi_soft_advance_f64", p(self.state), st)

    def _launch(self, stream):
        st = ctypes.c_void_p(stream.cuda_stream)
        for k in range(len(self.PARTS)):
            self._part(k, st)

    def phase(self, k, stream=None):
        """Run launch group k of a step (PARTS); all groups in order = one step."""
        s = stream if stream is not None else torch.cuda.current_stream(self.device)
        with torch.cuda.stream(s):
            self._part(k, ctypes.c_void_p(s.cuda_stream))

    # kernel launches of one step: kill (2), solve (4 products), velocity,
    # dt, eta advection, pin, omega advection, mask, extrapolation (prepare,
    # collect, 8 multi-block sweeps of 3 launches, the single-block finisher,
    # fold, copy back), stress, stress mask, div tau + curl (2), tether,
    # penalise (2), diffusion (2), advance
    LAUNCHES_PER_STEP = (2 + 4 + 1 + 1 + 1 + 1 + 1 + 1 + (2 + 3 * 8 + 3) + 1 + 1 + 2 + 1 + 2
                         + 2 + 1)

    def step(self, n=1, stream=None):
        """Advance n steps (asynchronous on `stream`, default torch's current)."""
        s = stream if stream is not None else torch.cuda.current_stream(self.device)
        with torch.cuda.stream(s):
            for _ in range(n):
                self._launch(s)

    def capture(self, steps_per_replay=1):
        """Capture `steps_per_replay` steps into a CUDA graph (replay with replay())."""
        torch.cuda.synchronize(self.device)
        g = torch.cuda.CUDAGraph()
        s = torch.cuda.Stream(self.device)
        with torch.cuda.stream(s):
            with torch.cuda.graph(g, stream=s):
                self.step(steps_per_replay, stream=s)
        torch.cuda.synchronize(self.device)
        self.graph = g
        return g

    def replay(self):
        self.graph.replay()

    @property
    def t(self):
        return float(self.state[SOFT_T])

    @property
    def dt(self):
        return float(self.state[SOFT_DT])

    @property
    def steps(self):
        return int(self.state[SOFT_STEPS])

    def status(self):
        """Sticky status bits (1 << AXI_ERR_*; 0 = healthy)."""
        return int(self.state[SOFT_STATUS:SOFT_STATUS + 1].cpu().numpy().view(np.uint64)[0])

    # the fields, as SoftSphereSimulation names them
    def __getattr__(self, name):
        sim = self.__dict__.get("sim")
        if sim is not None and hasattr(sim, name):
            return getattr(sim, name)
        raise AttributeError(name)
