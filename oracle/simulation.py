"""Per-timestep driver loops of the reference examples, restated for the oracle.

TEST INFRASTRUCTURE ONLY. Each ``*_step`` follows one iteration of a
reference driver loop and takes a ``kern`` namespace holding the kernel
functions, so the same loop runs with the oracle's restated kernels
(``oracle.kernels``) or with the reference's own kernel modules when the
golden vectors are generated.

Cases (sizes and parameters are the caller's):
  * rigid sphere in a uniform stream: examples/FlowPastSphere/flow_past_sphere.py:107-188
  * freely sedimenting rigid sphere: examples/SedimentingRigidSphere/falling_rigid_sphere.py:96-187
  * soft elastic sphere: examples/SoftSphereStreaming/soft_sphere_streaming.py:129-272,
    with the scikit-fmm narrow-band reinitialisation (:196-199) left out: the
    level set is the analytic pinned one (:191-193) in the band and keeps its
    previous value elsewhere (scikit-fmm is not available; parity unpinned
    for that call site).
"""
from dataclasses import dataclass, field

import numpy as np

EPS = np.finfo(float).eps


def grid(nz, nr, dx, z0=0.0, r0=0.0):
    """Cell-centred coordinates as the examples build them
    (examples/FlowPastSphere/flow_past_sphere.py:58-60)."""
    z = np.linspace(z0 + dx / 2, z0 + nz * dx - dx / 2, nz)
    r = np.linspace(r0 + dx / 2, r0 + nr * dx - dx / 2, nr)
    Z, R = np.meshgrid(z, r)
    return z, r, Z, R


@dataclass
class RigidSphereCase:
    nz: int = 512
    nr: int = 256
    dx: float = 1.0 / 256
    z_cm: float = 0.5
    r_sphere: float = 0.0625
    U0: float = 1.0
    Re: float = 100.0
    lam: float = 1e4
    cfl: float = 0.1
    kill_width: int = 3
    ramp: bool = True
    noise: float = 1e-6
    seed: int = 0

    @property
    def nu(self):
        return self.U0 * 2 * self.r_sphere / self.Re

    @property
    def t_ramp(self):
        return 20 * self.r_sphere / self.U0

    @property
    def moll_zone(self):
        return self.dx * 2 ** 0.5


@dataclass
class RigidState:
    vorticity: np.ndarray
    psi: np.ndarray
    u_z: np.ndarray
    u_r: np.ndarray
    char_func: np.ndarray
    t: float = 0.0
    it: int = 0
    dt: float = 0.0
    Cd: float = 0.0
    history: list = field(default_factory=list)


def rigid_sphere_init(case, kern):
    z, r, Z, R = grid(case.nz, case.nr, case.dx)
    rng = np.random.default_rng(case.seed)
    w = case.noise * rng.standard_normal((case.nr, case.nz))
    phi0 = -np.sqrt((Z - case.z_cm) ** 2 + (R - 0.0) ** 2) + case.r_sphere
    chi = 0 * Z
    kern.smooth_Heaviside(chi, phi0, case.moll_zone)
    st = RigidState(vorticity=w, psi=0 * Z, u_z=0 * Z, u_r=0 * Z, char_func=chi)
    return st, (z, r, Z, R)


def rigid_sphere_step(case, st, coords, solver, advect, kern, tmp=None):
    """One iteration of examples/FlowPastSphere/flow_past_sphere.py:107-188."""
    z, r, Z, R = coords
    dx = case.dx
    w = st.vorticity
    kern.kill_boundary_vorticity_sine_z(w, Z, case.kill_width, dx)
    kern.kill_boundary_vorticity_sine_r(w, R, case.kill_width, dx)
    solver.solve(solution_field=st.psi, rhs_field=w)
    kern.compute_velocity_from_psi_unb(st.u_z, st.u_r, st.psi, R, dx)
    prefac = 1.0
    if case.ramp and st.t < case.t_ramp:
        prefac = np.sin(0.5 * np.pi * st.t / case.t_ramp)
    st.u_z[...] += case.U0 * prefac
    dt = min(0.9 * dx ** 2 / 4 / case.nu,
             case.cfl * dx / (np.amax(np.fabs(st.u_z) + np.fabs(st.u_r)) + EPS))
    u_z_upen = st.u_z.copy()
    u_r_upen = st.u_r.copy()
    kern.brinkmann_penalize(case.lam, dt, st.char_func, 0.0, 0.0, u_z_upen, u_r_upen,
                            st.u_z, st.u_r)
    penal = np.zeros_like(w)
    kern.compute_vorticity_from_velocity_unb(penal, st.u_z - u_z_upen, st.u_r - u_r_upen, dx)
    w[...] += penal
    st.Cd = (2 * 2 * np.pi * dx * dx * case.lam * np.sum(R * st.char_func * st.u_z)
             / (np.pi * case.r_sphere ** 2))
    advect(w, st.u_z, st.u_r, dt)
    if tmp is None:
        tmp = np.zeros_like(w)
    kern.diffusion_RK2_unb(w, tmp, R, case.nu, dt, dx)
    st.dt = dt
    st.t += dt
    st.it += 1
    return st


@dataclass
class SedimentingCase:
    """examples/SedimentingRigidSphere/falling_rigid_sphere.py:24-79 defaults."""
    nz: int = 512
    nr: int = 128
    dx: float = 1.0 / 512
    z_cm: float = 0.6
    r_sphere: float = 0.025
    rho_f: float = 1.0
    rho_s: float = 1.1
    nu: float = 0.01
    lam: float = 1e4
    cfl: float = 0.1
    kill_width: int = 3
    gravity: float = 9.81

    @property
    def moll_zone(self):
        return self.dx * 2 ** 0.5


@dataclass
class SedimentingState:
    vorticity: np.ndarray
    psi: np.ndarray
    u_z: np.ndarray
    u_r: np.ndarray
    char_func: np.ndarray
    part_mass: float
    part_vol: float
    U_z_cm_part: float = 0.0
    part_Z_cm: float = 0.0
    diff: float = 0.0
    F_total: float = 0.0
    Cd: float = 0.0
    t: float = 0.0
    it: int = 0
    dt: float = 0.0


def sedimenting_init(case, kern, vorticity=None):
    z, r, Z, R = grid(case.nz, case.nr, case.dx)
    phi0 = -np.sqrt((Z - case.z_cm) ** 2 + (R - 0.0) ** 2) + case.r_sphere
    chi = 0 * Z
    kern.smooth_Heaviside(chi, phi0, case.moll_zone)
    dx = case.dx
    part_mass = 2 * np.pi * dx * dx * case.rho_s * np.sum(chi * R)
    part_vol = 2 * np.pi * dx * dx * np.sum(chi * R)
    w = 0 * Z if vorticity is None else vorticity.copy()
    st = SedimentingState(vorticity=w, psi=0 * Z, u_z=0 * Z, u_r=0 * Z, char_func=chi,
                          part_mass=part_mass, part_vol=part_vol, part_Z_cm=case.z_cm)
    return st, (z, r, Z, R)


def sedimenting_step(case, st, coords, solver, advect, kern, tmp=None):
    """One iteration of examples/SedimentingRigidSphere/falling_rigid_sphere.py:96-187."""
    z, r, Z, R = coords
    dx = case.dx
    g = (case.rho_s - case.rho_f) * case.gravity
    w = st.vorticity
    kern.kill_boundary_vorticity_sine_z(w, Z, case.kill_width, dx)
    kern.kill_boundary_vorticity_sine_r(w, R, case.kill_width, dx)
    solver.solve(solution_field=st.psi, rhs_field=w)
    kern.compute_velocity_from_psi_unb(st.u_z, st.u_r, st.psi, R, dx)
    dt = min(0.9 * dx ** 2 / 4 / case.nu,
             case.cfl * dx / (np.amax(np.fabs(st.u_z) + np.fabs(st.u_r)) + EPS))
    u_z_upen = st.u_z.copy()
    u_r_upen = st.u_r.copy()
    kern.brinkmann_penalize(case.lam, dt, st.char_func, st.U_z_cm_part, 0.0,
                            u_z_upen, u_r_upen, st.u_z, st.u_r)
    penal = np.zeros_like(w)
    kern.compute_vorticity_from_velocity_unb(penal, st.u_z - u_z_upen, st.u_r - u_r_upen, dx)
    w[...] += penal
    F_pen, F_un = kern.compute_force_on_body(R, st.char_func, case.rho_f, case.lam, st.u_z,
                                             st.U_z_cm_part, st.part_vol, dt, st.diff)
    F_total = 2 * np.pi * dx * dx * F_pen + F_un
    phi0 = -np.sqrt((Z - st.part_Z_cm) ** 2 + (R - 0.0) ** 2) + case.r_sphere
    kern.smooth_Heaviside(st.char_func, phi0, case.moll_zone)
    advect(w, st.u_z, st.u_r, dt)
    if tmp is None:
        tmp = np.zeros_like(w)
    kern.diffusion_RK2_unb(w, tmp, R, case.nu, dt, dx)
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


@dataclass
class SoftSphereCase:
    """Soft neo-Hookean sphere (examples/SoftSphereStreaming/soft_sphere_streaming.py:31-63),
    driven by a penalised forcing region (a tether sphere moving with the
    oscillation, as in the example)."""
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


@dataclass
class SoftState:
    vorticity: np.ndarray
    psi: np.ndarray
    u_z: np.ndarray
    u_r: np.ndarray
    eta1: np.ndarray
    eta2: np.ndarray
    ball_phi: np.ndarray
    ball_char_func: np.ndarray
    tether_char_func: np.ndarray
    t: float = 0.0
    it: int = 0
    dt: float = 0.0


def soft_sphere_init(case, kern):
    z, r, Z, R = grid(case.nz, case.nr, case.dx)
    phi = -np.sqrt((Z - case.z_cm) ** 2 + R ** 2) + case.r_ball
    chi = 0 * Z
    kern.smooth_Heaviside(chi, phi, case.moll_zone)
    tphi = -np.sqrt((Z - case.z_cm) ** 2 + R ** 2) + case.zeta * case.r_ball
    tchi = 0 * Z
    kern.smooth_Heaviside(tchi, tphi, case.moll_zone)
    st = SoftState(vorticity=0 * Z, psi=0 * Z, u_z=0 * Z, u_r=0 * Z, eta1=Z.copy(),
                   eta2=R.copy(), ball_phi=phi, ball_char_func=chi, tether_char_func=tchi)
    return st, (z, r, Z, R)


def soft_sphere_step(case, st, coords, solver, advect_w, advect_eta, kern):
    """One iteration of examples/SoftSphereStreaming/soft_sphere_streaming.py:129-272
    (no plotting / averaging, no scikit-fmm reinitialisation)."""
    z, r, Z, R = coords
    dx = case.dx
    nr = case.nr
    w = st.vorticity
    kern.kill_boundary_vorticity_sine_z(w, Z, case.kill_width, dx)
    kern.kill_boundary_vorticity_sine_r(w, R, case.kill_width, dx)
    solver.solve(solution_field=st.psi, rhs_field=w)
    kern.compute_velocity_from_psi_unb(st.u_z, st.u_r, st.psi, R, dx)
    dt = min(case.cfl * dx / np.sqrt(case.G / case.rho_f),
             case.cfl * dx / (np.amax(np.fabs(st.u_z) + np.fabs(st.u_r)) + EPS),
             0.9 * dx ** 2 / 4 / case.nu)
    advect_eta(st.eta1, st.eta2, st.u_z, st.u_r, dt)
    phi_orig = -np.sqrt((st.eta1 - case.z_cm) ** 2 + (st.eta2 - 0.0) ** 2) + case.r_ball
    band = np.where(st.ball_phi > -3 * dx)
    st.ball_phi[band] = phi_orig[band]
    advect_w(w, st.u_z, st.u_r, dt)
    kern.smooth_Heaviside(st.ball_char_func, st.ball_phi, case.moll_zone)
    inside_solid = st.ball_char_func > 0.5
    nzd = 2 * nr
    zd = np.linspace(dx / 2, nzd * dx - dx / 2, nzd) if nzd > case.nz else z
    phi_d = np.zeros((2 * nr, case.nz))
    e1_d = np.zeros((2 * nr, case.nz))
    e2_d = np.zeros((2 * nr, case.nz))
    kern.extrapolate_eta_with_least_squares(inside_solid, st.ball_phi, st.eta1, st.eta2,
                                            phi_d, e1_d, e2_d, case.extrap_zone, nr, zd)
    s11, s12, s22 = (np.zeros_like(w) for _ in range(3))
    e1z, e1r, e2z, e2r = (np.zeros_like(w) for _ in range(4))
    kern.solid_sigma(s11, s12, s22, case.G, dx, st.eta1, st.eta2, e1z, e1r, e2z, e2r)
    s11[...] = st.ball_char_func * s11
    s12[...] = st.ball_char_func * s12
    s22[...] = st.ball_char_func * s22
    tau_z = np.zeros_like(w)
    tau_r = np.zeros_like(w)
    kern.update_vorticity_from_solid_stress(w, tau_z, tau_r, s11, s12, s22, R, dt, dx)
    z_cm_t = case.z_cm + case.e * case.r_ball * np.sin(case.omega * st.t)
    tphi = -np.sqrt((Z - z_cm_t) ** 2 + (R - 0.0) ** 2) + case.zeta * case.r_ball
    kern.smooth_Heaviside(st.tether_char_func, tphi, case.moll_zone)
    u_z_upen = st.u_z.copy()
    u_r_upen = st.u_r.copy()
    kern.brinkmann_penalize(case.lam, dt, st.tether_char_func,
                            case.U0 * np.cos(case.omega * st.t), 0.0,
                            u_z_upen, u_r_upen, st.u_z, st.u_r)
    penal = np.zeros_like(w)
    kern.compute_vorticity_from_velocity_unb(penal, st.u_z - u_z_upen, st.u_r - u_r_upen, dx)
    w[...] += penal
    tmp = np.zeros_like(w)
    kern.diffusion_RK2_unb(w, tmp, R, case.nu, dt, dx)
    st.dt = dt
    st.t += dt
    st.it += 1
    return st
