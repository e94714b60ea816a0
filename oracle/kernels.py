"""Numpy restatement of the PyAxisymFlow per-timestep kernels (the oracle).

TEST INFRASTRUCTURE ONLY (see ``oracle/__init__.py``). Every function keeps
the reference's argument order, in-place semantics and elementwise operation
order, and cites the reference file:line it restates. Paths are relative to
the PyAxisymFlow project root.

Deviation kept on purpose: ``numpy.linalg.eig`` in numpy >= 2 returns complex
arrays even when every imaginary part is zero, while the numpy the reference
pins (``pyproject.toml``: numpy ^1.20) returned real arrays in that case. The
oracle follows the pinned behaviour (real eigenbases) and asserts that the
imaginary parts it drops are exactly zero.
"""
import numpy as np

NEUMANN_ZR = "homogenous_neumann_along_z_and_r"
NEUMANN_R_PERIODIC_Z = "homogenous_neumann_along_r_and_periodic_along_z"
DIRICHLET_R_PERIODIC_Z = "homogenous_dirichlet_along_r_and_periodic_along_z"

# pystencils' create_kernel(ghost_layers=None) skips max|offset| cells at every
# border of every axis; all four ENO3 flux kernels touch offsets up to 2
# (pyaxisymflow/pyst_kernels/advection_flux.py:32-44, 61-73, 88-100, 115-127),
# so fluxes are only written on [2:-2, 2:-2] of the mirrored buffer.
ENO3_GHOST_LAYERS = 2


def _real(a):
    if np.iscomplexobj(a):
        if np.any(a.imag != 0):
            raise ValueError("eigen decomposition has a non-zero imaginary part")
        return np.ascontiguousarray(a.real)
    return a


def _eig_sorted_desc(mat):
    # FastDiagonalisationStokesSolver.py:109-113 (eig, then descending sort)
    vals, vecs = np.linalg.eig(mat)
    idx = vals.argsort()[::-1]
    vals = vals[idx]
    vecs = vecs[:, idx]
    return _real(vals), _real(vecs)


def _tridiag(n, lo, d, up):
    m = np.zeros((n, n))
    i = np.arange(n)
    m[i, i] = d
    m[i[1:], i[:-1]] = lo
    m[i[:-1], i[1:]] = up
    return m


class _FastDiagonalisationBase:
    """Shared eigenbasis engine of the three spectral solvers."""

    def _radial_coord(self, dx, nr):
        # FastDiagonalisationStokesSolver.py:20-24
        return np.linspace(dx / 2, nr * dx - dx / 2, nr).reshape(nr, 1)

    def _finish(self, eig_vals_r, eig_vecs_r, eig_vals_z, eig_vecs_z, spectrum):
        self.eig_vecs_r = eig_vecs_r
        self.inv_of_eig_vecs_r = np.linalg.inv(eig_vecs_r)
        self.tranpose_of_eig_vecs_z = np.ascontiguousarray(eig_vecs_z.T)
        self.tranpose_of_inv_of_eig_vecs_z = np.ascontiguousarray(
            np.linalg.inv(eig_vecs_z).T
        )
        self.eig_vals_r = eig_vals_r
        self.eig_vals_z = eig_vals_z
        self.inv_eig_val_matrix = 1.0 / spectrum
        self.spectral_field_buffer = np.zeros_like(self.inv_eig_val_matrix)

    def _transform(self, rhs):
        # FastDiagonalisationStokesSolver.py:137-156: multi_dot of three
        # equally costed factors evaluates A @ (B @ C)
        buf = self.inv_of_eig_vecs_r @ (rhs @ self.tranpose_of_inv_of_eig_vecs_z)
        buf *= self.inv_eig_val_matrix
        return self.eig_vecs_r @ (buf @ self.tranpose_of_eig_vecs_z)


class FastDiagonalisationStokesSolver(_FastDiagonalisationBase):
    """Restates kernels/FastDiagonalisationStokesSolver.py:6-156."""

    def __init__(self, grid_size_r, grid_size_z, dx, real_dtype=np.float64,
                 bc_type=NEUMANN_ZR):
        self.dx = dx
        self.grid_size_r = grid_size_r
        self.grid_size_z = grid_size_z
        self.bc_type = bc_type
        self.radial_coord = self._radial_coord(dx, grid_size_r)
        inv_dx2 = 1 / dx / dx
        inv_2dx = 1 / 2 / dx
        nz, nr = grid_size_z, grid_size_r
        # construct_fdm_matrices :41-67
        pz = _tridiag(nz, -inv_dx2, 2 * inv_dx2, -inv_dx2)
        pr = _tridiag(nr, -inv_dx2, 2 * inv_dx2, -inv_dx2)
        dr = _tridiag(nr, inv_2dx, 0.0, -inv_2dx)
        dr = dr / self.radial_coord
        # apply_boundary_conds_to_poisson_matrices :69-97
        if bc_type == NEUMANN_ZR:
            pz[0, 0] = inv_dx2
            pz[-1, -1] = inv_dx2
            pr[-1, -1] = inv_dx2
            dr[-1, -2] = 0
        elif bc_type == NEUMANN_R_PERIODIC_Z:
            pz[0, -1] = pz[0, 1]
            pz[-1, 0] = pz[-1, -2]
            pr[-1, -1] = inv_dx2
            dr[-1, -2] = 0
        elif bc_type == DIRICHLET_R_PERIODIC_Z:
            pz[0, -1] = pz[0, 1]
            pz[-1, 0] = pz[-1, -2]
        # compute_spectral_decomp_of_poisson_matrices :99-128
        vr, er = _eig_sorted_desc(pr - dr)
        vz, ez = _eig_sorted_desc(pz)
        self._finish(vr, er, vz, ez, vz.reshape(1, nz) + vr.reshape(nr, 1))

    def solve(self, solution_field, rhs_field):
        # :130-156
        solution_field[...] = self._transform(rhs_field * self.radial_coord)


class FastDiagonalisationPotentialSolver(_FastDiagonalisationBase):
    """Restates kernels/FastDiagonalisationPotentialSolver.py:6-145."""

    def __init__(self, grid_size_r, grid_size_z, dx, real_dtype=np.float64,
                 bc_type=NEUMANN_ZR):
        self.dx = dx
        self.grid_size_r = grid_size_r
        self.grid_size_z = grid_size_z
        self.bc_type = bc_type
        self.radial_coord = self._radial_coord(dx, grid_size_r)
        inv_dx2 = 1 / dx / dx
        inv_2dx = 1 / 2 / dx
        nz, nr = grid_size_z, grid_size_r
        # :41-67
        pz = _tridiag(nz, inv_dx2, -2 * inv_dx2, inv_dx2)
        pr = _tridiag(nr, inv_dx2, -2 * inv_dx2, inv_dx2)
        dr = _tridiag(nr, -inv_2dx, 0.0, inv_2dx) / self.radial_coord
        # :69-86
        if bc_type == NEUMANN_ZR:
            pz[0, 0] = -inv_dx2
            pz[-1, -1] = -inv_dx2
            pr[-1, -1] = -inv_dx2
            dr[-1, -2] = 0
        # :88-117
        vr, er = _eig_sorted_desc(pr + dr)
        vz, ez = _eig_sorted_desc(pz)
        self._finish(vr, er, vz, ez, vz.reshape(1, nz) + vr.reshape(nr, 1))

    def solve(self, solution_field, rhs_field):
        # :119-145
        solution_field[...] = self._transform(rhs_field)


class ImplicitEulerDiffusionStepper(_FastDiagonalisationBase):
    """Restates kernels/implicit_diffusion_solver.py:6-143."""

    def __init__(self, time_step, kinematic_viscosity, grid_size_r, grid_size_z,
                 dx, real_dtype=np.float64):
        self.time_step = time_step
        self.nu_times_dt = time_step * kinematic_viscosity
        self.dx = dx
        self.grid_size_r = grid_size_r
        self.grid_size_z = grid_size_z
        self.radial_coord = self._radial_coord(dx, grid_size_r)
        r = self.radial_coord
        inv_dx2 = 1 / dx / dx
        inv_2dx = 1 / 2 / dx
        nz, nr = grid_size_z, grid_size_r
        # :40-72
        pz = _tridiag(nz, inv_dx2, -2 * inv_dx2, inv_dx2)
        pr = _tridiag(nr, inv_dx2, -2 * inv_dx2, inv_dx2)
        npr = _tridiag(nr, -inv_2dx, 0.0, inv_2dx)
        npr = npr / r - np.identity(nr) / (r ** 2)
        # :74-106
        vr, er = _eig_sorted_desc(pr + npr)
        vz, ez = _eig_sorted_desc(pz)
        spectrum = 1.0 - self.nu_times_dt * (vz.reshape(1, nz) + vr.reshape(nr, 1))
        self._finish(vr, er, vz, ez, spectrum)

    def step(self, vorticity_field, dt):
        # :108-143
        if dt != self.time_step:
            raise ValueError(
                "dt should be constant throughout the simulation if using "
                "implicit diffusion! Please use the value of dt being used "
                "to initialize the implicit diffusion stepper"
            )
        vorticity_field[...] = self._transform(vorticity_field)


# --------------------------------------------------------------------------
# pointwise / stencil kernels
# --------------------------------------------------------------------------

def compute_velocity_from_psi_unb(u_z, u_r, psi, R, dx):
    """kernels/compute_velocity_from_psi.py:4-17."""
    u_z[1:-1, :] = (psi[2:, :] - psi[:-2, :]) / (2 * dx) / R[1:-1, :]
    u_z[0, :] = (-psi[2, :] + 4 * psi[1, :] - 3 * psi[0, :]) / (2 * dx) / R[0, :]
    u_z[-1, :] = (psi[-3, :] - 4 * psi[-2, :] + 3 * psi[-1, :]) / (2 * dx) / R[-1, :]
    u_r[:, 1:-1] = -(psi[:, 2:] - psi[:, :-2]) / (2 * dx) / R[:, 1:-1]
    u_r[:, 0] = -(-psi[:, 2] + 4 * psi[:, 1] - 3 * psi[:, 0]) / (2 * dx) / R[:, 0]
    u_r[:, -1] = -(psi[:, -3] - 4 * psi[:, -2] + 3 * psi[:, -1]) / (2 * dx) / R[:, -1]


def compute_velocity_from_psi_periodic(u_z, u_r, psi, R, dx, per_communicator):
    """kernels/compute_velocity_from_psi.py:20-34."""
    per_communicator(psi)
    compute_velocity_from_psi_unb(u_z, u_r, psi, R, dx)


def compute_vorticity_from_velocity_unb(vort, u_z, u_r, dx):
    """kernels/compute_vorticity_from_velocity.py:4-13."""
    vort[1:-1, 1:-1] = (u_r[1:-1, 2:] - u_r[1:-1, :-2]) / (2 * dx) - (
        u_z[2:, 1:-1] - u_z[:-2, 1:-1]
    ) / (2 * dx)


def compute_vorticity_from_velocity_periodic(vort, u_z, u_r, dx, per_communicator):
    """kernels/compute_vorticity_from_velocity.py:16-28."""
    per_communicator(u_r)
    per_communicator(u_z)
    compute_vorticity_from_velocity_unb(vort, u_z, u_r, dx)


def brinkmann_penalize(lam, dt, char_func, U_z, U_r, grid_u_z, grid_u_r,
                       penalized_u_z, penalized_u_r):
    """kernels/brinkmann_penalize.py:4-16."""
    penalized_u_z[...] = (grid_u_z + lam * dt * char_func * U_z) / (
        1 + lam * dt * char_func
    )
    penalized_u_r[...] = (grid_u_r + lam * dt * char_func * U_r) / (
        1 + lam * dt * char_func
    )


def smooth_Heaviside(H, phi, blend_w):
    """kernels/smooth_Heaviside.py:5-14."""
    H[...] = 0 * H
    H[...] = H + (phi >= blend_w)
    H[...] = H + (np.fabs(phi) < blend_w) * 0.5 * (
        1 + phi / blend_w + np.sin(np.pi * phi / blend_w) / np.pi
    )


def kill_boundary_vorticity_sine_z(vorticity, Z, width, dx):
    """kernels/kill_boundary_vorticity_sine.py:4-14 (literal ``1 - Z``)."""
    vorticity[:, :width] = np.sin(
        np.pi * (Z[:, :width] - 0.5 * dx) / 2 / (width - 1) / dx
    ) * vorticity[:, (width - 1)].reshape(-1, 1)
    vorticity[:, -width:] = np.sin(
        np.pi * (1 - Z[:, -width:] - 0.5 * dx) / 2 / (width - 1) / dx
    ) * vorticity[:, -width].reshape(-1, 1)


def kill_boundary_vorticity_sine_r(vorticity, R, width, dx):
    """kernels/kill_boundary_vorticity_sine.py:17-27 (literal ``1 - R``)."""
    vorticity[-width:, :] = (
        np.sin(np.pi * (1 - R[-width:, :] - 0.5 * dx) / 2 / (width - 1) / dx)
        * vorticity[-width, :]
    )
    vorticity[0, :] = 0.0


def _rk2_operator(w, R, dx):
    # kernels/diffusion_RK2.py:15-25 (the bracketed operator)
    return (
        (w[2:, 1:-1] + w[:-2, 1:-1] + w[1:-1, 2:] + w[1:-1, :-2] - 4 * w[1:-1, 1:-1])
        / (dx ** 2)
        + (w[2:, 1:-1] - w[:-2, 1:-1]) / (2 * dx) / R[1:-1, 1:-1]
        - w[1:-1, 1:-1] * (R[1:-1, 1:-1] ** -2)
    )


def diffusion_RK2_unb(vorticity, temp_vorticity, R, nu, dt, dx):
    """kernels/diffusion_RK2.py:4-44."""
    temp_vorticity[...] = vorticity
    temp_vorticity[1:-1, 1:-1] += 0.5 * nu * dt * _rk2_operator(vorticity, R, dx)
    vorticity[1:-1, 1:-1] += nu * dt * _rk2_operator(temp_vorticity, R, dx)


def diffusion_RK2_periodic(vorticity, temp_vorticity, R, nu, dt, dx, per_communicator):
    """kernels/diffusion_RK2.py:47-89."""
    per_communicator(vorticity)
    temp_vorticity[...] = vorticity
    temp_vorticity[1:-1, 1:-1] += 0.5 * nu * dt * _rk2_operator(vorticity, R, dx)
    per_communicator(temp_vorticity)
    vorticity[1:-1, 1:-1] += nu * dt * _rk2_operator(temp_vorticity, R, dx)


def gen_periodic_boundary_ghost_comm(ghost_size):
    """kernels/periodic_boundary_ghost_comm.py:4-15."""
    assert ghost_size > 0 and isinstance(ghost_size, int), "invalid ghost size"

    def periodic_boundary_ghost_comm(field):
        field[:, :ghost_size] = field[:, -2 * ghost_size: -ghost_size]
        field[:, -ghost_size:] = field[:, ghost_size: 2 * ghost_size]

    return periodic_boundary_ghost_comm


def gen_periodic_boundary_ghost_comm_eta(ghost_size, Z_max, dx):
    """kernels/periodic_boundary_ghost_comm.py:18-33."""
    assert ghost_size > 0 and isinstance(ghost_size, int), "invalid ghost size"

    def periodic_boundary_ghost_comm(field):
        field[:, :ghost_size] = (
            field[:, -2 * ghost_size: -ghost_size] - Z_max + 2 * ghost_size * dx
        )
        field[:, -ghost_size:] = (
            field[:, ghost_size: 2 * ghost_size] + Z_max - 2 * ghost_size * dx
        )

    return periodic_boundary_ghost_comm


def compute_force_on_body(R, part_char_func, rho_f, brink_lam, u_z, U_z_cm_part,
                          part_vol, dt, diff):
    """kernels/compute_forces.py:4-17."""
    F_pen = rho_f * brink_lam * np.sum(R * part_char_func * (u_z - U_z_cm_part))
    F_un = (diff * part_vol) / dt
    return F_pen, F_un


def force_projection(rho_s, char_func, u_z, u_r, R):
    """kernels/force_projection.py:5-15."""
    U_z = np.sum(rho_s * char_func * u_z * R) / np.sum(rho_s * char_func * R)
    U_r = np.sum(rho_s * char_func * u_r * R) / np.sum(rho_s * char_func * R)
    return U_z, U_r


# --------------------------------------------------------------------------
# ENO3 advection (pystencils kernels restated)
# --------------------------------------------------------------------------

def _eno3_face_conservative(fm1, f0, f1, f2, um1, u0, u1, u2):
    """Upwinded 3rd-order face value of f*u between cells 0 and 1.

    pyaxisymflow/pyst_kernels/advection_flux.py:32-44 (x_front); x_back
    (:61-73) is the same face seen from the right cell, so the selector
    ``u[0] > -u[1]`` and both branches coincide term by term.
    """
    left = (1 / 3) * f1 * u1 + (5 / 6) * f0 * u0 - (1 / 6) * fm1 * um1
    right = (1 / 3) * f0 * u0 + (5 / 6) * f1 * u1 - (1 / 6) * f2 * u2
    return np.where(u0 > -u1, left, right)


def _eno3_face_non_conservative(fm1, f0, f1, f2, u0, u1):
    """Upwinded 3rd-order face value of f (no velocity inside).

    pyaxisymflow/pyst_kernels/advection_flux.py:189-202 (front) and
    :219-236 (back). The trailing ``* velocity[0, 0]`` uses the velocity of
    the cell being updated, so it is applied by the caller.
    """
    left = (1 / 3) * f1 + (5 / 6) * f0 - (1 / 6) * fm1
    right = (1 / 3) * f0 + (5 / 6) * f1 - (1 / 6) * f2
    return np.where(u0 > -u1, left, right)


def advection_timestep_euler_forward_eno3(field, velocity, dt_by_dx, conservative):
    """One Euler-forward ENO3 advection step of a 2-D field, in place.

    pyaxisymflow/pyst_kernels/advection_timestep.py:37-54 (conservative) and
    :85-102 (non-conservative): flux = 0; flux += a*F_x_front; flux -=
    a*F_x_back; flux += a*F_y_front; flux -= a*F_y_back with a = -dt/dx, all on
    the interior [2:-2, 2:-2] (pystencils ghost layers); then field += flux over
    the whole array. Axis 1 is "x" (velocity[0]), axis 0 is "y" (velocity[1]).
    """
    g = ENO3_GHOST_LAYERS
    n0, n1 = field.shape
    a = -dt_by_dx
    flux = np.zeros_like(field)
    f = field
    ux, uy = velocity[0], velocity[1]
    s0 = slice(g, n0 - g)
    s1 = slice(g, n1 - g)

    def sh(arr, d0, d1):
        return arr[g + d0: n0 - g + d0, g + d1: n1 - g + d1]

    inner = flux[s0, s1]
    if conservative:
        xf = _eno3_face_conservative(sh(f, 0, -1), sh(f, 0, 0), sh(f, 0, 1), sh(f, 0, 2),
                                     sh(ux, 0, -1), sh(ux, 0, 0), sh(ux, 0, 1), sh(ux, 0, 2))
        xb = _eno3_face_conservative(sh(f, 0, -2), sh(f, 0, -1), sh(f, 0, 0), sh(f, 0, 1),
                                     sh(ux, 0, -2), sh(ux, 0, -1), sh(ux, 0, 0), sh(ux, 0, 1))
        yf = _eno3_face_conservative(sh(f, -1, 0), sh(f, 0, 0), sh(f, 1, 0), sh(f, 2, 0),
                                     sh(uy, -1, 0), sh(uy, 0, 0), sh(uy, 1, 0), sh(uy, 2, 0))
        yb = _eno3_face_conservative(sh(f, -2, 0), sh(f, -1, 0), sh(f, 0, 0), sh(f, 1, 0),
                                     sh(uy, -2, 0), sh(uy, -1, 0), sh(uy, 0, 0), sh(uy, 1, 0))
        inner[...] = inner + a * xf
        inner[...] = inner - a * xb
        inner[...] = inner + a * yf
        inner[...] = inner - a * yb
    else:
        # advection_flux.py:189-202: advection_flux + inv_dx * (face) * velocity[0, 0]
        u0x = sh(ux, 0, 0)
        u0y = sh(uy, 0, 0)
        xf = _eno3_face_non_conservative(sh(f, 0, -1), sh(f, 0, 0), sh(f, 0, 1), sh(f, 0, 2),
                                         u0x, sh(ux, 0, 1))
        xb = _eno3_face_non_conservative(sh(f, 0, -2), sh(f, 0, -1), sh(f, 0, 0), sh(f, 0, 1),
                                         sh(ux, 0, -1), u0x)
        yf = _eno3_face_non_conservative(sh(f, -1, 0), sh(f, 0, 0), sh(f, 1, 0), sh(f, 2, 0),
                                         u0y, sh(uy, 1, 0))
        yb = _eno3_face_non_conservative(sh(f, -2, 0), sh(f, -1, 0), sh(f, 0, 0), sh(f, 1, 0),
                                         sh(uy, -1, 0), u0y)
        inner[...] = inner + (a * xf) * u0x
        inner[...] = inner - (a * xb) * u0x
        inner[...] = inner + (a * yf) * u0y
        inner[...] = inner - (a * yb) * u0y
    field[...] = field + flux


def _mirror(field, grid_size_r, parity):
    # kernels/advect_vorticity_via_eno3.py:28-33: lower half = parity * flip
    doubled = np.zeros((2 * grid_size_r, field.shape[1]))
    doubled[grid_size_r:, :] = field
    doubled[:grid_size_r, :] = parity * np.flip(field, axis=0)
    return doubled


def gen_advect_vorticity_via_eno3(dx, grid_size_r, grid_size_z, real_t=np.float64,
                                  num_threads=False):
    """kernels/advect_vorticity_via_eno3.py:8-44."""

    def advect_vorticity_via_eno3(vorticity, u_z, u_r, dt):
        u_double = np.stack([_mirror(u_z, grid_size_r, 1.0), _mirror(u_r, grid_size_r, -1.0)])
        vd = _mirror(vorticity, grid_size_r, -1.0)
        advection_timestep_euler_forward_eno3(vd, u_double, dt / dx, conservative=True)
        vorticity[...] = vd[grid_size_r:, :]

    return advect_vorticity_via_eno3


def gen_advect_vorticity_via_eno3_periodic(dx, grid_size_r, grid_size_z, per_communicator,
                                           real_t=np.float64, num_threads=False):
    """kernels/advect_vorticity_via_eno3.py:47-91."""
    inner = gen_advect_vorticity_via_eno3(dx, grid_size_r, grid_size_z)

    def advect_vorticity_via_eno3_periodic(vorticity, u_z, u_r, dt):
        per_communicator(u_z)
        per_communicator(u_r)
        per_communicator(vorticity)
        inner(vorticity, u_z, u_r, dt)

    return advect_vorticity_via_eno3_periodic


def gen_advect_refmap_via_eno3(dx, grid_size_r, grid_size_z, real_t=np.float64,
                               num_threads=False):
    """elasto_kernels/advect_refmap_via_eno3.py:8-54 (eta1 even, eta2 odd)."""

    def advect_refmap_via_eno3(eta1, eta2, u_z, u_r, dt):
        u_double = np.stack([_mirror(u_z, grid_size_r, 1.0), _mirror(u_r, grid_size_r, -1.0)])
        e1 = _mirror(eta1, grid_size_r, 1.0)
        advection_timestep_euler_forward_eno3(e1, u_double, dt / dx, conservative=False)
        eta1[...] = e1[grid_size_r:, :]
        e2 = _mirror(eta2, grid_size_r, -1.0)
        advection_timestep_euler_forward_eno3(e2, u_double, dt / dx, conservative=False)
        eta2[...] = e2[grid_size_r:, :]

    return advect_refmap_via_eno3


def gen_advect_refmap_via_eno3_periodic(dx, grid_size_r, grid_size_z, per_communicator1,
                                        per_communicator2, real_t=np.float64,
                                        num_threads=False):
    """elasto_kernels/advect_refmap_via_eno3.py:57-115."""
    inner = gen_advect_refmap_via_eno3(dx, grid_size_r, grid_size_z)

    def advect_refmap_via_eno3_periodic(eta1, eta2, u_z, u_r, dt):
        per_communicator1(u_z)
        per_communicator1(u_r)
        per_communicator2(eta1)
        per_communicator1(eta2)
        inner(eta1, eta2, u_z, u_r, dt)

    return advect_refmap_via_eno3_periodic


# --------------------------------------------------------------------------
# elasto kernels
# --------------------------------------------------------------------------

def solid_sigma(sigma_s_11, sigma_s_12, sigma_s_22, G, dx, eta_1, eta_2,
                eta_1z, eta_1r, eta_2z, eta_2r):
    """elasto_kernels/solid_sigma.py:4-29."""
    eta_1z[:, 1:-1] = (eta_1[:, 2:] - eta_1[:, :-2]) / (2 * dx)
    eta_2z[:, 1:-1] = (eta_2[:, 2:] - eta_2[:, :-2]) / (2 * dx)
    eta_1r[1:-1, 1:-1] = (eta_1[2:, 1:-1] - eta_1[:-2, 1:-1]) / (2 * dx)
    eta_1r[0, :] = (-eta_1[2, :] + 4 * eta_1[1, :] - 3 * eta_1[0, :]) / (2 * dx)
    eta_2r[1:-1, 1:-1] = (eta_2[2:, 1:-1] - eta_2[:-2, 1:-1]) / (2 * dx)
    eta_2r[0, :] = (-eta_2[2, :] + 4 * eta_2[1, :] - 3 * eta_2[0, :]) / (2 * dx)
    sigma_s_12[...] = -G * (eta_1z * eta_1r + eta_2z * eta_2r)
    sigma_s_11[...] = (0.5 * G) * (eta_1r ** 2 + eta_2r ** 2 - eta_1z ** 2 - eta_2z ** 2)
    sigma_s_22[...] = -sigma_s_11


def update_vorticity_from_solid_stress(vorticity, tau_z, tau_r, tau11, tau12, tau22,
                                       R, dt, dx):
    """elasto_kernels/div_tau.py:4-34."""
    tau_z[1:-1, 1:-1] = (
        tau11[1:-1, 2:] - tau11[1:-1, :-2] + tau12[2:, 1:-1] - tau12[:-2, 1:-1]
    ) / (2 * dx) + tau12[1:-1, 1:-1] / R[1:-1, 1:-1]
    tau_z[0, 1:-1] = (
        tau11[0, 2:] - tau11[0, :-2] - tau12[2, 1:-1] + 4 * tau12[1, 1:-1]
        - 3 * tau12[0, 1:-1]
    ) / (2 * dx) + tau12[0, 1:-1] / R[0, 1:-1]
    tau_r[1:-1, 1:-1] = (
        tau12[1:-1, 2:] - tau12[1:-1, :-2] + tau22[2:, 1:-1] - tau22[:-2, 1:-1]
    ) / (2 * dx) + tau22[1:-1, 1:-1] / R[1:-1, 1:-1]
    tau_r[0, 1:-1] = (
        tau12[0, 2:] - tau12[0, :-2] - tau22[2, 1:-1] + 4 * tau22[1, 1:-1]
        - 3 * tau22[0, 1:-1]
    ) / (2 * dx) + tau22[0, 1:-1] / R[0, 1:-1]
    vorticity[1:-1, 1:-1] += (
        dt * (tau_r[1:-1, 2:] - tau_r[1:-1, :-2] - tau_z[2:, 1:-1] + tau_z[:-2, 1:-1])
        / (2 * dx)
    )


# --------------------------------------------------------------------------
# least-squares eta extrapolation (core/src/extrapolate_using_least_squares.hpp)
# --------------------------------------------------------------------------

def _c_int_abs(x):
    # The reference calls unqualified ``abs`` on a double, which resolves to
    # C ``int abs(int)``: the argument is truncated toward zero first.
    return float(abs(int(x)))


def gauss_elimination(A, n_coeffs, n_components):
    """core/src/lstsq/least_squares.hpp:10-59: partial pivoting, in place.

    ``A`` is (n_coeffs, n_coeffs + n_components); returns sol[comp][coeff].
    Pivot search (:311-320) compares ``abs(A[k][i]) > max_element`` with the
    integer ``abs`` (truncated magnitudes), and stores ``std::abs`` of the new
    maximum; this is restated exactly, so the row choice matches bit for bit.
    """
    A = np.array(A, dtype=np.float64)
    ncol = n_coeffs + n_components
    for i in range(n_coeffs):
        max_row = i
        max_el = _c_int_abs(A[i, i])
        for k in range(i + 1, n_coeffs):
            if _c_int_abs(A[k, i]) > max_el:
                max_el = abs(A[k, i])
                max_row = k
        for k in range(i, ncol):
            A[max_row, k], A[i, k] = A[i, k], A[max_row, k]
        for k in range(i + 1, n_coeffs):
            c = -A[k, i] / A[i, i]
            A[k, i] = 0.0
            for j in range(i + 1, ncol):
                A[k, j] += c * A[i, j]
    sol = np.zeros((n_components, n_coeffs))
    for comp in range(n_components):
        for i in range(n_coeffs - 1, -1, -1):
            sol[comp, i] = A[i, n_coeffs + comp] / A[i, i]
            for k in range(i - 1, -1, -1):
                A[k, n_coeffs + comp] -= A[k, i] * sol[comp, i]
    return sol


def _start_code(positional_sum, total_sum):
    # core/src/lstsq/ExtrapolationConfig.hpp:131-158 with grid size 3:
    # code = int(2 * t / total) where t rounds sums > 4 up to the next even
    # number (computed in float), start = (2 * code - 6) / 2 in integers.
    t = float(np.float32(np.ceil(0.5 * positional_sum) * 2.0)) if positional_sum > 4 \
        else float(positional_sum)
    code = int(np.float64(2.0 * np.float32(t)) / total_sum)
    v = 2 * code - 6
    return int(v / 2)  # C++ integer division truncates toward zero


def _ls_front(cf, tf):
    """Front scan of core/src/extrapolate_using_least_squares.hpp:196-253.

    Returns (j, i, start_x, start_y) for every cell with current ^ target set
    and at least one known cell among its 8 neighbours. Neighbours outside the
    2-D array count as unknown (the reference reads past the array there).
    """
    n0, n1 = cf.shape
    pad = np.zeros((n0 + 2, n1 + 2), dtype=np.int64)
    pad[1:-1, 1:-1] = cf
    s = np.zeros((n0, n1), dtype=np.int64)
    sx = np.zeros((n0, n1), dtype=np.int64)
    sy = np.zeros((n0, n1), dtype=np.int64)
    for jl in (-1, 0, 1):
        for il in (-1, 0, 1):
            v = pad[1 + jl: 1 + jl + n0, 1 + il: 1 + il + n1]
            if not (jl == 0 and il == 0):
                s += v  # sum_mask: every cell but the centre
            sx += v * (il + 1)  # x_mask = k % 3
            sy += v * (jl + 1)  # y_mask = k / 3
    sel = ((cf ^ tf) != 0) & (s != 0)
    js, is_ = np.nonzero(sel)  # row-major order, as the reference's scan
    return [(int(j), int(i), _start_code(int(sx[j, i]), int(s[j, i])),
             _start_code(int(sy[j, i]), int(s[j, i]))) for j, i in zip(js, is_)]


def extrapolate_using_least_squares_till_first_order(current_flag, target_flag,
                                                     eta_x, eta_y, grid_x, grid_y,
                                                     max_sweeps=1 << 20):
    """core/src/extrapolate_using_least_squares.hpp:142-446, 450-467.

    First-order (c0 + c1*x + c2*y) fit on a 3x3 window, repeated front sweeps
    until no flagged cell has a known neighbour. Arrays are modified in place;
    flags are int16 as in core/src/extrapolate_using_least_squares_bind.cpp.
    A window that would leave the array raises (the reference reads out of
    bounds there). Returns the number of sweeps that changed cells.
    """
    n0, n1 = current_flag.shape
    cf = current_flag
    sweeps = 0
    while True:
        infos = _ls_front(cf, target_flag)
        if not infos:
            return sweeps
        sweeps += 1
        if sweeps > max_sweeps:
            raise RuntimeError("least-squares extrapolation did not converge")
        for (j, i, stx, sty) in infos:
            j0, i0 = j + sty, i + stx
            if j0 < 0 or i0 < 0 or j0 + 3 > n0 or i0 + 3 > n1:
                raise ValueError("least-squares window leaves the grid")
            xs, ys, ms, r0, r1 = [], [], [], [], []
            for jl in range(j0, j0 + 3):
                for il in range(i0, i0 + 3):
                    m = float(cf[jl, il])
                    xs.append(float(grid_x[il]))
                    ys.append(float(grid_y[jl]))
                    ms.append(m)
                    r0.append(m * eta_x[jl, il])
                    r1.append(m * eta_y[jl, il])
            # binomial_fill_data_parallel :67-85 -> rows [m, m*x, m*y]
            lhs = [ms, [m * x for m, x in zip(ms, xs)], [m * y for m, y in zip(ms, ys)]]
            ata = np.zeros((3, 5))
            for a in range(3):
                for b in range(3):
                    acc = 0.0
                    for p in range(9):
                        acc += lhs[a][p] * lhs[b][p]
                    ata[a, b] = acc
                for d, rv in enumerate((r0, r1)):
                    acc = 0.0
                    for p in range(9):
                        acc += lhs[a][p] * rv[p]
                    ata[a, 3 + d] = acc
            sol = gauss_elimination(ata, 3, 2)
            loc = (1.0, float(grid_x[i]), float(grid_y[j]))
            for d, out in enumerate((eta_x, eta_y)):
                acc = 0.0
                for k in range(3):
                    acc += sol[d, k] * loc[k]
                out[j, i] = acc
        for (j, i, _, _) in infos:
            cf[j, i] = 1


def extrapolate_eta_using_least_squares(inp_phi, phi_thresh_lower_bound,
                                        phi_thresh_upper_bound, inp_eta_X, inp_eta_Y,
                                        inp_x, inp_y):
    """elasto_kernels/extrapolate_using_least_squares.py:8-38."""
    current_flag = np.asarray(inp_phi < phi_thresh_lower_bound, dtype=np.int16)
    target_flag = np.asarray(inp_phi < phi_thresh_upper_bound, dtype=np.int16)
    extrapolate_using_least_squares_till_first_order(
        current_flag, target_flag, inp_eta_X, inp_eta_Y, inp_x, inp_y
    )


def extrapolate_eta_with_least_squares(inside_solid, ball_phi, eta1, eta2,
                                       ball_phi_double, eta1_double, eta2_double,
                                       extrap_zone, grid_size_r, z):
    """elasto_kernels/extrapolate_eta_using_least_squares_unb.py:7-30."""
    ball_phi_double[grid_size_r:, :] = -ball_phi
    eta1_double[grid_size_r:, :] = inside_solid * eta1
    eta2_double[grid_size_r:, :] = inside_solid * eta2
    ball_phi_double[:grid_size_r, :] = -np.flip(ball_phi, axis=0)
    eta1_double[:grid_size_r, :] = np.flip(eta1_double[grid_size_r:, :], axis=0)
    eta2_double[:grid_size_r, :] = -np.flip(eta2_double[grid_size_r:, :], axis=0)
    extrapolate_eta_using_least_squares(
        ball_phi_double, 0, extrap_zone, eta1_double, eta2_double, z, z
    )
    eta1[...] = eta1_double[grid_size_r:, :]
    eta2[...] = eta2_double[grid_size_r:, :]


# --------------------------------------------------------------------------
# Particle remeshing (remeshed vortex method): P2M with the MP4 kernel
# --------------------------------------------------------------------------

def _mp4_inner(t):
    """MP4 for |x| <= 1 (core/src/particle_kernels/MP4.hpp, _f<0>)."""
    return 1.0 + t * t * (-2.5 + 1.5 * t)


def _mp4_outer(t):
    """MP4 for 1 < |x| <= 2 (core/src/particle_kernels/MP4.hpp, _f<1>)."""
    return 2.0 + t * (-4.0 + t * (2.5 - 0.5 * t))


def _mp4_stencil(pos):
    """Stencil anchor and the four weights per particle along one axis
    (core/src/interpolation/particles_to_mesh_2D.hpp:60-118): the anchor is
    the mesh index nearest above the particle on the cell-centred mesh; slot
    k (offset k - 2) has scaled distance |pos - ((h + 0.5) + (k - 2))| and
    weight _f<1> for the outer slots 0 and 3, _f<0> for the inner slots 1 and
    2 (core/src/particle_kernels/KernelWrapper.hpp:31-47)."""
    fl = np.floor(pos)
    h = (pos >= fl + 0.5).astype(np.int64) + fl.astype(np.int64)
    hd = h.astype(np.float64)
    w = np.empty(pos.shape + (4,))
    for k in range(4):
        d = np.fabs(pos - ((hd + 0.5) + float(k - 2)))
        w[..., k] = _mp4_outer(d) if k in (0, 3) else _mp4_inner(d)
    return h, w


def _particles_to_mesh_mp4(px, py, vin, out, dx, dy, periodic):
    n0, n1 = out.shape
    pos_x = np.asarray(px, dtype=np.float64) / dx
    pos_y = np.asarray(py, dtype=np.float64) / dy
    hx, wx = _mp4_stencil(pos_x.reshape(-1))
    hy, wy = _mp4_stencil(pos_y.reshape(-1))
    inp = np.asarray(vin, dtype=np.float64).reshape(-1)
    s = np.arange(-2, 2)
    # (particle, sy, sx) in the reference's loop order
    my = hy[:, None, None] + s[None, :, None]
    mx = hx[:, None, None] + s[None, None, :]
    weight = wy[:, :, None] * wx[:, None, :]
    val = weight * inp[:, None, None]
    if periodic:
        # (h + s + n) % n (particles_to_mesh_2D.hpp:122-137); C's % truncates
        ry, rx = my + n0, mx + n1
        if ry.min() < 0 or rx.min() < 0:
            raise ValueError("particle too far outside the periodic domain")
        idx = (rx % n1) + n1 * (ry % n0)
        valid = np.ones(idx.shape, dtype=bool)
    else:
        # one-sided near the edges: mesh points outside the grid are skipped
        # (particles_to_mesh_2D.hpp:266-318)
        valid = (my >= 0) & (my < n0) & (mx >= 0) & (mx < n1)
        idx = np.where(valid, mx + n1 * my, 0)
    flat = np.zeros(n0 * n1)
    np.add.at(flat, idx[valid], val[valid])
    out[...] = flat.reshape(n0, n1)


def particles_to_mesh_2D_mp4(particle_positions_x, particle_positions_y,
                             input_field_at_particle_positions, output_field_at_mesh,
                             delta_x, delta_y):
    """core/src/particles_to_mesh.hpp:69-91 (periodic in both directions,
    core/src/interpolation/particles_to_mesh_2D.hpp:14-143)."""
    _particles_to_mesh_mp4(particle_positions_x, particle_positions_y,
                           input_field_at_particle_positions, output_field_at_mesh,
                           delta_x, delta_y, periodic=True)


def particles_to_mesh_2D_unbounded_mp4(particle_positions_x, particle_positions_y,
                                       input_field_at_particle_positions,
                                       output_field_at_mesh, delta_x, delta_y):
    """core/src/particles_to_mesh.hpp:163-184 (unbounded,
    core/src/interpolation/particles_to_mesh_2D.hpp:152-324)."""
    _particles_to_mesh_mp4(particle_positions_x, particle_positions_y,
                           input_field_at_particle_positions, output_field_at_mesh,
                           delta_x, delta_y, periodic=False)


def _mesh_to_particles_mp4(in_x, in_y, px, py, out_x, out_y, dx, dy, periodic):
    """core/src/interpolation/mesh_to_particles_2D.hpp:11-183 (periodic) and
    :185-420 (unbounded): per particle, each stencil row is summed along x
    from 0.0 in the order sx = -2 .. 1, then the rows are weighted along y and
    summed from 0.0 in the order sy = -2 .. 1. The unbounded form clips the
    stencil at the mesh edges (:313-344) but accumulates all four rows."""
    n0, n1 = np.asarray(in_x).shape
    fx = np.asarray(in_x, dtype=np.float64).reshape(-1)
    fy = np.asarray(in_y, dtype=np.float64).reshape(-1)
    hx, wx = _mp4_stencil(np.asarray(px, dtype=np.float64).reshape(-1) / dx)
    hy, wy = _mp4_stencil(np.asarray(py, dtype=np.float64).reshape(-1) / dy)
    n = hx.size
    ps_x = np.zeros((n, 4))
    ps_y = np.zeros((n, 4))
    for sy in range(-2, 2):
        my = hy + sy
        acc_x = np.zeros(n)
        acc_y = np.zeros(n)
        for sx in range(-2, 2):
            mx = hx + sx
            if periodic:
                # (h + s + n) % n, wrapped like a mathematical modulo
                idx = ((mx + n1) % n1) + n1 * ((my + n0) % n0)
                ok = np.ones(n, dtype=bool)
            else:
                ok = (mx >= 0) & (mx < n1) & (my >= 0) & (my < n0)
                idx = np.where(ok, mx + n1 * my, 0)
            w = wx[:, sx + 2]
            acc_x = np.where(ok, acc_x + w * fx[idx], acc_x)
            acc_y = np.where(ok, acc_y + w * fy[idx], acc_y)
        ps_x[:, sy + 2] = acc_x
        ps_y[:, sy + 2] = acc_y
    rx = np.zeros(n)
    ry = np.zeros(n)
    for k in range(4):
        rx = rx + wy[:, k] * ps_x[:, k]
        ry = ry + wy[:, k] * ps_y[:, k]
    out_x[...] = rx.reshape(out_x.shape)
    out_y[...] = ry.reshape(out_y.shape)


def mesh_to_particles_2D_mp4(input_field_x, input_field_y, particle_positions_x,
                             particle_positions_y, output_field_x, output_field_y,
                             delta_x, delta_y):
    """core/src/mesh_to_particles.hpp (mesh_to_particles_2D_mp4, periodic)."""
    _mesh_to_particles_mp4(input_field_x, input_field_y, particle_positions_x,
                           particle_positions_y, output_field_x, output_field_y,
                           delta_x, delta_y, periodic=True)


def mesh_to_particles_2D_unbounded_mp4(input_field_x, input_field_y, particle_positions_x,
                                       particle_positions_y, output_field_x, output_field_y,
                                       delta_x, delta_y):
    """core/src/mesh_to_particles.hpp (mesh_to_particles_2D_unbounded_mp4)."""
    _mesh_to_particles_mp4(input_field_x, input_field_y, particle_positions_x,
                           particle_positions_y, output_field_x, output_field_y,
                           delta_x, delta_y, periodic=False)


def _advect_vorticity_via_particles(z_particles, r_particles, vort_particles, vorticity,
                                    Z_double, R_double, grid_size_r, u_z, u_r, dx, dt,
                                    p2m):
    z_particles[grid_size_r:, :] += u_z * dt
    z_particles[:grid_size_r, :] += np.flip(u_z, axis=0) * dt
    r_particles[grid_size_r:, :] += u_r * dt
    r_particles[:grid_size_r, :] += -np.flip(u_r, axis=0) * dt
    vort_particles[grid_size_r:, :] = vorticity
    vort_particles[:grid_size_r, :] = -np.flip(vorticity, axis=0)
    vort_double = 0 * Z_double
    p2m(z_particles, r_particles, vort_particles, vort_double, dx, dx)
    z_particles[...] = Z_double
    r_particles[...] = R_double
    vorticity[...] = vort_double[grid_size_r:, :]


def advect_vorticity_via_particles(z_particles, r_particles, vort_particles, vorticity,
                                   Z_double, R_double, grid_size_r, u_z, u_r, dx, dt):
    """kernels/advect_particle.py:5-35."""
    _advect_vorticity_via_particles(z_particles, r_particles, vort_particles, vorticity,
                                    Z_double, R_double, grid_size_r, u_z, u_r, dx, dt,
                                    particles_to_mesh_2D_unbounded_mp4)


def advect_vorticity_via_particles_periodic(z_particles, r_particles, vort_particles,
                                            vorticity, Z_double, R_double, grid_size_r, u_z,
                                            u_r, dx, dt):
    """kernels/advect_particle.py:38-68."""
    _advect_vorticity_via_particles(z_particles, r_particles, vort_particles, vorticity,
                                    Z_double, R_double, grid_size_r, u_z, u_r, dx, dt,
                                    particles_to_mesh_2D_mp4)
