"""Generate the golden vectors in tests/golden/ by running the reference itself.

Run in a container where the PyAxisymFlow sources are present:

    python tests/golden/make_golden.py /path/to/PyAxisymFlow

What runs unmodified from the reference:
  * every numba kernel under ``pyaxisymflow/kernels`` and
    ``pyaxisymflow/elasto_kernels`` (numba is replaced by an identity ``njit``,
    the mode the reference's own Makefile uses for coverage:
    ``NUMBA_DISABLE_JIT=1``);
  * the three spectral solvers (numpy/scipy). ``numpy.linalg.eig`` is wrapped
    to return real arrays when every imaginary part is exactly zero, which is
    what the numpy the reference pins (^1.20) did; with numpy >= 2 the
    implicit diffusion stepper cannot write its complex result into a float
    field otherwise;
  * the C++ least-squares extrapolator and particle-to-mesh interpolation,
    compiled from the reference headers by ``oracle/build.py``
    (``oracle/_ref/libref_lsq.so``, ``oracle/_ref/libref_p2m.so``), and
    ``kernels/advect_particle.py`` over the latter.

  * the pystencils ENO3 advection kernels (``pyst_kernels/advection_flux.py``,
    ``advection_timestep.py``, ``elementwise_ops.py``) and the closures that
    call them (``kernels/advect_vorticity_via_eno3.py``,
    ``elasto_kernels/advect_refmap_via_eno3.py``): pystencils is not
    installed, so ``tests/golden/pystencils_standin`` (a test-only restatement
    of the pystencils subset they use) takes its place. The kernels' own
    symbolic expressions are built, ordered and printed by sympy and evaluated
    literally in IEEE double (what pystencils' compiler flags may reorder is
    not modelled).

The full-step vectors (rigid, sedimenting and soft loops) therefore run the
reference's code for every kernel of the step, ENO3 included.

Run with the path of the reference sources as the first argument; nothing is
written into that tree (bytecode writing is switched off).
"""
import ctypes
import os
import sys
import tempfile
import types

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, REPO)

from oracle import kernels as OK  # noqa: E402
from oracle import simulation as sim  # noqa: E402


def _install_reference(ref_root):
    # the reference tree is read-only source: no __pycache__ written into it
    sys.dont_write_bytecode = True
    sys.path.insert(0, os.path.join(HERE, "pystencils_standin"))
    stub = tempfile.mkdtemp(prefix="numba_stub_")
    os.makedirs(os.path.join(stub, "numba"))
    with open(os.path.join(stub, "numba", "__init__.py"), "w") as f:
        f.write(
            "def njit(*a, **k):\n"
            "    if len(a) == 1 and callable(a[0]) and not k:\n"
            "        return a[0]\n"
            "    return lambda f: f\n"
        )
    sys.path.insert(0, stub)
    sys.path.insert(0, ref_root)
    orig_eig = np.linalg.eig

    def eig_pinned(a):
        w, v = orig_eig(a)
        if np.iscomplexobj(w) and not np.any(w.imag) and not np.any(v.imag):
            return w.real.copy(), v.real.copy()
        return w, v

    np.linalg.eig = eig_pinned


def _ref_kernels():
    from pyaxisymflow.kernels import brinkmann_penalize as bp
    from pyaxisymflow.kernels import compute_velocity_from_psi as cv
    from pyaxisymflow.kernels import compute_vorticity_from_velocity as cw
    from pyaxisymflow.kernels import smooth_Heaviside as sh
    from pyaxisymflow.kernels import kill_boundary_vorticity_sine as kb
    from pyaxisymflow.kernels import diffusion_RK2 as dr
    from pyaxisymflow.kernels import periodic_boundary_ghost_comm as pg
    from pyaxisymflow.kernels import compute_forces as cf
    from pyaxisymflow.kernels import force_projection as fp
    from pyaxisymflow.elasto_kernels import solid_sigma as ss
    from pyaxisymflow.elasto_kernels import div_tau as dt
    from pyaxisymflow.kernels import FastDiagonalisationStokesSolver as fs
    from pyaxisymflow.kernels import FastDiagonalisationPotentialSolver as fpo
    from pyaxisymflow.kernels import implicit_diffusion_solver as ids
    from pyaxisymflow.kernels import advect_vorticity_via_eno3 as aw
    from pyaxisymflow.elasto_kernels import advect_refmap_via_eno3 as ae

    ns = types.SimpleNamespace(
        brinkmann_penalize=bp.brinkmann_penalize,
        compute_velocity_from_psi_unb=cv.compute_velocity_from_psi_unb,
        compute_velocity_from_psi_periodic=cv.compute_velocity_from_psi_periodic,
        compute_vorticity_from_velocity_unb=cw.compute_vorticity_from_velocity_unb,
        compute_vorticity_from_velocity_periodic=cw.compute_vorticity_from_velocity_periodic,
        smooth_Heaviside=sh.smooth_Heaviside,
        kill_boundary_vorticity_sine_z=kb.kill_boundary_vorticity_sine_z,
        kill_boundary_vorticity_sine_r=kb.kill_boundary_vorticity_sine_r,
        diffusion_RK2_unb=dr.diffusion_RK2_unb,
        diffusion_RK2_periodic=dr.diffusion_RK2_periodic,
        gen_periodic_boundary_ghost_comm=pg.gen_periodic_boundary_ghost_comm,
        gen_periodic_boundary_ghost_comm_eta=pg.gen_periodic_boundary_ghost_comm_eta,
        compute_force_on_body=cf.compute_force_on_body,
        force_projection=fp.force_projection,
        solid_sigma=ss.solid_sigma,
        update_vorticity_from_solid_stress=dt.update_vorticity_from_solid_stress,
        FastDiagonalisationStokesSolver=fs.FastDiagonalisationStokesSolver,
        FastDiagonalisationPotentialSolver=fpo.FastDiagonalisationPotentialSolver,
        ImplicitEulerDiffusionStepper=ids.ImplicitEulerDiffusionStepper,
        gen_advect_vorticity_via_eno3=aw.gen_advect_vorticity_via_eno3,
        gen_advect_vorticity_via_eno3_periodic=aw.gen_advect_vorticity_via_eno3_periodic,
        gen_advect_refmap_via_eno3=ae.gen_advect_refmap_via_eno3,
        gen_advect_refmap_via_eno3_periodic=ae.gen_advect_refmap_via_eno3_periodic,
        extrapolate_eta_with_least_squares=None,
    )
    return ns


def _ref_lsq_lib():
    path = os.path.join(REPO, "oracle", "_ref", "libref_lsq.so")
    lib = ctypes.CDLL(path)
    return lib


def _ref_extrapolate(lib):
    P = ctypes.POINTER(ctypes.c_double)
    S = ctypes.POINTER(ctypes.c_short)

    def extrap_first_order(cf, tf, ex, ey, gx, gy):
        gx = np.ascontiguousarray(gx, dtype=np.float64)
        gy = np.ascontiguousarray(gy, dtype=np.float64)
        lib.ref_extrapolate_till_first_order(
            cf.ctypes.data_as(S), tf.ctypes.data_as(S), ex.ctypes.data_as(P),
            ey.ctypes.data_as(P), gx.ctypes.data_as(P), gy.ctypes.data_as(P),
            cf.shape[0], cf.shape[1], len(gx), len(gy))

    def extrapolate_eta_with_least_squares(inside_solid, ball_phi, eta1, eta2,
                                           ball_phi_double, eta1_double, eta2_double,
                                           extrap_zone, grid_size_r, z):
        # elasto_kernels/extrapolate_eta_using_least_squares_unb.py:19-30 and
        # elasto_kernels/extrapolate_using_least_squares.py:33-38, calling the
        # compiled reference core
        ball_phi_double[grid_size_r:, :] = -ball_phi
        eta1_double[grid_size_r:, :] = inside_solid * eta1
        eta2_double[grid_size_r:, :] = inside_solid * eta2
        ball_phi_double[:grid_size_r, :] = -np.flip(ball_phi, axis=0)
        eta1_double[:grid_size_r, :] = np.flip(eta1_double[grid_size_r:, :], axis=0)
        eta2_double[:grid_size_r, :] = -np.flip(eta2_double[grid_size_r:, :], axis=0)
        cf = np.asarray(ball_phi_double < 0, dtype=np.int16)
        tf = np.asarray(ball_phi_double < extrap_zone, dtype=np.int16)
        extrap_first_order(cf, tf, eta1_double, eta2_double, z, z)
        eta1[...] = eta1_double[grid_size_r:, :]
        eta2[...] = eta2_double[grid_size_r:, :]

    return extrap_first_order, extrapolate_eta_with_least_squares


def _coords(nr, nz, dx):
    z = np.linspace(dx / 2, nz * dx - dx / 2, nz)
    r = np.linspace(dx / 2, nr * dx - dx / 2, nr)
    Z, R = np.meshgrid(z, r)
    return z, r, Z, R


def kernel_vectors(ref):
    """Single-kernel known answers on seeded inputs (odd, non-square sizes)."""
    out = {}
    rng = np.random.default_rng(20240611)
    for tag, (nr, nz) in {"a": (20, 28), "b": (17, 23)}.items():
        dx = 1.0 / nz
        z, r, Z, R = _coords(nr, nz, dx)
        psi = rng.standard_normal((nr, nz))
        out[f"{tag}/R"] = R
        out[f"{tag}/Z"] = Z
        out[f"{tag}/dx"] = np.array(dx)
        out[f"{tag}/psi"] = psi
        u_z = np.zeros_like(psi)
        u_r = np.zeros_like(psi)
        ref.compute_velocity_from_psi_unb(u_z, u_r, psi, R, dx)
        out[f"{tag}/velocity_u_z"] = u_z
        out[f"{tag}/velocity_u_r"] = u_r
        vort = rng.standard_normal((nr, nz))
        out[f"{tag}/vort_in"] = vort.copy()
        ref.compute_vorticity_from_velocity_unb(vort, u_z, u_r, dx)
        out[f"{tag}/vorticity_from_velocity"] = vort
        # Brinkman with a smooth mask and nonzero body velocity
        chi = rng.random((nr, nz))
        pz = np.zeros_like(chi)
        pr = np.zeros_like(chi)
        ref.brinkmann_penalize(1e4, 3.7e-3, chi, 0.3, -0.2, u_z, u_r, pz, pr)
        out[f"{tag}/chi"] = chi
        out[f"{tag}/brinkman_u_z"] = pz
        out[f"{tag}/brinkman_u_r"] = pr
        # smooth Heaviside of a sphere level set
        phi = -np.sqrt((Z - 0.5) ** 2 + R ** 2) + 0.3
        H = np.zeros_like(phi)
        w = dx * 2 ** 0.5
        ref.smooth_Heaviside(H, phi, w)
        out[f"{tag}/phi"] = phi
        out[f"{tag}/heaviside_w"] = np.array(w)
        out[f"{tag}/heaviside"] = H
        # kill boundary vorticity
        wk = rng.standard_normal((nr, nz))
        out[f"{tag}/kill_in"] = wk.copy()
        ref.kill_boundary_vorticity_sine_z(wk, Z, 3, dx)
        out[f"{tag}/kill_z"] = wk.copy()
        ref.kill_boundary_vorticity_sine_r(wk, R, 3, dx)
        out[f"{tag}/kill_zr"] = wk
        # RK2 diffusion
        wd = rng.standard_normal((nr, nz))
        tmp = np.zeros_like(wd)
        out[f"{tag}/diff_in"] = wd.copy()
        ref.diffusion_RK2_unb(wd, tmp, R, 1e-2, 0.2 * dx * dx / 1e-2, dx)
        out[f"{tag}/diff_nu"] = np.array(1e-2)
        out[f"{tag}/diff_dt"] = np.array(0.2 * dx * dx / 1e-2)
        out[f"{tag}/diffusion_unb"] = wd
        out[f"{tag}/diffusion_unb_temp"] = tmp
        comm = ref.gen_periodic_boundary_ghost_comm(2)
        wp = rng.standard_normal((nr, nz))
        tmp = np.zeros_like(wp)
        out[f"{tag}/diffp_in"] = wp.copy()
        ref.diffusion_RK2_periodic(wp, tmp, R, 1e-2, 0.2 * dx * dx / 1e-2, dx, comm)
        out[f"{tag}/diffusion_periodic"] = wp
        # ghost exchange (plain and eta-shifted)
        g = rng.standard_normal((nr, nz))
        out[f"{tag}/ghost_in"] = g.copy()
        comm(g)
        out[f"{tag}/ghost"] = g
        g2 = out[f"{tag}/ghost_in"].copy()
        ref.gen_periodic_boundary_ghost_comm_eta(2, nz * dx, dx)(g2)
        out[f"{tag}/ghost_eta"] = g2
        # periodic velocity / vorticity
        psi_p = psi.copy()
        uzp = np.zeros_like(psi)
        urp = np.zeros_like(psi)
        ref.compute_velocity_from_psi_periodic(uzp, urp, psi_p, R, dx, comm)
        out[f"{tag}/velocity_periodic_u_z"] = uzp
        out[f"{tag}/velocity_periodic_u_r"] = urp
        out[f"{tag}/velocity_periodic_psi"] = psi_p
        # forces
        uz_f = rng.standard_normal((nr, nz))
        Fp, Fu = ref.compute_force_on_body(R, chi, 1.3, 1e4, uz_f, 0.25, 0.7, 2e-3, 1e-4)
        out[f"{tag}/force_u_z"] = uz_f
        out[f"{tag}/force"] = np.array([Fp, Fu])
        ur_f = rng.standard_normal((nr, nz))
        Uz, Ur = ref.force_projection(2.5, chi, uz_f, ur_f, R)
        out[f"{tag}/proj_u_r"] = ur_f
        out[f"{tag}/projection"] = np.array([Uz, Ur])
        # elasto: solid stress and its curl
        e1 = Z + 0.01 * rng.standard_normal((nr, nz))
        e2 = R + 0.01 * rng.standard_normal((nr, nz))
        s11, s12, s22, a, b, c, d = (np.zeros_like(e1) for _ in range(7))
        ref.solid_sigma(s11, s12, s22, 0.37, dx, e1, e2, a, b, c, d)
        out[f"{tag}/eta1"] = e1
        out[f"{tag}/eta2"] = e2
        for k, v in dict(s11=s11, s12=s12, s22=s22, e1z=a, e1r=b, e2z=c, e2r=d).items():
            out[f"{tag}/sigma_{k}"] = v
        wv = rng.standard_normal((nr, nz))
        tz = np.zeros_like(wv)
        tr = np.zeros_like(wv)
        out[f"{tag}/divtau_in"] = wv.copy()
        ref.update_vorticity_from_solid_stress(wv, tz, tr, s11, s12, s22, R, 1.5e-3, dx)
        out[f"{tag}/divtau_w"] = wv
        out[f"{tag}/divtau_tau_z"] = tz
        out[f"{tag}/divtau_tau_r"] = tr
    return out


def solver_vectors(ref):
    out = {}
    rng = np.random.default_rng(7)
    nr, nz = 24, 40
    dx = 1.0 / nz
    rhs = rng.standard_normal((nr, nz))
    out["rhs"] = rhs
    out["dx"] = np.array(dx)
    for bc in (OK.NEUMANN_ZR, OK.NEUMANN_R_PERIODIC_Z, OK.DIRICHLET_R_PERIODIC_Z):
        s = ref.FastDiagonalisationStokesSolver(nr, nz, dx, bc_type=bc)
        psi = np.zeros_like(rhs)
        s.solve(solution_field=psi, rhs_field=rhs)
        out[f"stokes/{bc}"] = psi
    p = ref.FastDiagonalisationPotentialSolver(nr, nz, dx)
    phi = np.zeros_like(rhs)
    p.solve(solution_field=phi, rhs_field=rhs)
    out["potential"] = phi
    dt = 0.25 * dx * dx / 1e-2
    st = ref.ImplicitEulerDiffusionStepper(dt, 1e-2, nr, nz, dx)
    w = rhs.copy()
    st.step(vorticity_field=w, dt=dt)
    out["implicit_diffusion_dt"] = np.array(dt)
    out["implicit_diffusion"] = w
    return out


def lsq_vectors(extrap_first_order):
    out = {}
    kat = np.array([[2.56, 0.86, 4.2, 1.964, 1.284],
                    [0.86, 0.32, 1.4, 0.666, 0.45],
                    [4.2, 1.4, 7.0, 3.22, 2.1]])
    out["gauss_kat_in"] = kat
    # expected solution from core/src/lstsq/test_least_squares.cpp:38-39
    out["gauss_kat_expected"] = np.array([[0.7, 0.2, 0.0], [0.3, 0.6, 0.0]])
    rng = np.random.default_rng(11)
    lib = _ref_lsq_lib()
    P = ctypes.POINTER(ctypes.c_double)
    systems = rng.standard_normal((64, 3, 5)) * rng.choice([0.1, 1.0, 10.0], size=(64, 3, 5))
    sols = np.zeros((64, 2, 3))
    for k in range(64):
        a = np.ascontiguousarray(systems[k])
        s = np.zeros(6)
        lib.ref_gauss_elimination_3x2(a.ctypes.data_as(P), s.ctypes.data_as(P))
        sols[k] = s.reshape(2, 3)
    out["gauss_random_in"] = systems
    out["gauss_random_out"] = sols
    for tag, (n0, n1, seed) in {"a": (40, 36, 3), "b": (64, 64, 4)}.items():
        dx = 1.0 / n1
        x = np.linspace(dx / 2, n1 * dx - dx / 2, n1)
        y = np.linspace(dx / 2, n0 * dx - dx / 2, n0)
        X, Y = np.meshgrid(x, y)
        r2 = np.random.default_rng(seed)
        rad = 0.2 + 0.05 * r2.random()
        phi = np.sqrt((X - 0.5) ** 2 + (Y - n0 * dx / 2) ** 2) - rad
        cf = np.asarray(phi < 0, dtype=np.int16)
        tf = np.asarray(phi < 6 * dx, dtype=np.int16)
        ex = (X + 0.01 * np.sin(7 * Y)) * cf
        ey = (Y + 0.01 * np.cos(5 * X)) * cf
        out[f"{tag}/current_flag"] = cf.copy()
        out[f"{tag}/target_flag"] = tf.copy()
        out[f"{tag}/eta_x_in"] = ex.copy()
        out[f"{tag}/eta_y_in"] = ey.copy()
        out[f"{tag}/grid_x"] = x
        out[f"{tag}/grid_y"] = y
        extrap_first_order(cf, tf, ex, ey, x, y)
        out[f"{tag}/current_flag_out"] = cf
        out[f"{tag}/eta_x_out"] = ex
        out[f"{tag}/eta_y_out"] = ey
    return out


def step_vectors(ref):
    """Full-step loops on small grids, every kernel the reference's own."""
    out = {}
    # rigid sphere (flow past sphere), config-1 geometry scaled to 64 x 32
    case = sim.RigidSphereCase(nz=64, nr=32, dx=2.0 / 64, r_sphere=0.125, z_cm=0.5)
    st, coords = sim.rigid_sphere_init(case, ref)
    out["rigid/omega0"] = st.vorticity.copy()
    out["rigid/chi"] = st.char_func.copy()
    solver = ref.FastDiagonalisationStokesSolver(case.nr, case.nz, case.dx)
    adv = ref.gen_advect_vorticity_via_eno3(case.dx, case.nr, case.nz)
    dts, cds = [], []
    for n in range(40):
        sim.rigid_sphere_step(case, st, coords, solver, adv, ref)
        dts.append(st.dt)
        cds.append(st.Cd)
        if n + 1 in (1, 10, 40):
            out[f"rigid/omega_{n + 1}"] = st.vorticity.copy()
            out[f"rigid/psi_{n + 1}"] = st.psi.copy()
            out[f"rigid/u_z_{n + 1}"] = st.u_z.copy()
            out[f"rigid/u_r_{n + 1}"] = st.u_r.copy()
    out["rigid/dt"] = np.array(dts)
    out["rigid/Cd"] = np.array(cds)
    # sedimenting sphere, moving mask + FP64 force integrals
    scase = sim.SedimentingCase(nz=64, nr=16, dx=1.0 / 64, r_sphere=0.08, z_cm=0.6,
                                nu=0.01, rho_s=1.5)
    rng = np.random.default_rng(5)
    w0 = 1e-3 * rng.standard_normal((16, 64))
    sst, scoords = sim.sedimenting_init(scase, ref, vorticity=w0)
    out["sediment/omega0"] = w0
    ssolver = ref.FastDiagonalisationStokesSolver(scase.nr, scase.nz, scase.dx)
    sadv = ref.gen_advect_vorticity_via_eno3(scase.dx, scase.nr, scase.nz)
    hist = []
    for n in range(30):
        sim.sedimenting_step(scase, sst, scoords, ssolver, sadv, ref)
        hist.append([sst.dt, sst.U_z_cm_part, sst.part_Z_cm, sst.F_total, sst.Cd])
    out["sediment/omega_30"] = sst.vorticity.copy()
    out["sediment/chi_30"] = sst.char_func.copy()
    out["sediment/history"] = np.array(hist)
    return out


def soft_vectors(ref):
    out = {}
    case = sim.SoftSphereCase(nz=64, nr=32, dx=1.0 / 64, r_ball=0.15, lam=1e6)
    st, coords = sim.soft_sphere_init(case, ref)
    solver = ref.FastDiagonalisationStokesSolver(case.nr, case.nz, case.dx)
    adv_w = ref.gen_advect_vorticity_via_eno3(case.dx, case.nr, case.nz)
    adv_e = ref.gen_advect_refmap_via_eno3(case.dx, case.nr, case.nz)
    for n in range(12):
        sim.soft_sphere_step(case, st, coords, solver, adv_w, adv_e, ref)
    out["soft/omega_12"] = st.vorticity.copy()
    out["soft/eta1_12"] = st.eta1.copy()
    out["soft/eta2_12"] = st.eta2.copy()
    out["soft/phi_12"] = st.ball_phi.copy()
    out["soft/chi_12"] = st.ball_char_func.copy()
    out["soft/t_12"] = np.array(st.t)
    return out


def eno3_vectors(ref):
    """The reference's own ENO3 advection closures (vorticity: conservative,
    reference map: non-conservative; unbounded and periodic) on seeded
    fields, through the pystencils stand-in. Case "tie" draws velocities from
    a few multiples of 1/4, so many faces have u0 == -u1 exactly (the
    upwind test is strict)."""
    out = {}
    rng = np.random.default_rng(31)
    for tag, (nr, nz, tie) in {"a": (24, 40, False), "b": (37, 29, False),
                               "tie": (20, 32, True)}.items():
        dx = 1.0 / nz
        dt = 0.37 * dx
        z, r, Z, R = _coords(nr, nz, dx)
        if tie:
            uz = 0.25 * rng.integers(-3, 4, (nr, nz)).astype(np.float64)
            ur = 0.25 * rng.integers(-3, 4, (nr, nz)).astype(np.float64)
        else:
            uz = rng.standard_normal((nr, nz))
            ur = rng.standard_normal((nr, nz))
        w0 = rng.standard_normal((nr, nz))
        e10 = Z + 0.05 * rng.standard_normal((nr, nz))
        e20 = R + 0.05 * rng.standard_normal((nr, nz))
        out[f"{tag}/dx"], out[f"{tag}/dt"] = np.array(dx), np.array(dt)
        out[f"{tag}/u_z"], out[f"{tag}/u_r"] = uz, ur
        out[f"{tag}/w0"], out[f"{tag}/eta1_0"], out[f"{tag}/eta2_0"] = w0, e10, e20
        # two successive calls of one closure (its buffers carry over)
        adv = ref.gen_advect_vorticity_via_eno3(dx, nr, nz)
        w = w0.copy()
        adv(w, uz, ur, dt)
        out[f"{tag}/w_1"] = w.copy()
        adv(w, uz, ur, dt)
        out[f"{tag}/w_2"] = w.copy()
        adve = ref.gen_advect_refmap_via_eno3(dx, nr, nz)
        e1, e2 = e10.copy(), e20.copy()
        adve(e1, e2, uz, ur, dt)
        out[f"{tag}/eta1_1"], out[f"{tag}/eta2_1"] = e1.copy(), e2.copy()
        # periodic along z (2 ghost columns each side)
        comm = ref.gen_periodic_boundary_ghost_comm(2)
        comm_eta = ref.gen_periodic_boundary_ghost_comm_eta(2, nz * dx, dx)
        advp = ref.gen_advect_vorticity_via_eno3_periodic(dx, nr, nz, comm)
        uzp, urp, wp = uz.copy(), ur.copy(), w0.copy()
        advp(wp, uzp, urp, dt)
        out[f"{tag}/w_periodic"] = wp
        advpe = ref.gen_advect_refmap_via_eno3_periodic(dx, nr, nz, comm, comm_eta)
        uzp, urp, e1, e2 = uz.copy(), ur.copy(), e10.copy(), e20.copy()
        advpe(e1, e2, uzp, urp, dt)
        out[f"{tag}/eta1_periodic"], out[f"{tag}/eta2_periodic"] = e1, e2
    return out


def _ref_p2m_module():
    """A stand-in for the compiled module pyaxisymflow.core.particles_to_mesh
    whose 2-D MP4 functions call the reference's own C++
    (oracle/_ref/libref_p2m.so, built from core/src/particles_to_mesh.hpp)."""
    lib = ctypes.CDLL(os.path.join(REPO, "oracle", "_ref", "libref_p2m.so"))
    P = ctypes.c_void_p
    for f in (lib.ref_p2m_2d_mp4, lib.ref_p2m_2d_unbounded_mp4):
        f.argtypes = [P, P, P, P, ctypes.c_int, ctypes.c_int, ctypes.c_double, ctypes.c_double]

    def wrap(fn):
        def call(x, y, vin, out, dx, dy):
            arrs = [np.ascontiguousarray(a, dtype=np.float64) for a in (x, y, vin)]
            assert out.flags.c_contiguous and out.dtype == np.float64
            fn(arrs[0].ctypes.data, arrs[1].ctypes.data, arrs[2].ctypes.data, out.ctypes.data,
               out.shape[0], out.shape[1], dx, dy)
        return call

    mod = types.ModuleType("pyaxisymflow.core.particles_to_mesh")
    mod.particles_to_mesh_2D_mp4 = wrap(lib.ref_p2m_2d_mp4)
    mod.particles_to_mesh_2D_unbounded_mp4 = wrap(lib.ref_p2m_2d_unbounded_mp4)
    return mod


def p2m_vectors():
    """Particle-to-mesh (MP4) and vorticity advection by remeshed particles,
    computed by the reference: the C++ interpolation compiled from its header
    and kernels/advect_particle.py run unmodified over it."""
    mod = _ref_p2m_module()
    sys.modules["pyaxisymflow.core.particles_to_mesh"] = mod
    import pyaxisymflow.core
    pyaxisymflow.core.particles_to_mesh = mod
    from pyaxisymflow.kernels import advect_particle as ap
    rng = np.random.default_rng(11)
    out = {}
    # (tag, n0, n1, dx, displacement in cells; None = anywhere in the domain)
    for tag, n0, n1, dx, disp in (("a", 16, 24, 0.1, 0.95), ("b", 64, 48, 1.0 / 64, 0.3),
                                  ("c", 40, 40, 0.05, None)):
        Z, R = np.meshgrid((np.arange(n1) + 0.5) * dx, (np.arange(n0) + 0.5) * dx)
        if disp is None:
            px = rng.uniform(0.0, n1 * dx, Z.shape)
            py = rng.uniform(0.0, n0 * dx, Z.shape)
        else:
            px = Z + disp * dx * rng.uniform(-1.0, 1.0, Z.shape)
            py = R + disp * dx * rng.uniform(-1.0, 1.0, Z.shape)
        v = rng.standard_normal(Z.shape)
        out[f"{tag}/px"], out[f"{tag}/py"], out[f"{tag}/v"] = px, py, v
        out[f"{tag}/dx"] = np.array(dx)
        for name, fn in (("periodic", mod.particles_to_mesh_2D_mp4),
                         ("unbounded", mod.particles_to_mesh_2D_unbounded_mp4)):
            o = np.zeros((n0, n1))
            fn(px, py, v, o, dx, dx)
            out[f"{tag}/{name}"] = o
    # two steps of each advection function on a (2 nr, nz) mirrored domain
    nr, nz = 24, 32
    dx = 1.0 / nz
    z = (np.arange(nz) + 0.5) * dx
    r2 = (np.arange(2 * nr) + 0.5) * dx
    Zd, Rd = np.meshgrid(z, r2)
    w0 = rng.standard_normal((nr, nz))
    uz = rng.uniform(-1.0, 1.0, (nr, nz))
    ur = rng.uniform(-1.0, 1.0, (nr, nz))
    dt = 0.5 * dx
    out["adv/w0"], out["adv/u_z"], out["adv/u_r"] = w0, uz, ur
    out["adv/dx"], out["adv/dt"], out["adv/nr"] = np.array(dx), np.array(dt), np.array(nr)
    for name, fn in (("unbounded", ap.advect_vorticity_via_particles),
                     ("periodic", ap.advect_vorticity_via_particles_periodic)):
        w = w0.copy()
        zp, rp, vp = Zd.copy(), Rd.copy(), np.zeros_like(Zd)
        for _ in range(2):
            fn(zp, rp, vp, w, Zd, Rd, nr, uz, ur, dx, dt)
        out[f"adv/{name}"] = w
    return out


def m2p_vectors():
    """Mesh-to-particle (MP4) interpolation computed by the reference's C++
    (core/src/mesh_to_particles.hpp, compiled into oracle/_ref/libref_p2m.so):
    periodic and unbounded forms, particles scattered in and around the mesh,
    particle arrays shaped differently from the mesh."""
    lib = ctypes.CDLL(os.path.join(REPO, "oracle", "_ref", "libref_p2m.so"))
    P, I, D = ctypes.c_void_p, ctypes.c_int, ctypes.c_double
    for f in (lib.ref_m2p_2d_mp4, lib.ref_m2p_2d_unbounded_mp4):
        f.argtypes = [P, P, I, I, P, P, P, P, I, I, D, D]
    rng = np.random.default_rng(12)
    out = {}
    # (tag, mesh n0, n1, particles p0, p1, dx, margin around the mesh in cells)
    for tag, n0, n1, p0, p1, dx, margin in (("a", 16, 24, 16, 24, 0.1, 2.5),
                                            ("b", 48, 32, 20, 28, 1.0 / 48, 0.0),
                                            ("c", 12, 40, 30, 10, 0.05, 1.0)):
        fx, fy = rng.standard_normal((n0, n1)), rng.standard_normal((n0, n1))
        px = rng.uniform(-margin, n1 + margin, (p0, p1)) * dx
        py = rng.uniform(-margin, n0 + margin, (p0, p1)) * dx
        out[f"{tag}/fx"], out[f"{tag}/fy"], out[f"{tag}/px"], out[f"{tag}/py"] = fx, fy, px, py
        out[f"{tag}/dx"] = np.array(dx)
        for name, fn in (("periodic", lib.ref_m2p_2d_mp4),
                         ("unbounded", lib.ref_m2p_2d_unbounded_mp4)):
            ox, oy = np.zeros((p0, p1)), np.zeros((p0, p1))
            fn(fx.ctypes.data, fy.ctypes.data, n0, n1, px.ctypes.data, py.ctypes.data,
               ox.ctypes.data, oy.ctypes.data, p0, p1, dx, dx)
            out[f"{tag}/{name}_x"], out[f"{tag}/{name}_y"] = ox, oy
    return out


def main(ref_root):
    _install_reference(ref_root)
    ref = _ref_kernels()
    extrap_first_order, ref.extrapolate_eta_with_least_squares = _ref_extrapolate(_ref_lsq_lib())
    np.savez_compressed(os.path.join(HERE, "kernels.npz"), **kernel_vectors(ref))
    np.savez_compressed(os.path.join(HERE, "solvers.npz"), **solver_vectors(ref))
    np.savez_compressed(os.path.join(HERE, "lsq.npz"), **lsq_vectors(extrap_first_order))
    np.savez_compressed(os.path.join(HERE, "p2m.npz"), **p2m_vectors())
    np.savez_compressed(os.path.join(HERE, "m2p.npz"), **m2p_vectors())
    np.savez_compressed(os.path.join(HERE, "steps.npz"), **step_vectors(ref))
    np.savez_compressed(os.path.join(HERE, "soft.npz"), **soft_vectors(ref))
    np.savez_compressed(os.path.join(HERE, "eno3.npz"), **eno3_vectors(ref))
    print("golden vectors written to", HERE)


if __name__ == "__main__":
    if len(sys.argv) < 2:
        sys.exit("usage: make_golden.py REFERENCE_ROOT [m2p|p2m|eno3]")
    root = sys.argv[1]
    if len(sys.argv) > 2 and sys.argv[2] == "m2p":
        # only the mesh-to-particle vectors (needs oracle/_ref/libref_p2m.so)
        np.savez_compressed(os.path.join(HERE, "m2p.npz"), **m2p_vectors())
        print("m2p vectors written to", HERE)
    elif len(sys.argv) > 2 and sys.argv[2] == "eno3":
        # only the ENO3 vectors (reference kernels through the stand-in)
        _install_reference(root)
        np.savez_compressed(os.path.join(HERE, "eno3.npz"), **eno3_vectors(_ref_kernels()))
        print("eno3 vectors written to", HERE)
    elif len(sys.argv) > 2 and sys.argv[2] == "p2m":
        # only the particle remeshing vectors
        _install_reference(root)
        np.savez_compressed(os.path.join(HERE, "p2m.npz"), **p2m_vectors())
        print("p2m vectors written to", HERE)
    else:
        main(root)
