"""CUDA kernels through the C ABI against the reference golden vectors and the oracle.

Bit-exact where the reference kernel has no transcendental function (the CUDA
kernels issue the reference's operations in its order, without FMA
contraction); within a few ulp where sin/pow enter (CUDA's libm differs from
glibc's in the last bit); 1e-12 relative L2 for the dense spectral solves.
FP32 variants are checked against the FP64 oracle at FP32 accuracy.
"""
import numpy as np
import pytest
import torch

from oracle import kernels as K

pytestmark = pytest.mark.gpu

# CUDA sin / pow vs glibc: a few ulp on O(1) values
ULP_RTOL = 1e-15
ULP_ATOL = 1e-15
SOLVE_RTOL = 1e-12
F32_RTOL = 2e-5


def dev(a, dtype=torch.float64):
    return torch.tensor(np.ascontiguousarray(a), dtype=dtype, device="cuda")


def host(t):
    torch.cuda.synchronize()
    return t.detach().to("cpu", torch.float64).numpy()


def rel_l2(a, b):
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))


@pytest.fixture(scope="module")
def gk():
    from pyaxisymflow_gb300 import _native
    _native.lib()
    from pyaxisymflow_gb300.kernels import (brinkmann_penalize, compute_forces,
                                            compute_velocity_from_psi,
                                            compute_vorticity_from_velocity, diffusion_RK2,
                                            force_projection, kill_boundary_vorticity_sine,
                                            periodic_boundary_ghost_comm, smooth_Heaviside)
    from pyaxisymflow_gb300.elasto_kernels import div_tau, solid_sigma

    class NS:
        pass

    ns = NS()
    for mod in (brinkmann_penalize, compute_forces, compute_velocity_from_psi,
                compute_vorticity_from_velocity, diffusion_RK2, force_projection,
                kill_boundary_vorticity_sine, periodic_boundary_ghost_comm, smooth_Heaviside,
                div_tau, solid_sigma):
        for k, v in vars(mod).items():
            if callable(v) and not k.startswith("_"):
                setattr(ns, k, v)
    return ns


@pytest.mark.parametrize("tag", ["a", "b"])
def test_pointwise_against_reference_golden(golden, gk, tag):
    g = golden("kernels")
    R, Z, dx = g[f"{tag}/R"], g[f"{tag}/Z"], float(g[f"{tag}/dx"])
    dR, dZ = dev(R), dev(Z)
    psi = dev(g[f"{tag}/psi"])
    uz, ur = torch.zeros_like(psi), torch.zeros_like(psi)
    gk.compute_velocity_from_psi_unb(uz, ur, psi, dR, dx)
    np.testing.assert_array_equal(host(uz), g[f"{tag}/velocity_u_z"])
    np.testing.assert_array_equal(host(ur), g[f"{tag}/velocity_u_r"])
    vort = dev(g[f"{tag}/vort_in"])
    gk.compute_vorticity_from_velocity_unb(vort, uz, ur, dx)
    np.testing.assert_array_equal(host(vort), g[f"{tag}/vorticity_from_velocity"])
    chi = dev(g[f"{tag}/chi"])
    pz, pr = torch.zeros_like(chi), torch.zeros_like(chi)
    gk.brinkmann_penalize(1e4, 3.7e-3, chi, 0.3, -0.2, uz, ur, pz, pr)
    np.testing.assert_array_equal(host(pz), g[f"{tag}/brinkman_u_z"])
    np.testing.assert_array_equal(host(pr), g[f"{tag}/brinkman_u_r"])
    # smoothed Heaviside: exact 0 / 1 outside the blend band, ulp-close inside
    phi = g[f"{tag}/phi"]
    w = float(g[f"{tag}/heaviside_w"])
    H = torch.zeros_like(chi)
    gk.smooth_Heaviside(H, dev(phi), w)
    h, ref = host(H), g[f"{tag}/heaviside"]
    band = np.abs(phi) < w
    np.testing.assert_array_equal(h[~band], ref[~band])
    np.testing.assert_allclose(h[band], ref[band], rtol=ULP_RTOL, atol=ULP_ATOL)
    np.testing.assert_array_equal(h > 0.5, ref > 0.5)
    wk = dev(g[f"{tag}/kill_in"])
    gk.kill_boundary_vorticity_sine_z(wk, dZ, 3, dx)
    np.testing.assert_allclose(host(wk), g[f"{tag}/kill_z"], rtol=ULP_RTOL, atol=ULP_ATOL)
    gk.kill_boundary_vorticity_sine_r(wk, dR, 3, dx)
    np.testing.assert_allclose(host(wk), g[f"{tag}/kill_zr"], rtol=ULP_RTOL, atol=ULP_ATOL)
    nu, dt = float(g[f"{tag}/diff_nu"]), float(g[f"{tag}/diff_dt"])
    wd = dev(g[f"{tag}/diff_in"])
    tmp = torch.zeros_like(wd)
    gk.diffusion_RK2_unb(wd, tmp, dR, nu, dt, dx)
    np.testing.assert_allclose(host(wd), g[f"{tag}/diffusion_unb"], rtol=1e-14, atol=1e-14)
    np.testing.assert_allclose(host(tmp), g[f"{tag}/diffusion_unb_temp"], rtol=1e-14, atol=1e-14)
    comm = gk.gen_periodic_boundary_ghost_comm(2)
    wp = dev(g[f"{tag}/diffp_in"])
    gk.diffusion_RK2_periodic(wp, torch.zeros_like(wp), dR, nu, dt, dx, comm)
    np.testing.assert_allclose(host(wp), g[f"{tag}/diffusion_periodic"], rtol=1e-14, atol=1e-14)
    gi = dev(g[f"{tag}/ghost_in"])
    comm(gi)
    np.testing.assert_array_equal(host(gi), g[f"{tag}/ghost"])
    gi = dev(g[f"{tag}/ghost_in"])
    gk.gen_periodic_boundary_ghost_comm_eta(2, psi.shape[1] * dx, dx)(gi)
    np.testing.assert_array_equal(host(gi), g[f"{tag}/ghost_eta"])
    psi_p = dev(g[f"{tag}/psi"])
    uzp, urp = torch.zeros_like(psi), torch.zeros_like(psi)
    gk.compute_velocity_from_psi_periodic(uzp, urp, psi_p, dR, dx, comm)
    np.testing.assert_array_equal(host(uzp), g[f"{tag}/velocity_periodic_u_z"])
    np.testing.assert_array_equal(host(urp), g[f"{tag}/velocity_periodic_u_r"])
    np.testing.assert_array_equal(host(psi_p), g[f"{tag}/velocity_periodic_psi"])


@pytest.mark.parametrize("tag", ["a", "b"])
def test_forces_and_elasto_against_reference_golden(golden, gk, tag):
    g = golden("kernels")
    R, dx = g[f"{tag}/R"], float(g[f"{tag}/dx"])
    dR = dev(R)
    chi = dev(g[f"{tag}/chi"])
    Fp, Fu = gk.compute_force_on_body(dR, chi, 1.3, 1e4, dev(g[f"{tag}/force_u_z"]), 0.25, 0.7,
                                      2e-3, 1e-4)
    np.testing.assert_allclose([Fp, Fu], g[f"{tag}/force"], rtol=1e-13)
    Uz, Ur = gk.force_projection(2.5, chi, dev(g[f"{tag}/force_u_z"]), dev(g[f"{tag}/proj_u_r"]),
                                 dR)
    np.testing.assert_allclose([Uz, Ur], g[f"{tag}/projection"], rtol=1e-12)
    e1, e2 = dev(g[f"{tag}/eta1"]), dev(g[f"{tag}/eta2"])
    s11, s12, s22, a, b, c, d = (torch.zeros_like(e1) for _ in range(7))
    gk.solid_sigma(s11, s12, s22, 0.37, dx, e1, e2, a, b, c, d)
    for k, v in dict(s11=s11, s12=s12, s22=s22, e1z=a, e1r=b, e2z=c, e2r=d).items():
        np.testing.assert_array_equal(host(v), g[f"{tag}/sigma_{k}"], err_msg=k)
    wv = dev(g[f"{tag}/divtau_in"])
    tz, tr = torch.zeros_like(wv), torch.zeros_like(wv)
    gk.update_vorticity_from_solid_stress(wv, tz, tr, s11, s12, s22, dR, 1.5e-3, dx)
    np.testing.assert_array_equal(host(wv), g[f"{tag}/divtau_w"])
    np.testing.assert_array_equal(host(tz), g[f"{tag}/divtau_tau_z"])
    np.testing.assert_array_equal(host(tr), g[f"{tag}/divtau_tau_r"])


def test_brinkman_kat(gk):
    """The reference's own test: tests/test_kernels/test_brinkmann_penalize.py:6-26."""
    n = 16
    chi = torch.full((n, n), 4.0, dtype=torch.float64, device="cuda")
    z = torch.zeros_like(chi)
    pz, pr = torch.zeros_like(chi), torch.zeros_like(chi)
    gk.brinkmann_penalize(2.0, 3.0, chi, 1.0, 2.0, z, z, pz, pr)
    denom = 1.0 + 2.0 * 3.0 * 4.0
    np.testing.assert_allclose(host(pz), 2.0 * 3.0 * 1.0 * 4.0 / denom * np.ones((n, n)))
    np.testing.assert_allclose(host(pr), 2.0 * 3.0 * 2.0 * 4.0 / denom * np.ones((n, n)))


@pytest.mark.parametrize("nr,nz", [(3, 5), (7, 9), (33, 65), (128, 256), (257, 130)])
def test_eno3_vorticity_matches_oracle_bitwise(nr, nz):
    from pyaxisymflow_gb300.kernels.advect_vorticity_via_eno3 import gen_advect_vorticity_via_eno3
    rng = np.random.default_rng(nr * 1000 + nz)
    dx = 1.0 / nz
    w = rng.standard_normal((nr, nz))
    uz = rng.standard_normal((nr, nz))
    ur = rng.standard_normal((nr, nz))
    # include exact ties u0 == -u1 on some faces
    uz[:, 1::7] = -uz[:, 0:-1:7][:, : uz[:, 1::7].shape[1]]
    dt = 0.1 * dx
    ref = w.copy()
    K.gen_advect_vorticity_via_eno3(dx, nr, nz)(ref, uz, ur, dt)
    tw = dev(w)
    gen_advect_vorticity_via_eno3(dx, nr, nz)(tw, dev(uz), dev(ur), dt)
    np.testing.assert_array_equal(host(tw), ref)


@pytest.mark.parametrize("nr,nz", [(4, 6), (32, 64), (100, 37)])
def test_eno3_refmap_matches_oracle_bitwise(nr, nz):
    from pyaxisymflow_gb300.elasto_kernels.advect_refmap_via_eno3 import gen_advect_refmap_via_eno3
    rng = np.random.default_rng(nr + 7 * nz)
    dx = 1.0 / nz
    e1 = rng.standard_normal((nr, nz))
    e2 = rng.standard_normal((nr, nz))
    uz = rng.standard_normal((nr, nz))
    ur = rng.standard_normal((nr, nz))
    dt = 0.1 * dx
    r1, r2 = e1.copy(), e2.copy()
    K.gen_advect_refmap_via_eno3(dx, nr, nz)(r1, r2, uz, ur, dt)
    t1, t2 = dev(e1), dev(e2)
    gen_advect_refmap_via_eno3(dx, nr, nz)(t1, t2, dev(uz), dev(ur), dt)
    np.testing.assert_array_equal(host(t1), r1)
    np.testing.assert_array_equal(host(t2), r2)


def test_eno3_periodic_variants():
    from pyaxisymflow_gb300.elasto_kernels.advect_refmap_via_eno3 import \
        gen_advect_refmap_via_eno3_periodic
    from pyaxisymflow_gb300.kernels.advect_vorticity_via_eno3 import \
        gen_advect_vorticity_via_eno3_periodic
    from pyaxisymflow_gb300.kernels.periodic_boundary_ghost_comm import (
        gen_periodic_boundary_ghost_comm, gen_periodic_boundary_ghost_comm_eta)
    nr, nz, g = 24, 40, 2
    dx = 1.0 / nz
    rng = np.random.default_rng(3)
    w, uz, ur = (rng.standard_normal((nr, nz)) for _ in range(3))
    e1, e2 = rng.standard_normal((nr, nz)), rng.standard_normal((nr, nz))
    dt = 0.05 * dx
    c_ref = K.gen_periodic_boundary_ghost_comm(g)
    c_ref_eta = K.gen_periodic_boundary_ghost_comm_eta(g, nz * dx, dx)
    rw, ruz, rur = w.copy(), uz.copy(), ur.copy()
    K.gen_advect_vorticity_via_eno3_periodic(dx, nr, nz, c_ref)(rw, ruz, rur, dt)
    tw, tuz, tur = dev(w), dev(uz), dev(ur)
    comm = gen_periodic_boundary_ghost_comm(g)
    gen_advect_vorticity_via_eno3_periodic(dx, nr, nz, comm)(tw, tuz, tur, dt)
    np.testing.assert_array_equal(host(tw), rw)
    np.testing.assert_array_equal(host(tuz), ruz)
    r1, r2, ruz, rur = e1.copy(), e2.copy(), uz.copy(), ur.copy()
    K.gen_advect_refmap_via_eno3_periodic(dx, nr, nz, c_ref, c_ref_eta)(r1, r2, ruz, rur, dt)
    t1, t2, tuz, tur = dev(e1), dev(e2), dev(uz), dev(ur)
    gen_advect_refmap_via_eno3_periodic(dx, nr, nz, comm,
                                        gen_periodic_boundary_ghost_comm_eta(g, nz * dx, dx))(
        t1, t2, tuz, tur, dt)
    np.testing.assert_array_equal(host(t1), r1)
    np.testing.assert_array_equal(host(t2), r2)


@pytest.mark.parametrize("tag", ["a", "b", "tie"])
def test_eno3_matches_reference_expressions(golden, tag):
    """The CUDA ENO3 steps (FP64, through the drop-in closures) against the
    reference's own pystencils kernels evaluated in sympy's term order
    (tests/golden/eno3.npz): a few units in the last place of the field
    magnitude, exact upwind ties included; unbounded and periodic,
    conservative (vorticity) and non-conservative (reference map)."""
    from pyaxisymflow_gb300.elasto_kernels.advect_refmap_via_eno3 import (
        gen_advect_refmap_via_eno3, gen_advect_refmap_via_eno3_periodic)
    from pyaxisymflow_gb300.kernels.advect_vorticity_via_eno3 import (
        gen_advect_vorticity_via_eno3, gen_advect_vorticity_via_eno3_periodic)
    from pyaxisymflow_gb300.kernels.periodic_boundary_ghost_comm import (
        gen_periodic_boundary_ghost_comm, gen_periodic_boundary_ghost_comm_eta)
    g = golden("eno3")
    dx, dt = float(g[f"{tag}/dx"]), float(g[f"{tag}/dt"])
    uz, ur, w0 = g[f"{tag}/u_z"], g[f"{tag}/u_r"], g[f"{tag}/w0"]
    nr, nz = w0.shape

    def close(t, ref):
        scale = max(float(np.abs(ref).max()), 1.0)
        err = float(np.abs(host(t) - ref).max())
        assert err <= 1e-14 * scale, err

    adv = gen_advect_vorticity_via_eno3(dx, nr, nz)
    tw = dev(w0)
    adv(tw, dev(uz), dev(ur), dt)
    close(tw, g[f"{tag}/w_1"])
    adv(tw, dev(uz), dev(ur), dt)
    close(tw, g[f"{tag}/w_2"])
    t1, t2 = dev(g[f"{tag}/eta1_0"]), dev(g[f"{tag}/eta2_0"])
    gen_advect_refmap_via_eno3(dx, nr, nz)(t1, t2, dev(uz), dev(ur), dt)
    close(t1, g[f"{tag}/eta1_1"])
    close(t2, g[f"{tag}/eta2_1"])
    comm = gen_periodic_boundary_ghost_comm(2)
    tw = dev(w0)
    gen_advect_vorticity_via_eno3_periodic(dx, nr, nz, comm)(tw, dev(uz), dev(ur), dt)
    close(tw, g[f"{tag}/w_periodic"])
    t1, t2 = dev(g[f"{tag}/eta1_0"]), dev(g[f"{tag}/eta2_0"])
    gen_advect_refmap_via_eno3_periodic(
        dx, nr, nz, comm, gen_periodic_boundary_ghost_comm_eta(2, nz * dx, dx))(
        t1, t2, dev(uz), dev(ur), dt)
    close(t1, g[f"{tag}/eta1_periodic"])
    close(t2, g[f"{tag}/eta2_periodic"])


def test_spectral_solvers_against_reference_golden(golden):
    from pyaxisymflow_gb300.kernels.FastDiagonalisationPotentialSolver import \
        FastDiagonalisationPotentialSolver
    from pyaxisymflow_gb300.kernels.FastDiagonalisationStokesSolver import \
        FastDiagonalisationStokesSolver
    from pyaxisymflow_gb300.kernels.implicit_diffusion_solver import \
        ImplicitEulerDiffusionStepper
    g = golden("solvers")
    rhs, dx = g["rhs"], float(g["dx"])
    nr, nz = rhs.shape
    for bc in (K.NEUMANN_ZR, K.NEUMANN_R_PERIODIC_Z):
        s = FastDiagonalisationStokesSolver(nr, nz, dx, bc_type=bc)
        psi = torch.zeros((nr, nz), dtype=torch.float64, device="cuda")
        s.solve(psi, dev(rhs))
        assert rel_l2(host(psi), g[f"stokes/{bc}"]) < SOLVE_RTOL, bc
    # The Neumann-Neumann potential operator has a zero eigenvalue; the
    # reference divides by its rounded value (~1e-12, LAPACK-build dependent),
    # so its output is dominated by that one mode and differs between LAPACK
    # builds (x86 golden vs this machine). Compare with the oracle on this
    # machine instead: same LAPACK, same eigenbases.
    p = FastDiagonalisationPotentialSolver(nr, nz, dx)
    phi = torch.zeros((nr, nz), dtype=torch.float64, device="cuda")
    p.solve(phi, dev(rhs))
    ref_here = np.zeros_like(rhs)
    K.FastDiagonalisationPotentialSolver(nr, nz, dx).solve(ref_here, rhs)
    assert rel_l2(host(phi), ref_here) < SOLVE_RTOL
    dt = float(g["implicit_diffusion_dt"])
    st = ImplicitEulerDiffusionStepper(dt, 1e-2, nr, nz, dx)
    w = dev(rhs)
    st.step(w, dt)
    assert rel_l2(host(w), g["implicit_diffusion"]) < SOLVE_RTOL
    with pytest.raises(ValueError):
        st.step(w, 2 * dt)


@pytest.mark.parametrize("nr,nz", [(32, 64), (64, 128), (128, 256), (256, 512)])
def test_stokes_solve_matches_oracle(nr, nz):
    from pyaxisymflow_gb300.kernels.FastDiagonalisationStokesSolver import \
        FastDiagonalisationStokesSolver
    dx = 1.0 / nz
    rng = np.random.default_rng(nr)
    w = rng.standard_normal((nr, nz))
    ref = np.zeros_like(w)
    K.FastDiagonalisationStokesSolver(nr, nz, dx).solve(ref, w)
    psi = torch.zeros((nr, nz), dtype=torch.float64, device="cuda")
    FastDiagonalisationStokesSolver(nr, nz, dx).solve(psi, dev(w))
    assert rel_l2(host(psi), ref) < SOLVE_RTOL


def test_periodic_solve_on_strided_slice():
    """Periodic examples solve on field[:, g:-g] (a strided view)."""
    from pyaxisymflow_gb300.kernels.FastDiagonalisationStokesSolver import \
        FastDiagonalisationStokesSolver
    nr, nz, g = 24, 44, 2
    dx = 1.0 / (nz - 2 * g)
    rng = np.random.default_rng(9)
    w = rng.standard_normal((nr, nz))
    ref = np.zeros_like(w)
    K.FastDiagonalisationStokesSolver(nr, nz - 2 * g, dx, bc_type=K.NEUMANN_R_PERIODIC_Z).solve(
        ref[:, g:-g], w[:, g:-g])
    tw = dev(w)
    psi = torch.zeros_like(tw)
    FastDiagonalisationStokesSolver(nr, nz - 2 * g, dx, bc_type=K.NEUMANN_R_PERIODIC_Z).solve(
        psi[:, g:-g], tw[:, g:-g])
    out = host(psi)
    assert rel_l2(out[:, g:-g], ref[:, g:-g]) < SOLVE_RTOL
    assert np.all(out[:, :g] == 0) and np.all(out[:, -g:] == 0)


@pytest.mark.parametrize("tag", ["a", "b"])
def test_least_squares_extrapolation_bit_exact(golden, tag):
    from pyaxisymflow_gb300.core.extrapolate_using_least_squares import \
        extrapolate_using_least_squares_till_first_order
    g = golden("lsq")
    cf = torch.tensor(g[f"{tag}/current_flag"], dtype=torch.int16, device="cuda")
    tf = torch.tensor(g[f"{tag}/target_flag"], dtype=torch.int16, device="cuda")
    ex, ey = dev(g[f"{tag}/eta_x_in"]), dev(g[f"{tag}/eta_y_in"])
    sweeps = extrapolate_using_least_squares_till_first_order(
        cf, tf, ex, ey, dev(g[f"{tag}/grid_x"]), dev(g[f"{tag}/grid_y"]))
    assert sweeps > 0
    np.testing.assert_array_equal(cf.cpu().numpy(), g[f"{tag}/current_flag_out"])
    np.testing.assert_array_equal(host(ex), g[f"{tag}/eta_x_out"])
    np.testing.assert_array_equal(host(ey), g[f"{tag}/eta_y_out"])


def test_least_squares_iteration_cap_reports_status():
    """A cell with current=1, target=0 and a known neighbour is re-selected
    forever by the reference's loop; here the sweep cap turns it into an error."""
    from pyaxisymflow_gb300._native import AXI_ERR_NOT_CONVERGED, AxiError
    from pyaxisymflow_gb300.core.extrapolate_using_least_squares import \
        extrapolate_using_least_squares_till_first_order
    n = 16
    cf = torch.zeros((n, n), dtype=torch.int16, device="cuda")
    tf = torch.zeros_like(cf)
    cf[7:9, 7:9] = 1
    tf[7:9, 7:9] = 0
    x = torch.linspace(0, 1, n, dtype=torch.float64, device="cuda")
    ex = torch.zeros((n, n), dtype=torch.float64, device="cuda")
    ey = torch.zeros_like(ex)
    with pytest.raises(AxiError) as e:
        extrapolate_using_least_squares_till_first_order(cf, tf, ex, ey, x, x, max_sweeps=5)
    assert e.value.status == AXI_ERR_NOT_CONVERGED


def test_extrapolate_eta_with_least_squares_matches_oracle():
    from pyaxisymflow_gb300.elasto_kernels.extrapolate_eta_using_least_squares_unb import \
        extrapolate_eta_with_least_squares
    nz, nr = 64, 32
    dx = 1.0 / nz
    z = np.linspace(dx / 2, nz * dx - dx / 2, nz)
    r = np.linspace(dx / 2, nr * dx - dx / 2, nr)
    Z, R = np.meshgrid(z, r)
    phi = -np.sqrt((Z - 0.5) ** 2 + R ** 2) + 0.2
    eta1 = Z + 0.01 * np.sin(3 * R)
    eta2 = R + 0.01 * np.cos(2 * Z)
    inside = phi > 0
    zone = 6 * dx
    r1, r2 = eta1.copy(), eta2.copy()
    K.extrapolate_eta_with_least_squares(inside, phi, r1, r2, np.zeros((2 * nr, nz)),
                                         np.zeros((2 * nr, nz)), np.zeros((2 * nr, nz)), zone, nr,
                                         z)
    t1, t2 = dev(eta1), dev(eta2)
    bufs = [torch.zeros((2 * nr, nz), dtype=torch.float64, device="cuda") for _ in range(3)]
    extrapolate_eta_with_least_squares(torch.tensor(inside, device="cuda"), dev(phi), t1, t2,
                                       *bufs, zone, nr, dev(z))
    np.testing.assert_array_equal(host(t1), r1)
    np.testing.assert_array_equal(host(t2), r2)


@pytest.mark.parametrize("nr,nz", [(20, 28), (128, 256)])
def test_f32_kernels_close_to_fp64_oracle(gk, nr, nz):
    rng = np.random.default_rng(nr)
    dx = 1.0 / nz
    z = np.linspace(dx / 2, nz * dx - dx / 2, nz)
    r = np.linspace(dx / 2, nr * dx - dx / 2, nr)
    Z, R = np.meshgrid(z, r)
    psi = rng.standard_normal((nr, nz))
    uz, ur = np.zeros_like(psi), np.zeros_like(psi)
    K.compute_velocity_from_psi_unb(uz, ur, psi, R, dx)
    f = torch.float32
    tuz, tur = torch.zeros((nr, nz), dtype=f, device="cuda"), torch.zeros((nr, nz), dtype=f,
                                                                          device="cuda")
    gk.compute_velocity_from_psi_unb(tuz, tur, dev(psi, f), dev(R, f), dx)
    assert rel_l2(host(tuz), uz) < F32_RTOL and rel_l2(host(tur), ur) < F32_RTOL
    w = rng.standard_normal((nr, nz))
    ref = w.copy()
    K.diffusion_RK2_unb(ref, np.zeros_like(w), R, 1e-2, 0.2 * dx * dx / 1e-2, dx)
    tw = dev(w, f)
    gk.diffusion_RK2_unb(tw, torch.zeros_like(tw), dev(R, f), 1e-2, 0.2 * dx * dx / 1e-2, dx)
    assert rel_l2(host(tw), ref) < F32_RTOL
    from pyaxisymflow_gb300.kernels.advect_vorticity_via_eno3 import gen_advect_vorticity_via_eno3
    ref = w.copy()
    K.gen_advect_vorticity_via_eno3(dx, nr, nz)(ref, uz / 10, ur / 10, 0.1 * dx)
    tw = dev(w, f)
    gen_advect_vorticity_via_eno3(dx, nr, nz)(tw, dev(uz / 10, f), dev(ur / 10, f), 0.1 * dx)
    assert rel_l2(host(tw), ref) < F32_RTOL


def test_errors_are_raised(gk):
    from pyaxisymflow_gb300._native import AxiError
    t = torch.zeros((2, 2), dtype=torch.float64, device="cuda")
    with pytest.raises(AxiError):
        gk.compute_velocity_from_psi_unb(t, t, t, t, 0.1)
    with pytest.raises(ValueError):
        gk.compute_velocity_from_psi_unb(t.cpu(), t, t, t, 0.1)
    with pytest.raises(TypeError):
        gk.brinkmann_penalize(1.0, 1.0, t, 0.0, 0.0, t, t, t, t.float())
