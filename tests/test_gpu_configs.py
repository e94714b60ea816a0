"""Parity at the configured sizes and horizons of the benchmark workloads.

These run the oracle (numpy FP64, the reference's algorithm) for minutes of
CPU time: config 1 (512 x 256 rigid sphere, 1000 steps), config 4
(sedimenting spheres of the seeded ensemble at 256 x 128 and 1024 x 512, 200
steps), config 2 (soft sphere at 1024 x 512, 50 steps) and config 3 (the
2048 x 1024 periodic streamfunction solve with 32 vortex rings).

Tolerances: the FP64 engine with dense z products follows the oracle's
products and order, 1e-12; with the z products as DCTs it uses the exact
eigenbasis of the z operator where the reference uses LAPACK's (1e-12 apart
per solve on these grids), 2e-11. The soft loop is held to the oracle's own
floor, measured in the test (see there).
"""
import numpy as np
import pytest
import torch

from oracle import kernels as K
from oracle import simulation as sim

pytestmark = pytest.mark.gpu

FIELDS = ("omega", "psi", "u_z", "u_r")


def rel_l2(a, b):
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))


def check(ens, oracle_state, tol_dense, tol_dct, label):
    theirs = {"omega": oracle_state.vorticity, "psi": oracle_state.psi,
              "u_z": oracle_state.u_z, "u_r": oracle_state.u_r}
    for e in ens:
        tol = tol_dct if e.dct else tol_dense
        for f in FIELDS:
            err = rel_l2(e.fields[0][f].cpu().numpy(), theirs[f])
            assert err < tol, (label, "dct" if e.dct else "dense", f, err)


def test_config1_rigid_sphere_512x256_1000_steps():
    """Config 1: flow past a rigid sphere, 512 x 256, Re 100, 1000 steps from
    seeded noise, FP64 engine (dense and DCT z products) against the oracle."""
    from pyaxisymflow_gb300.engine import RigidBodyCase, RigidEnsemble
    steps = 1000
    c = RigidBodyCase()
    oc = sim.RigidSphereCase(nz=c.nz, nr=c.nr, dx=c.dx, z_cm=c.z_cm, r_sphere=c.r_sphere,
                             U0=c.U0, Re=c.Re, lam=c.lam, cfl=c.cfl, kill_width=c.kill_width,
                             ramp=c.ramp, noise=c.noise, seed=c.seed)
    st, coords = sim.rigid_sphere_init(oc, K)
    solver = K.FastDiagonalisationStokesSolver(oc.nr, oc.nz, oc.dx)
    adv = K.gen_advect_vorticity_via_eno3(oc.dx, oc.nr, oc.nz)
    ens = [RigidEnsemble([c], precision="f64", dct=dct) for dct in (False, True)]
    for _ in range(steps):
        sim.rigid_sphere_step(oc, st, coords, solver, adv, K)
    for e in ens:
        e.step(steps)
    torch.cuda.synchronize()
    assert not any(e.status().any() for e in ens)
    check(ens, st, 1e-12, 2e-11, "config 1")
    for e in ens:
        assert abs(e.state[0, 2].item() - st.Cd) <= 1e-10 * abs(st.Cd)


@pytest.mark.parametrize("index", [14, 9, 37, 49])
def test_config4_sedimenting_sphere_200_steps(index):
    """Config 4: freely sedimenting spheres of the seeded 64-case ensemble, one
    per grid size (case 14: 256 x 128, Re 301, radius 0.043; case 9: 512 x 256,
    Re 755, radius 0.087; case 37: 768 x 384, Re 622, radius 0.118; case 49:
    1024 x 512, Re 871, radius 0.093), 200 steps, FP64 engine against the
    oracle: fields, body position and velocity."""
    import bench
    from pyaxisymflow_gb300.engine import ST_UBODY, ST_ZCM, RigidEnsemble
    c = bench.ensemble_cases("ensemble64")[index]
    steps = 200
    oc = sim.SedimentingCase(nz=c.nz, nr=c.nr, dx=c.dx, z_cm=c.z_cm, r_sphere=c.r_sphere,
                             rho_f=c.rho_f, rho_s=c.rho_s, nu=c.nu, lam=c.lam, cfl=c.cfl,
                             kill_width=c.kill_width, gravity=c.gravity)
    w0 = c.noise * np.random.default_rng(c.seed).standard_normal((c.nr, c.nz))
    st, coords = sim.sedimenting_init(oc, K, vorticity=w0)
    solver = K.FastDiagonalisationStokesSolver(oc.nr, oc.nz, oc.dx)
    adv = K.gen_advect_vorticity_via_eno3(oc.dx, oc.nr, oc.nz)
    ens = [RigidEnsemble([c], precision="f64", dct=dct) for dct in (False, True)]
    for _ in range(steps):
        sim.sedimenting_step(oc, st, coords, solver, adv, K)
    for e in ens:
        e.step(steps)
    torch.cuda.synchronize()
    check(ens, st, 1e-12, 2e-11, f"config 4 case {index}")
    for e in ens:
        s = e.state[0].cpu().numpy()
        tol = 2e-11 if e.dct else 1e-12
        assert abs(s[ST_ZCM] - st.part_Z_cm) <= tol * abs(st.part_Z_cm)
        assert abs(s[ST_UBODY] - st.U_z_cm_part) <= tol * abs(st.U_z_cm_part)


def _soft_oracle(case, steps, psi_noise_seed=None):
    """The oracle's soft loop; with `psi_noise_seed`, psi is moved by one
    double ulp at a seeded random third of its cells after every solve (the
    size of difference a different BLAS summation order makes)."""
    st, coords = sim.soft_sphere_init(case, K)
    solver = K.FastDiagonalisationStokesSolver(case.nr, case.nz, case.dx)
    if psi_noise_seed is not None:
        rng = np.random.default_rng(psi_noise_seed)
        plain = solver.solve

        def solve(solution_field, rhs_field):
            plain(solution_field=solution_field, rhs_field=rhs_field)
            solution_field *= 1 + np.finfo(float).eps * rng.choice([-1.0, 0.0, 1.0],
                                                                   solution_field.shape)
        solver.solve = solve
    aw = K.gen_advect_vorticity_via_eno3(case.dx, case.nr, case.nz)
    ae = K.gen_advect_refmap_via_eno3(case.dx, case.nr, case.nz)
    for _ in range(steps):
        sim.soft_sphere_step(case, st, coords, solver, aw, ae, K)
    return st


def test_config2_soft_sphere_1024x512_50_steps():
    """Config 2: the soft neo-Hookean sphere loop (reference-map advection,
    level-set pinning, least-squares extrapolation, solid stress, penalised
    forcing) at 1024 x 512, radius 0.1, G 1e-3, U(t) = 0.1 cos(2 pi t), 50 steps, FP64
    through the drop-in kernels (dt formed on the host) and through the
    device-resident engine, each against the oracle's soft loop.

    The loop differentiates eta (close to the coordinates z, r, so of size 1)
    over 2 dx: a difference of one ulp in eta is 1e-13 of the stress, and the
    penalised, stiff loop carries it on. The oracle is run a second time with
    psi moved by one ulp after each solve (what another BLAS summation order
    does); the GPU runs are held to that floor (4x the control's difference,
    or 1e-12 where the control is smaller), and the solid mask chi > 0.5 must
    agree at every cell."""
    import bench
    from pyaxisymflow_gb300.simulation import SoftSphereEngine, SoftSphereSimulation
    steps = 50
    case = bench.soft_case()
    st = _soft_oracle(case, steps)
    control = _soft_oracle(case, steps, psi_noise_seed=7)
    # the host-dt drop-in loop and the device-resident engine
    runs = {"drop-in": SoftSphereSimulation(case, device="cuda"),
            "engine": SoftSphereEngine(case, device="cuda")}
    runs["drop-in"].run(steps)
    runs["engine"].step(steps)
    torch.cuda.synchronize()
    report = {}
    for label, s in runs.items():
        for f, t, ref, ctl in (("omega", s.vorticity, st.vorticity, control.vorticity),
                               ("eta1", s.eta1, st.eta1, control.eta1),
                               ("eta2", s.eta2, st.eta2, control.eta2),
                               ("phi", s.ball_phi, st.ball_phi, control.ball_phi),
                               ("chi", s.ball_char_func, st.ball_char_func,
                                control.ball_char_func)):
            err, floor = rel_l2(t.cpu().numpy(), ref), rel_l2(ctl, ref)
            report[(label, f)] = (err, floor)
            assert err <= max(1e-12, 4 * floor), (label, f, err, floor)
        np.testing.assert_array_equal(s.ball_char_func.cpu().numpy() > 0.5,
                                      st.ball_char_func > 0.5)
        assert abs(s.t - st.t) <= 1e-13 * st.t
    print("config 2, rel L2 vs oracle (GPU, oracle one-ulp control):", report)
    assert runs["engine"].status() == 0
    # the engine with the z products of the solve as FP64 DCTs (exact cosine
    # basis instead of LAPACK's eigenvectors): 2e-11, as the rigid FP64 DCT
    # engine (measured: omega 5.1e-13, eta 3.0e-13, psi 9.4e-12)
    e = SoftSphereEngine(case, device="cuda", dct=True)
    e.step(steps)
    torch.cuda.synchronize()
    for f, t, ref in (("omega", e.vorticity, st.vorticity), ("eta1", e.eta1, st.eta1),
                      ("eta2", e.eta2, st.eta2), ("phi", e.ball_phi, st.ball_phi),
                      ("psi", e.psi, st.psi)):
        err = rel_l2(t.cpu().numpy(), ref)
        assert err < 2e-11, ("dct", f, err)
    assert e.status() == 0


def test_config3_periodic_poisson_2048x1024():
    """Config 3: 2048 x 1024 streamfunction solve, periodic z, 32 seeded
    Gaussian vortex rings: the FP32 tensor-core solve with one refinement step
    against the FP64 solve (itself within 1e-12 of the oracle), psi to 1e-8;
    velocities by the FP32 stencil from psi as a float pair against the FP64
    ones, 1e-5 (the mixed-precision bound)."""
    import bench
    from pyaxisymflow_gb300.kernels.compute_velocity_from_psi import \
        compute_velocity_from_psi_unb
    from pyaxisymflow_gb300.kernels.FastDiagonalisationStokesSolver import \
        FastDiagonalisationStokesSolver
    nz, nr = 2048, 1024
    dx = 1.0 / nr
    bc = "homogenous_neumann_along_r_and_periodic_along_z"
    w, Z, R = bench.vortex_rings(nr, nz, dx)
    tw = torch.tensor(w, dtype=torch.float64, device="cuda")
    s64 = FastDiagonalisationStokesSolver(nr, nz, dx, bc_type=bc, device="cuda")
    s32 = FastDiagonalisationStokesSolver(nr, nz, dx, bc_type=bc, device="cuda",
                                          real_dtype=np.float32, refine=1)
    p64, p32 = torch.zeros_like(tw), torch.zeros_like(tw)
    s64.solve(p64, tw)
    s32.solve(p32, tw)
    torch.cuda.synchronize()
    assert s32.engine.tc_status() == 0
    e_psi = float(torch.linalg.norm(p32 - p64) / torch.linalg.norm(p64))
    assert e_psi < 1e-8, e_psi
    tR = torch.tensor(R, dtype=torch.float64, device="cuda")
    u64 = [torch.zeros_like(tw) for _ in range(2)]
    compute_velocity_from_psi_unb(u64[0], u64[1], p64, tR, dx)
    # FP32 stencils on psi kept as a float pair hi + lo (as the fused engine
    # keeps it): the velocity differences psi_{j+1} - psi_{j-1} cancel about
    # three digits on this grid, so a single float psi (rounding 6e-8) would
    # leave 1.6e-5 in u; the pair keeps the solve's accuracy
    f32 = dict(dtype=torch.float32, device="cuda")
    hi = p32.float()
    lo = (p32 - hi.double()).float()
    tRf = tR.float()
    parts = []
    for part in (hi, lo):
        u = [torch.zeros((nr, nz), **f32) for _ in range(2)]
        compute_velocity_from_psi_unb(u[0], u[1], part, tRf, dx)
        parts.append(u)
    u32 = [parts[0][k] + parts[1][k] for k in range(2)]
    single = [torch.zeros((nr, nz), **f32) for _ in range(2)]
    compute_velocity_from_psi_unb(single[0], single[1], hi, tRf, dx)
    torch.cuda.synchronize()
    errs = [float(torch.linalg.norm(a.double() - b) / torch.linalg.norm(b))
            for a, b in zip(u32, u64)]
    errs_single = [float(torch.linalg.norm(a.double() - b) / torch.linalg.norm(b))
                   for a, b in zip(single, u64)]
    print("config 3: psi", e_psi, "u (pair)", errs, "u (single float psi)", errs_single)
    # measured: psi 2.3e-9, u_z 6.4e-7, u_r 2.4e-6 (the velocity differentiates
    # the solve's remaining error); a single float psi gives u_r 1.6e-5
    assert max(errs) < 1e-5, errs
