"""Full per-timestep loops on the GPU against the golden vectors and the oracle."""
import numpy as np
import pytest
import torch

from oracle import kernels as K
from oracle import simulation as sim

pytestmark = pytest.mark.gpu


def rel_l2(a, b):
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))


def test_rigid_sphere_loop_against_golden(golden):
    from pyaxisymflow_gb300.simulation import RigidSphereSimulation
    g = golden("steps")
    case = sim.RigidSphereCase(nz=64, nr=32, dx=2.0 / 64, r_sphere=0.125, z_cm=0.5)
    s = RigidSphereSimulation(case, device="cuda")
    np.testing.assert_array_equal(s.vorticity.cpu().numpy(), g["rigid/omega0"])
    np.testing.assert_array_equal(s.char_func.cpu().numpy() > 0.5, g["rigid/chi"] > 0.5)
    dts = []
    for n in range(40):
        s.step()
        dts.append(s.dt)
        if n + 1 in (1, 10, 40):
            for f, t in (("omega", s.vorticity), ("psi", s.psi), ("u_z", s.u_z), ("u_r", s.u_r)):
                err = rel_l2(t.cpu().numpy(), g[f"rigid/{f}_{n + 1}"])
                assert err < 1e-12, (f, n + 1, err)
    np.testing.assert_allclose(dts, g["rigid/dt"], rtol=1e-13)


@pytest.mark.parametrize("steps", [20])
def test_rigid_sphere_full_size_against_oracle(steps):
    """512 x 256 (z in [0, 2], r in [0, 1], dx = 1/256, sphere 0.0625 at z = 0.5)."""
    from pyaxisymflow_gb300.simulation import RigidSphereSimulation
    case = sim.RigidSphereCase()
    st, coords = sim.rigid_sphere_init(case, K)
    solver = K.FastDiagonalisationStokesSolver(case.nr, case.nz, case.dx)
    adv = K.gen_advect_vorticity_via_eno3(case.dx, case.nr, case.nz)
    s = RigidSphereSimulation(case, device="cuda")
    for _ in range(steps):
        sim.rigid_sphere_step(case, st, coords, solver, adv, K)
        s.step()
    for f, t, ref in (("omega", s.vorticity, st.vorticity), ("psi", s.psi, st.psi),
                      ("u_z", s.u_z, st.u_z), ("u_r", s.u_r, st.u_r)):
        err = rel_l2(t.cpu().numpy(), ref)
        assert err < 1e-12, (f, err)
    assert abs(s.Cd - st.Cd) <= 1e-10 * abs(st.Cd)


def test_soft_sphere_loop_against_golden(golden):
    """Elasto path end to end: eta advection, level-set pinning, least-squares
    extrapolation, neo-Hookean stress and its curl, tether penalisation."""
    from pyaxisymflow_gb300.simulation import SoftSphereSimulation
    g = golden("soft")
    case = sim.SoftSphereCase(nz=64, nr=32, dx=1.0 / 64, r_ball=0.15, lam=1e6)
    s = SoftSphereSimulation(case, device="cuda")
    s.run(12)
    for f, t in (("omega", s.vorticity), ("eta1", s.eta1), ("eta2", s.eta2),
                 ("phi", s.ball_phi), ("chi", s.ball_char_func)):
        err = rel_l2(t.cpu().numpy(), g[f"soft/{f}_12"])
        assert err < 1e-12, (f, err)
    assert abs(s.t - float(g["soft/t_12"])) <= 1e-13 * float(g["soft/t_12"])
