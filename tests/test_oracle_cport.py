"""The CPU baseline's C + OpenMP restatement of the grid kernels
(oracle/cstep.c through oracle/cport.py) against the numpy oracle: the same
bits, step after step, for the rigid and the sedimenting sphere loops; and
the baseline runner (child process with fixed thread counts)."""
import json
import os
import subprocess
import sys

import numpy as np
import pytest

from oracle import cport
from oracle import kernels as K
from oracle import simulation as sim

HERE = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
FIELDS = ("vorticity", "psi", "u_z", "u_r", "char_func")


@pytest.mark.parametrize("nz,nr", [(64, 32), (192, 96)])
def test_rigid_sphere_loop_bit_exact(nz, nr):
    c = sim.RigidSphereCase(nz=nz, nr=nr, dx=2.0 / nz, r_sphere=0.1, z_cm=0.5)
    a, coords = sim.rigid_sphere_init(c, K)
    b, _ = sim.rigid_sphere_init(c, K)
    solver = K.FastDiagonalisationStokesSolver(c.nr, c.nz, c.dx)
    adv = K.gen_advect_vorticity_via_eno3(c.dx, c.nr, c.nz)
    ex = cport.CStepScratch(coords[3])
    for _ in range(25):
        sim.rigid_sphere_step(c, a, coords, solver, adv, K)
        cport.rigid_sphere_step(c, b, coords, solver, ex)
        for f in FIELDS:
            np.testing.assert_array_equal(getattr(b, f), getattr(a, f), err_msg=f)
        assert a.Cd == b.Cd and a.dt == b.dt


@pytest.mark.parametrize("nz,nr", [(64, 32), (192, 96)])
def test_sedimenting_sphere_loop_bit_exact(nz, nr):
    oc = sim.SedimentingCase(nz=nz, nr=nr, dx=1.0 / nz, r_sphere=0.08, z_cm=0.6, nu=0.01,
                             rho_s=2.0)
    w0 = 1e-6 * np.random.default_rng(3).standard_normal((nr, nz))
    a, coords = sim.sedimenting_init(oc, K, vorticity=w0)
    b, _ = sim.sedimenting_init(oc, K, vorticity=w0)
    solver = K.FastDiagonalisationStokesSolver(oc.nr, oc.nz, oc.dx)
    adv = K.gen_advect_vorticity_via_eno3(oc.dx, oc.nr, oc.nz)
    ex = cport.CStepScratch(coords[3])
    for _ in range(25):
        sim.sedimenting_step(oc, a, coords, solver, adv, K)
        cport.sedimenting_step(oc, b, coords, solver, ex)
        for f in FIELDS:
            np.testing.assert_array_equal(getattr(b, f), getattr(a, f), err_msg=f)
        assert (a.part_Z_cm, a.U_z_cm_part, a.Cd) == (b.part_Z_cm, b.U_z_cm_part, b.Cd)


def test_thread_count_does_not_change_results():
    c = sim.RigidSphereCase(nz=128, nr=64, dx=2.0 / 128, r_sphere=0.1, z_cm=0.5)
    out = []
    for th in (1, 3):
        cport.set_threads(th)
        st, coords = sim.rigid_sphere_init(c, K)
        solver = K.FastDiagonalisationStokesSolver(c.nr, c.nz, c.dx)
        ex = cport.CStepScratch(coords[3])
        for _ in range(10):
            cport.rigid_sphere_step(c, st, coords, solver, ex)
        out.append(st.vorticity.copy())
    cport.set_threads(os.cpu_count())
    np.testing.assert_array_equal(out[0], out[1])


def test_baseline_runner_child_process(tmp_path):
    params = [dict(nz=64, nr=32, dx=2.0 / 64, z_cm=1.5, r_sphere=0.08, U0=0.0, Re=100.0,
                   nu=0.0016, lam=1e4, cfl=0.1, kill_width=3, ramp=False, noise=1e-6, seed=1,
                   sediment=True, rho_f=1.0, rho_s=2.0, gravity=9.81),
              dict(nz=128, nr=64, dx=2.0 / 128, z_cm=0.5, r_sphere=0.1, U0=1.0, Re=100.0,
                   nu=0.002, lam=1e4, cfl=0.1, kill_width=3, ramp=True, noise=1e-6, seed=2,
                   sediment=False, rho_f=1.0, rho_s=1.1, gravity=9.81)]
    path = tmp_path / "cases.json"
    path.write_text(json.dumps(params))
    env = dict(os.environ, OMP_NUM_THREADS="2", OPENBLAS_NUM_THREADS="2",
               PYTHONDONTWRITEBYTECODE="1")
    r = subprocess.run([sys.executable, "-m", "oracle.cpu_baseline", str(path), "--seconds",
                        "0", "--warmup", "0", "--max-rounds", "3"], cwd=HERE, env=env,
                       capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    rec = json.loads(r.stdout.strip().splitlines()[-1])
    assert rec["rounds"] == 1 and rec["cases"] == 2 and rec["omp_threads"] == 2
    assert rec["cells_per_round"] == 64 * 32 + 128 * 64 and rec["value"] > 0
