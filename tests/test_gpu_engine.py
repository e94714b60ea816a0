"""The fused step engine against the oracle; alone vs batched; FP32 accuracy."""
import numpy as np
import pytest
import torch

from oracle import kernels as K
from oracle import simulation as sim

pytestmark = pytest.mark.gpu


def rel_l2(a, b):
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))


def oracle_case(c):
    return sim.RigidSphereCase(nz=c.nz, nr=c.nr, dx=c.dx, z_cm=c.z_cm, r_sphere=c.r_sphere,
                               U0=c.U0, Re=c.Re, lam=c.lam, cfl=c.cfl, kill_width=c.kill_width,
                               ramp=c.ramp, noise=c.noise, seed=c.seed)


def run_oracle(c, steps):
    oc = oracle_case(c)
    st, coords = sim.rigid_sphere_init(oc, K)
    solver = K.FastDiagonalisationStokesSolver(oc.nr, oc.nz, oc.dx)
    adv = K.gen_advect_vorticity_via_eno3(oc.dx, oc.nr, oc.nz)
    hist = []
    for _ in range(steps):
        sim.rigid_sphere_step(oc, st, coords, solver, adv, K)
        hist.append((st.dt, st.Cd))
    return st, np.array(hist)


@pytest.mark.parametrize("dct", [False, True])
@pytest.mark.parametrize("nz,nr,steps", [(64, 32, 40), (512, 256, 25)])
def test_engine_f64_matches_oracle(nz, nr, steps, dct):
    """The plain FP64 engine against the oracle, with the z products dense (the
    reference's own form, 1e-12) and as FP64 DCTs. The DCT uses the exact
    eigenvectors and eigenvalues of the z operator; the reference uses the
    ones LAPACK computes, whose low modes carry errors of about
    eps ||A|| / gap (1e-12 relative on one 512 x 256 solve against an exact
    DCT-basis solve in numpy, both with discrete-operator residuals of 2e-11):
    over the steps the two differ by up to a few 1e-12, so the DCT variant is
    held to 2e-11."""
    from pyaxisymflow_gb300.engine import RigidBodyCase, RigidEnsemble
    c = RigidBodyCase(nz=nz, nr=nr, dx=2.0 / nz, r_sphere=max(0.0625, 4 * 2.0 / nz))
    ref, hist = run_oracle(c, steps)
    e = RigidEnsemble([c], precision="f64", history_steps=steps, dct=dct)
    assert e.dct == dct
    e.step(steps)
    torch.cuda.synchronize()
    assert e.status()[0] == 0
    for name, mine, theirs in (("omega", e.fields[0]["omega"], ref.vorticity),
                               ("psi", e.fields[0]["psi"], ref.psi),
                               ("u_z", e.fields[0]["u_z"], ref.u_z),
                               ("u_r", e.fields[0]["u_r"], ref.u_r)):
        err = rel_l2(mine.cpu().numpy(), theirs)
        assert err < (2e-11 if dct else 1e-12), (name, err)
    h = e.history[0].cpu().numpy()
    np.testing.assert_allclose(h[:, 0], hist[:, 0], rtol=1e-12)
    np.testing.assert_allclose(h[:, 1], hist[:, 1], rtol=1e-10, atol=1e-12)
    assert abs(e.time()[0] - ref.t) <= 1e-12 * ref.t


def test_engine_alone_equals_in_the_mix():
    """Each case's result is bit-identical alone and batched with others."""
    from pyaxisymflow_gb300.engine import RigidBodyCase, RigidEnsemble
    cases = [RigidBodyCase(nz=128, nr=64, dx=2.0 / 128, r_sphere=0.1, Re=50.0, seed=1),
             RigidBodyCase(nz=96, nr=48, dx=2.0 / 96, r_sphere=0.12, Re=200.0, seed=2),
             RigidBodyCase(nz=256, nr=128, dx=2.0 / 256, r_sphere=0.08, Re=100.0, seed=3,
                           body="spheroid", aspect=1.5)]
    for prec in ("f64", "f32"):
        mix = RigidEnsemble(cases, precision=prec)
        mix.step(15)
        for k, c in enumerate(cases):
            alone = RigidEnsemble([c], precision=prec)
            alone.step(15)
            torch.cuda.synchronize()
            assert torch.equal(alone.fields[0]["omega"], mix.fields[k]["omega"]), (prec, k)
            assert torch.equal(alone.state[0], mix.state[k]), (prec, k)


def test_engine_graph_replay_equals_eager():
    from pyaxisymflow_gb300.engine import RigidBodyCase, RigidEnsemble
    c = RigidBodyCase(nz=128, nr=64, dx=2.0 / 128, r_sphere=0.1)
    a = RigidEnsemble([c], precision="f64")
    a.step(6)
    b = RigidEnsemble([c], precision="f64")
    b.capture(steps_per_replay=3)
    b.replay()
    b.replay()
    torch.cuda.synchronize()
    assert torch.equal(a.fields[0]["omega"], b.fields[0]["omega"])
    assert torch.equal(a.state, b.state)


@pytest.mark.parametrize("precision", ["f64", "f32"])
def test_vorticity_arena_host_round_trip(precision):
    """All cases' vorticity moves in one copy each way (store_vorticity /
    load_vorticity); loading is equivalent to replacing each case's omega."""
    from pyaxisymflow_gb300.engine import RigidBodyCase, RigidEnsemble
    cases = [RigidBodyCase(nz=64, nr=32, dx=2.0 / 64, r_sphere=0.125, seed=1),
             RigidBodyCase(nz=128, nr=64, dx=2.0 / 128, r_sphere=0.1, seed=2),
             RigidBodyCase(nz=96, nr=48, dx=2.0 / 96, r_sphere=0.1, seed=3)]
    a = RigidEnsemble(cases, precision=precision)
    b = RigidEnsemble(cases, precision=precision)
    a.step(3)
    b.step(3)
    host = torch.empty(a.omega_arena.numel(), dtype=a.dtype, pin_memory=True)
    a.store_vorticity(host)
    torch.cuda.synchronize()
    off = 0
    for k, c in enumerate(cases):
        n = c.nr * c.nz
        assert torch.equal(host[off:off + n].view(c.nr, c.nz), a.fields[k]["omega"].cpu())
        off += n
    assert off == host.numel()
    # perturb on the host, load into a; the same values per case into b
    host.mul_(1.5)
    a.load_vorticity(host)
    off = 0
    for k, c in enumerate(cases):
        n = c.nr * c.nz
        b.set_vorticity(k, host[off:off + n].view(c.nr, c.nz).cuda())
        off += n
    a.step(2)
    b.step(2)
    torch.cuda.synchronize()
    for k in range(len(cases)):
        assert torch.equal(a.fields[k]["omega"], b.fields[k]["omega"]), k
    assert torch.equal(a.state, b.state)
    # the arena survives a membership change: case 1 leaves, the others keep
    # their vorticity
    keep = [a.fields[0]["omega"].clone(), a.fields[2]["omega"].clone()]
    a.remove_case(a.members[1])
    assert a.omega_arena.numel() == sum(c.nr * c.nz for c in (cases[0], cases[2]))
    assert torch.equal(a.fields[0]["omega"], keep[0])
    assert torch.equal(a.fields[1]["omega"], keep[1])


@pytest.mark.parametrize("precision", ["f64", "f32"])
def test_host_pipeline_matches_single_ensemble(precision):
    """Overlapped host transfers over case groups give every case the same
    result as one ensemble round-tripping its vorticity through the host."""
    from pyaxisymflow_gb300.engine import ST_WORDS, HostPipeline, RigidBodyCase, RigidEnsemble
    cases = [RigidBodyCase(nz=64 * (1 + k % 3), nr=32 * (1 + k % 3), dx=2.0 / (64 * (1 + k % 3)),
                           r_sphere=0.125, seed=10 + k) for k in range(7)]
    pipe = HostPipeline(cases, groups=3, precision=precision)
    assert sorted(k for idx in pipe.index for k in idx) == list(range(len(cases)))
    ref = RigidEnsemble(cases, precision=precision)
    host = pipe.host_buffer()
    state = torch.empty((len(cases), ST_WORDS), dtype=torch.float64, pin_memory=True)
    # two direct steps, then one captured step (capture records without running)
    for _ in range(2):
        pipe.step(host, state)
        pipe.synchronize()
    pipe.capture(host, state)
    pipe.replay()
    pipe.synchronize()
    ref.step(3)
    torch.cuda.synchronize()
    row = 0
    for g, idx in enumerate(pipe.index):
        a = pipe.offsets[g]
        for k in idx:
            c = cases[k]
            n = c.nr * c.nz
            assert torch.equal(host[a:a + n].view(c.nr, c.nz), ref.fields[k]["omega"].cpu()), k
            assert torch.equal(state[row], ref.state[k].cpu()), k
            a += n
            row += 1


def test_host_pipeline_pipelined_steps_match_single_ensemble():
    """Per-group step graphs replayed without a barrier between steps (a
    group's next step follows only its own previous one), the host reading
    each step's state blocks one step behind: every case ends where one
    ensemble (one plan) does, and each step's state blocks are that step's."""
    from pyaxisymflow_gb300.engine import ST_T, ST_WORDS, HostPipeline, RigidBodyCase, \
        RigidEnsemble
    cases = [RigidBodyCase(nz=64 * (1 + k % 3), nr=32 * (1 + k % 3), dx=2.0 / (64 * (1 + k % 3)),
                           r_sphere=0.125, seed=20 + k) for k in range(18)]
    pipe = HostPipeline(cases, groups=2, precision="f32")
    # each host group of 9 cases steps as two plan groups of its own: the
    # captured group graphs hold the nested fork
    assert all(e.n_plans == 2 for e in pipe.ensembles)
    ref = RigidEnsemble(cases, precision="f32")
    ref.set_tuning({"plan_groups": 1})
    host = pipe.host_buffer()
    states = [torch.empty((len(cases), ST_WORDS), dtype=torch.float64, pin_memory=True)
              for _ in range(2)]
    pipe.capture_pipelined(host, states)
    order = [k for idx in pipe.index for k in idx]
    steps = 6
    seen = []
    for k in range(steps):
        pipe.replay_step(k)
        if k:
            seen.append(states[pipe.wait_step(k - 1)].clone())
    seen.append(states[pipe.wait_step(steps - 1)].clone())
    pipe.synchronize()
    for k in range(steps):
        ref.step(1)
        want = ref.state.cpu()
        for row, c in enumerate(order):
            assert torch.equal(seen[k][row], want[c]), (k, c)
    row = 0
    for g, idx in enumerate(pipe.index):
        a = pipe.offsets[g]
        for c in idx:
            n = cases[c].nr * cases[c].nz
            assert torch.equal(host[a:a + n].view(cases[c].nr, cases[c].nz),
                               ref.fields[c]["omega"].cpu()), c
            a += n
    assert float(seen[-1][0, ST_T]) > float(seen[0][0, ST_T])


@pytest.mark.parametrize("precision", ["f32", "f64"])
def test_plan_groups_give_identical_results(precision):
    """Nine uneven cases as one plan, as the automatic split (two plans on
    forked streams) and as four plans, stepped directly and from a captured
    graph: every field and state block equal."""
    from pyaxisymflow_gb300.engine import RigidBodyCase, RigidEnsemble
    cases = [RigidBodyCase(nz=64 * (1 + k % 3), nr=32 * (1 + k % 3), dx=2.0 / (64 * (1 + k % 3)),
                           r_sphere=0.125, z_cm=1.2, U0=0.0, ramp=False, sediment=k % 2 == 0,
                           rho_s=2.0, seed=40 + k) for k in range(9)]
    runs = []
    for groups in (1, 0, 4):
        e = RigidEnsemble(cases, precision=precision)
        e.set_tuning({"plan_groups": groups})
        assert e.n_plans == (1 if groups == 1 else (2 if groups == 0 else 4))
        assert sorted(k for p in e.plans for k in p[3]) == list(range(len(cases)))
        e.step(3)
        e.capture(2)
        e.replay()
        torch.cuda.synchronize()
        assert not e.status().any()
        runs.append(e)
    ref = runs[0]
    for e in runs[1:]:
        for a, b in zip(e.fields, ref.fields):
            for k in ("omega", "psi", "u_z", "u_r", "chi"):
                assert torch.equal(a[k], b[k]), k
        assert torch.equal(e.state, ref.state)


def test_engine_dct_z_transform_tracks_fp64():
    """The FP32 engine with the z products as DCTs (dct=True) against the
    FP64 engine, and no worse than the dense tensor-core form."""
    from pyaxisymflow_gb300.engine import RigidBodyCase, RigidEnsemble
    cases = [RigidBodyCase(nz=256, nr=128, dx=2.0 / 256, r_sphere=0.0625, seed=3),
             RigidBodyCase(nz=192, nr=96, dx=2.0 / 192, r_sphere=0.08, seed=4)]
    ref = RigidEnsemble(cases, precision="f64")
    dct = RigidEnsemble(cases, precision="f32", dct=True)
    dense = RigidEnsemble(cases, precision="f32", dct=False)
    assert dct.dct and not dense.dct
    for e in (ref, dct, dense):
        e.step(30)
    torch.cuda.synchronize()
    assert not dct.status().any()
    for k in range(len(cases)):
        for f in ("omega", "psi", "u_z", "u_r"):
            y = ref.fields[k][f].double().cpu().numpy()
            e_dct = rel_l2(dct.fields[k][f].double().cpu().numpy(), y)
            e_dense = rel_l2(dense.fields[k][f].double().cpu().numpy(), y)
            assert e_dct < 1e-5, (k, f, e_dct, e_dense)
            assert e_dct < 2 * e_dense + 1e-6, (k, f, e_dct, e_dense)
    # a grid the transform cannot take is refused, and by default falls back
    odd = RigidBodyCase(nz=100, nr=48, dx=2.0 / 100, r_sphere=0.1)
    with pytest.raises(ValueError, match="no DCT plan"):
        RigidEnsemble([odd], precision="f32", dct=True)
    assert not RigidEnsemble([odd], precision="f32").dct


@pytest.mark.parametrize("nz", [96, 1536, 2048])
def test_engine_dct_paths_agree_with_dense_products(nz):
    """The DCT's other kernel paths (generic length 96, shared-memory Stockham
    for 1536 and 2048) against the dense tensor-core z products."""
    from pyaxisymflow_gb300.engine import RigidBodyCase, RigidEnsemble
    c = RigidBodyCase(nz=nz, nr=nz // 2, dx=2.0 / nz, r_sphere=max(0.0625, 8 * 2.0 / nz),
                      seed=nz)
    a = RigidEnsemble([c], precision="f32", dct=True)
    b = RigidEnsemble([c], precision="f32", dct=False)
    a.step(5)
    b.step(5)
    torch.cuda.synchronize()
    assert not a.status().any()
    for f in ("psi", "u_z", "u_r", "omega"):
        x = a.fields[0][f].double().cpu().numpy()
        y = b.fields[0][f].double().cpu().numpy()
        assert rel_l2(x, y) < 2e-5, (nz, f, rel_l2(x, y))


def test_engine_f32_error_vs_fp64_oracle():
    from pyaxisymflow_gb300.engine import RigidBodyCase, RigidEnsemble
    c = RigidBodyCase(nz=256, nr=128, dx=2.0 / 256, r_sphere=0.0625)
    steps = 50
    ref, _ = run_oracle(c, steps)
    e = RigidEnsemble([c], precision="f32")
    e.step(steps)
    torch.cuda.synchronize()
    errs = {name: rel_l2(e.fields[0][name].double().cpu().numpy(), theirs)
            for name, theirs in (("omega", ref.vorticity), ("psi", ref.psi),
                                 ("u_z", ref.u_z), ("u_r", ref.u_r))}
    print("f32 rel L2 vs FP64 oracle after", steps, "steps:", errs)
    assert max(errs.values()) < 1e-4, errs


def test_engine_f32_tensor_cores_error_vs_fp64_oracle():
    """FP32 engine with the spectral products on tcgen05 (3xTF32): error vs the
    FP64 oracle stays at the FP32 level; same case set alone vs batched."""
    from pyaxisymflow_gb300.engine import RigidBodyCase, RigidEnsemble
    c = RigidBodyCase(nz=256, nr=128, dx=2.0 / 256, r_sphere=0.0625)
    steps = 50
    ref, _ = run_oracle(c, steps)
    e = RigidEnsemble([c], precision="f32", tensor_cores=True)
    e.step(steps)
    torch.cuda.synchronize()
    assert e.status()[0] == 0
    errs = {name: rel_l2(e.fields[0][name].double().cpu().numpy(), theirs)
            for name, theirs in (("omega", ref.vorticity), ("psi", ref.psi),
                                 ("u_z", ref.u_z), ("u_r", ref.u_r))}
    print("f32 tensor-core rel L2 vs FP64 oracle after", steps, "steps:", errs)
    assert max(errs.values()) < 1e-5, errs
    simt = RigidEnsemble([c], precision="f32", tensor_cores=False)
    simt.step(steps)
    d = rel_l2(e.fields[0]["omega"].double().cpu().numpy(),
               simt.fields[0]["omega"].double().cpu().numpy())
    assert d < 1e-5, d


@pytest.mark.parametrize("precision,tol", [("f64", 1e-12), ("f32", 1e-4)])
def test_engine_sedimenting_sphere_matches_oracle(precision, tol):
    """Freely sedimenting sphere (examples/SedimentingRigidSphere/falling_rigid_sphere.py):
    moving mask, FP64 force integral and body ODE on the device. The FP64
    engine follows the oracle to 1e-12 (body position, velocity and
    vorticity); one double ulp of noise in the oracle's own initial
    vorticity moves its result by 1e-15 over these 40 steps."""
    from pyaxisymflow_gb300.engine import (ST_UBODY, ST_ZCM, RigidBodyCase, RigidEnsemble)
    nz, nr, steps = 128, 64, 40
    oc = sim.SedimentingCase(nz=nz, nr=nr, dx=1.0 / nz, r_sphere=0.08, z_cm=0.6, nu=0.01,
                             rho_s=1.5)
    w0 = 1e-3 * np.random.default_rng(5).standard_normal((nr, nz))
    st, coords = sim.sedimenting_init(oc, K, vorticity=w0)
    solver = K.FastDiagonalisationStokesSolver(oc.nr, oc.nz, oc.dx)
    adv = K.gen_advect_vorticity_via_eno3(oc.dx, oc.nr, oc.nz)
    for _ in range(steps):
        sim.sedimenting_step(oc, st, coords, solver, adv, K)
    c = RigidBodyCase(nz=nz, nr=nr, dx=oc.dx, z_cm=oc.z_cm, r_sphere=oc.r_sphere, U0=0.0,
                      ramp=False, Re=1.0 * 2 * oc.r_sphere / oc.nu, lam=oc.lam, cfl=oc.cfl,
                      sediment=True, rho_f=oc.rho_f, rho_s=oc.rho_s, gravity=oc.gravity)
    assert abs(c.nu - oc.nu) < 1e-15
    e = RigidEnsemble([c], precision=precision, initial_vorticity=[w0])
    e.step(steps)
    torch.cuda.synchronize()
    assert e.status()[0] == 0
    s = e.state[0].cpu().numpy()
    assert abs(s[ST_ZCM] - st.part_Z_cm) <= tol * abs(st.part_Z_cm)
    assert abs(s[ST_UBODY] - st.U_z_cm_part) <= tol * abs(st.U_z_cm_part) + 1e-14
    err = rel_l2(e.fields[0]["omega"].double().cpu().numpy(), st.vorticity)
    assert err < (tol if precision == "f64" else tol * 10), err
    chi_err = np.abs(e.fields[0]["chi"].double().cpu().numpy() - st.char_func).max()
    assert chi_err < (1e-12 if precision == "f64" else 1e-5), chi_err


def test_engine_refined_solve_matches_fp64_solve():
    """The FP32 engine's solve with one refinement step per solve, started
    from the previous step's psi (AXI_PLAN_REFINE, the default with the DCT z
    transform) and kept as the pair psi + psi_lo: after a few steps, psi of
    the kill + transform phases equals the FP64 solve of the same (float)
    vorticity to better than float resolution, closer than the plain FP32
    solve."""
    from pyaxisymflow_gb300.engine import RigidBodyCase, RigidEnsemble
    from pyaxisymflow_gb300.kernels.FastDiagonalisationStokesSolver import \
        FastDiagonalisationStokesSolver
    cases = [RigidBodyCase(nz=256, nr=128, dx=2.0 / 256, r_sphere=0.08, Re=300.0, seed=3),
             RigidBodyCase(nz=768, nr=384, dx=2.0 / 768, r_sphere=0.06, z_cm=1.4, U0=0.0,
                           ramp=False, sediment=True, rho_s=2.0, Re=500.0, seed=4)]
    errs = {}
    for refine in (True, False):
        e = RigidEnsemble(cases, precision="f32", dct=True, refine=refine)
        assert e.refine == refine
        e.step(30)
        e.phase(0)      # kill
        e.phase(1)      # transform: psi of the current vorticity
        torch.cuda.synchronize()
        assert not e.status().any()
        worst = 0.0
        for k, c in enumerate(cases):
            s64 = FastDiagonalisationStokesSolver(c.nr, c.nz, c.dx, device="cuda")
            psi = torch.zeros((c.nr, c.nz), dtype=torch.float64, device="cuda")
            s64.solve(psi, e.fields[k]["omega"].double())
            mine = e.fields[k]["psi"].double()
            if refine:
                mine = mine + e.fields[k]["psi_lo"].double()
            worst = max(worst, rel_l2(mine.cpu().numpy(), psi.cpu().numpy()))
        errs[refine] = worst
    print("psi rel L2 vs the FP64 solve of the same vorticity:", errs)
    assert errs[True] < 1e-7, errs
    assert errs[True] < errs[False], errs


def test_engine_f32_drift_after_2000_steps_on_the_hardest_cases():
    """The FP32 engine (DCT z transforms, tcgen05 radial products, one
    refinement step per solve) against the FP64 engine (within 1e-12 of the
    oracle) after config 4's 2000 steps, on the two ensemble cases with the
    largest vorticity drift (case 9: 512 x 256, Re 755; case 14: 256 x 128,
    Re 301): psi and velocity within 1e-5, vorticity within 2e-5 (measured
    1.15e-5 and 9.5e-6; a float-sized change of the sphere radius moves the
    FP64 vorticity by 5e-6 over the same steps)."""
    import bench
    from pyaxisymflow_gb300.engine import RigidEnsemble
    cases = bench.ensemble_cases("ensemble64")
    sel = [cases[9], cases[14]]
    w0 = [c.noise * np.random.default_rng(c.seed).standard_normal((c.nr, c.nz)) for c in sel]
    a = RigidEnsemble(sel, precision="f64", initial_vorticity=w0)
    b = RigidEnsemble(sel, precision="f32", initial_vorticity=w0)
    assert b.refine and b.dct and b.tensor_cores
    a.step(2000)
    b.step(2000)
    torch.cuda.synchronize()
    assert not a.status().any() and not b.status().any()
    for k in range(len(sel)):
        fa, fb = a.fields[k], b.fields[k]
        errs = {}
        for n in ("omega", "psi", "u_z", "u_r"):
            ref = fa[n].double()
            got = fb[n].double()
            if n == "psi":
                got = got + fb["psi_lo"].double()
            errs[n] = float(torch.linalg.norm(got - ref) / torch.linalg.norm(ref))
        assert errs["omega"] < 2e-5 and max(errs["psi"], errs["u_z"], errs["u_r"]) < 1e-5, errs
