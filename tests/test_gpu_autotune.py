"""The launch autotuner: every launch choice gives bit-identical results, the
tuner applies and caches what it picks, and tuning leaves the state as it was."""
import pytest
import torch

pytestmark = pytest.mark.gpu


def mixed_cases():
    from pyaxisymflow_gb300.engine import RigidBodyCase
    return [RigidBodyCase(nz=256, nr=128, dx=2.0 / 256, r_sphere=0.08, Re=300.0, seed=1),
            RigidBodyCase(nz=512, nr=256, dx=2.0 / 512, r_sphere=0.06, z_cm=1.4, U0=0.0,
                          ramp=False, sediment=True, rho_s=2.0, Re=400.0, seed=2),
            RigidBodyCase(nz=768, nr=384, dx=2.0 / 768, r_sphere=0.1, Re=150.0, seed=3)]


def run(choices, steps=6):
    from pyaxisymflow_gb300.engine import RigidEnsemble
    e = RigidEnsemble(mixed_cases(), precision="f32")
    e.set_tuning(choices)
    e.step(steps)
    torch.cuda.synchronize()
    return e


def same(a, b):
    for fa, fb in zip(a.fields, b.fields):
        for k in ("omega", "psi", "psi_lo", "u_z", "u_r", "chi"):
            if not torch.equal(fa[k], fb[k]):
                return k
    return None if torch.equal(a.state, b.state) else "state"


def test_every_launch_choice_gives_identical_results():
    from pyaxisymflow_gb300.autotune import CANDIDATES
    ref = run({})
    assert not ref.status().any()
    for name, values in CANDIDATES.items():
        for v in values[1:]:
            e = run({name: v})
            assert same(e, ref) is None, (name, v, same(e, ref))


def test_tuner_applies_caches_and_restores(tmp_path):
    from pyaxisymflow_gb300.autotune import Autotuner, mix_key
    from pyaxisymflow_gb300.engine import RigidEnsemble
    cache = tmp_path / "tuning.json"
    tuner = Autotuner(cache_path=str(cache), reps=2)
    e = RigidEnsemble(mixed_cases(), precision="f32")
    e.step(2)
    torch.cuda.synchronize()
    before = [f["omega"].clone() for f in e.fields]
    state = e.state.clone()
    best = tuner.tune(e)
    torch.cuda.synchronize()
    # the chosen choices are in force and the state is as before tuning
    assert e.tuning == best
    assert list(e.info.tune.stencil_blocks_per_sm) == [best.get(k, 0) for k in (
        "vel_max_blocks", "penalise_blocks", "advect_blocks")]
    assert all(torch.equal(b, f["omega"]) for b, f in zip(before, e.fields))
    assert torch.equal(state, e.state)
    assert tuner.last["tuned_ms"] <= tuner.last["default_ms"]
    # the same mix again: from the cache (memory and file), no measurement
    n = tuner.measurements
    e2 = RigidEnsemble(mixed_cases(), precision="f32")
    assert tuner.tune(e2) == best and tuner.measurements == n and tuner.last["cached"]
    assert Autotuner(cache_path=str(cache)).cache[mix_key(e2)] == best
    # tuned and untuned runs continue identically
    e.step(4)
    ref = RigidEnsemble(mixed_cases(), precision="f32")
    ref.step(6)
    torch.cuda.synchronize()
    assert same(e, ref) is None
