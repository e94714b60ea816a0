"""Host-side scheduling logic of the engine, checked without a GPU: the split
of cases into plan groups, the automatic group count and the launch-choice
records."""
import types

import pytest

from pyaxisymflow_gb300.autotune import CANDIDATES, applicable, mix_key
from pyaxisymflow_gb300.engine import (TUNING_KEYS, AxiTuning, RigidBodyCase, RigidEnsemble,
                                       fill_tuning, split_by_cells)


def bench_like_cases():
    sizes = [256, 512, 768, 1024, 1024, 768, 512, 256, 1024, 512, 256, 768, 1024]
    return [RigidBodyCase(nz=nz, nr=nz // 2, dx=2.0 / nz, seed=k) for k, nz in enumerate(sizes)]


def test_split_by_cells_covers_balances_and_keeps_order():
    cases = bench_like_cases()
    cells = [c.nr * c.nz for c in cases]
    for groups in (1, 2, 3, 4):
        parts = split_by_cells(cases, groups)
        assert len(parts) == groups
        assert sorted(k for p in parts for k in p) == list(range(len(cases)))
        assert all(p == sorted(p) for p in parts)
        loads = [sum(cells[k] for k in p) for p in parts]
        # greedy largest-first: no group exceeds another by more than the
        # largest single case
        assert max(loads) - min(loads) <= max(cells)
    assert split_by_cells(cases, 1) == [list(range(len(cases)))]


def test_split_by_cells_small_inputs():
    one = [RigidBodyCase(nz=64, nr=32, dx=1.0 / 32)]
    assert split_by_cells(one, 4) == [[0]]
    assert split_by_cells(one, 0) == [[0]]
    two = one + [RigidBodyCase(nz=128, nr=64, dx=1.0 / 64)]
    assert split_by_cells(two, 2) in ([[0], [1]], [[1], [0]])


def test_automatic_plan_group_count():
    def count(n, choice=None):
        fake = types.SimpleNamespace(members=[None] * n,
                                     tuning={} if choice is None else {"plan_groups": choice},
                                     AUTO_PLAN_GROUPS=RigidEnsemble.AUTO_PLAN_GROUPS,
                                     AUTO_SPLIT_MIN_CASES=RigidEnsemble.AUTO_SPLIT_MIN_CASES)
        return RigidEnsemble.plan_group_count(fake)
    assert count(1) == 1
    assert count(RigidEnsemble.AUTO_SPLIT_MIN_CASES - 1) == 1
    assert count(RigidEnsemble.AUTO_SPLIT_MIN_CASES) == RigidEnsemble.AUTO_PLAN_GROUPS
    assert count(64) == 2 and count(64, 0) == 2
    assert count(64, 1) == 1 and count(64, 3) == 3
    # never more groups than cases
    assert count(2, 5) == 2


def test_plan_groups_is_a_host_choice():
    """plan_groups is accepted as a launch choice but is not part of the
    plan's axi_tuning record; unknown keys are refused."""
    assert "plan_groups" in TUNING_KEYS and "plan_groups" in CANDIDATES
    t = AxiTuning()
    fill_tuning(t, {"plan_groups": 3, "advect_blocks": 2, "prefetch_waves": -1})
    assert list(t.stencil_blocks_per_sm) == [0, 0, 2]
    assert t.prefetch_waves == -1 and t.reserved == 0
    with pytest.raises(ValueError):
        fill_tuning(AxiTuning(), {"plan_group": 2})


def test_tuner_applicability_and_mix_key():
    ens = types.SimpleNamespace(tensor_cores=True, dct=True, refine=True, precision="f32",
                                n_cases=1, cases=bench_like_cases()[:1])
    assert not applicable(ens, "plan_groups")
    ens.n_cases = 5
    assert applicable(ens, "plan_groups") and applicable(ens, "tc_tile_order")
    ens.cases = bench_like_cases()
    key = mix_key(ens)
    assert key.startswith("f32|tc1|dct1|refine1|")
    assert "512x1024:stream*4" in key and "128x256:stream*3" in key
