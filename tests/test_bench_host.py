"""Host-side logic of the benchmark, checked without a GPU: the seeded
workload, the selection of the hardest cases for the accuracy leg and the
summary of the clock samples taken during the timed region."""
import bench


def test_ensemble_workload_is_seeded_and_as_described():
    a = bench.ensemble_cases("ensemble64")
    b = bench.ensemble_cases("ensemble64")
    assert len(a) == 64
    assert [(c.nz, c.Re, c.r_sphere, c.rho_s) for c in a] == \
        [(c.nz, c.Re, c.r_sphere, c.rho_s) for c in b]
    assert {c.nz for c in a} == {256, 512, 768, 1024}
    for c in a:
        assert c.nr == c.nz // 2 and abs(c.dx - 2.0 / c.nz) < 1e-15
        assert 10.0 <= c.Re <= 1000.0 and 0.04 <= c.r_sphere <= 0.12
        assert 1.5 <= c.rho_s <= 4.0 and c.sediment
    assert sum(c.nr * c.nz for c in a) == 18415616
    assert len(bench.ensemble_cases("sphere512")) == 1


def test_accuracy_cases_pick_the_hardest_per_grid():
    cases = bench.ensemble_cases("ensemble64")
    idx = bench.accuracy_cases(cases)
    assert len(idx) == len(set(idx)) and 4 <= len(idx) <= 8
    for nz in {c.nz for c in cases}:
        group = [k for k, c in enumerate(cases) if c.nz == nz]
        assert max(group, key=lambda q: cases[q].Re) in idx
        assert min(group, key=lambda q: cases[q].r_sphere) in idx


def _sample(sm, mx, hw="Not Active", thermal="Not Active", sw_thermal="Not Active",
            power="Not Active"):
    return ["0", str(sm), str(mx), "500.0", "0x0", hw, thermal, sw_thermal, power]


def test_clock_summary_inside_the_timed_region():
    cs = bench.ClockSampler(0)
    cs.t0, cs.t1 = 10.0, 11.0
    cs.samples = [(9.0, _sample(900, 2070, hw="Active")),     # before: ignored
                  (10.2, _sample(2070, 2070)),
                  (10.5, _sample(2055, 2070, power="Active")),
                  (10.9, _sample(2070, 2070)),
                  (12.0, _sample(800, 2070, thermal="Active"))]  # after: ignored
    s = cs.summary()
    assert s["sm_mhz"] == 2070.0 and s["sm_max_mhz"] == 2070.0
    assert s["reasons"] == ["sw_power_cap"] and s["samples"] == 3


def test_clock_summary_fallbacks():
    cs = bench.ClockSampler(0)
    assert cs.summary()["reasons"] == ["unsampled"]
    cs.t0, cs.t1 = 10.0, 11.0
    # no sample inside the window: all samples are summarised
    cs.samples = [(5.0, _sample(1980, 2070, hw="Active")), (20.0, _sample(2070, 2070))]
    s = cs.summary()
    assert s["samples"] == 2 and s["reasons"] == ["hw_slowdown"]
    assert s["sm_mhz"] == 2025.0
