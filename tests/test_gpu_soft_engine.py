"""The soft-sphere loop with dt and t resident on the device
(SoftSphereEngine) against the host-dt drop-in loop, the golden vectors and
itself replayed from a CUDA graph."""
import numpy as np
import pytest
import torch

from oracle import simulation as sim

pytestmark = pytest.mark.gpu

FIELDS = ("vorticity", "eta1", "eta2", "ball_phi", "ball_char_func", "psi", "u_z", "u_r")


def rel_l2(a, b):
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))


def golden_case():
    return sim.SoftSphereCase(nz=64, nr=32, dx=1.0 / 64, r_ball=0.15, lam=1e6)


def test_engine_matches_host_dt_loop():
    """Same kernels and arithmetic as the host-dt loop; the device takes sin
    and cos of omega t (the host loop uses the C library's), so agreement is
    to round-off, not bits."""
    from pyaxisymflow_gb300.simulation import SoftSphereEngine, SoftSphereSimulation
    case = golden_case()
    host = SoftSphereSimulation(case, device="cuda")
    dev = SoftSphereEngine(case, device="cuda")
    for n in range(12):
        host.step()
        dev.step()
        torch.cuda.synchronize()
        assert abs(dev.dt - host.dt) <= 1e-15 * host.dt, n
    for f in FIELDS:
        err = rel_l2(getattr(dev, f).cpu().numpy(), getattr(host, f).cpu().numpy())
        assert err < 1e-13, (f, err)
    assert abs(dev.t - host.t) <= 1e-15 * host.t
    assert dev.steps == 12 and dev.status() == 0


def test_engine_against_golden(golden):
    from pyaxisymflow_gb300.simulation import SoftSphereEngine
    g = golden("soft")
    e = SoftSphereEngine(golden_case(), device="cuda")
    e.step(12)
    torch.cuda.synchronize()
    for f, name in (("vorticity", "omega"), ("eta1", "eta1"), ("eta2", "eta2"),
                    ("ball_phi", "phi"), ("ball_char_func", "chi")):
        err = rel_l2(getattr(e, f).cpu().numpy(), g[f"soft/{name}_12"])
        assert err < 1e-12, (f, err)
    assert abs(e.t - float(g["soft/t_12"])) <= 1e-13 * float(g["soft/t_12"])


def test_graph_replay_is_bit_identical():
    from pyaxisymflow_gb300.simulation import SoftSphereEngine
    case = sim.SoftSphereCase(nz=128, nr=64, dx=1.0 / 64, r_ball=0.15, lam=1e6)
    a = SoftSphereEngine(case, device="cuda")
    b = SoftSphereEngine(case, device="cuda")
    a.step(6)
    b.capture(1)
    for _ in range(6):
        b.replay()
    torch.cuda.synchronize()
    for f in FIELDS:
        assert torch.equal(getattr(a, f), getattr(b, f)), f
    assert torch.equal(a.state, b.state)
    assert b.steps == 6 and b.status() == 0 and float(b.state[4]) >= 1


def test_engine_fp64_dct_solve():
    """The z products of the solve as FP64 DCTs: the cosine basis
    diagonalises the Neumann z operator exactly, LAPACK's eigenvectors to
    ~1e-12, so the two solves differ at that level (psi most)."""
    from pyaxisymflow_gb300.simulation import SoftSphereEngine
    case = golden_case()
    dense = SoftSphereEngine(case, device="cuda")
    dct = SoftSphereEngine(case, device="cuda", dct=True)
    dense.step(12)
    dct.step(12)
    torch.cuda.synchronize()
    for f in FIELDS:
        err = rel_l2(getattr(dct, f).cpu().numpy(), getattr(dense, f).cpu().numpy())
        assert err < 2e-11, (f, err)
    assert dct.status() == 0 and dct.steps == 12


def test_extrapolation_failure_sets_a_status_bit():
    """An extrapolation that needs more sweeps than allowed fails with
    AXI_ERR_NOT_CONVERGED; the device loop records it in its status word
    instead of raising (it never reads back mid-step), and the sweep count
    reaches the cap plus one, as the single-block loop counts it."""
    from pyaxisymflow_gb300 import _native as N
    from pyaxisymflow_gb300.simulation import SOFT_SWEEPS, SoftSphereEngine
    case = golden_case()
    ok = SoftSphereEngine(case, device="cuda")
    capped = SoftSphereEngine(case, device="cuda")
    capped.max_sweeps = 2
    ok.step(2)
    capped.step(2)
    torch.cuda.synchronize()
    assert ok.status() == 0 and float(ok.state[SOFT_SWEEPS]) > 3
    assert capped.status() & (1 << N.AXI_ERR_NOT_CONVERGED)
    assert float(capped.state[SOFT_SWEEPS]) == 3
