"""Continuous-batching simulation server on one GPU.

Requests (a rigid-body case and a number of steps) arrive over time. The
server keeps every admitted case's fields resident on the device and advances
all of them with one fused launch sequence per step
(`engine.RigidEnsemble`); between steps it admits queued requests whose
arrival time has passed while the estimated device memory stays within a
budget (a fraction of the GPU's HBM), and retires the cases that finished.
Each case's arithmetic depends only on that case (tiles, reductions and
spectral products are per case), so a result is bit-identical whether the
case ran alone or in any mix.

Reported: cell-updates/s over the run, per-step latency percentiles (wall
time of one step of the whole batch) and completion latency percentiles
(arrival to last step).
"""
import time
from dataclasses import dataclass, field

import numpy as np
import torch

from .engine import RigidBodyCase, RigidEnsemble


@dataclass
class SimulationRequest:
    id: int
    case: RigidBodyCase
    steps: int
    arrival: float = 0.0          # seconds after the server starts


@dataclass
class Completion:
    id: int
    steps: int
    arrival: float
    admitted: float
    finished: float
    state: np.ndarray             # the case's device state block at the end
    vorticity: torch.Tensor = None


@dataclass
class ServerReport:
    completions: list
    step_latency_s: list = field(default_factory=list)
    cell_updates: int = 0
    wall_s: float = 0.0
    max_active: int = 0
    peak_bytes: int = 0

    def summary(self):
        lat = np.array(self.step_latency_s) if self.step_latency_s else np.zeros(1)
        comp = np.array([c.finished - c.arrival for c in self.completions]) \
            if self.completions else np.zeros(1)
        return {
            "requests": len(self.completions),
            "cell_updates_per_s": self.cell_updates / self.wall_s if self.wall_s else 0.0,
            "step_p50_ms": float(np.percentile(lat, 50) * 1e3),
            "step_p99_ms": float(np.percentile(lat, 99) * 1e3),
            "completion_p50_s": float(np.percentile(comp, 50)),
            "completion_p99_s": float(np.percentile(comp, 99)),
            "max_active_cases": self.max_active,
            "peak_device_bytes": self.peak_bytes,
            "wall_s": self.wall_s,
        }


class SimulationServer:
    """Admits requests against a device-memory budget and steps every active
    case together."""

    def __init__(self, precision="f32", device="cuda", hbm_budget=0.8, capacity=1024,
                 keep_vorticity=False):
        self.device = torch.device(device)
        self.ens = RigidEnsemble([], precision=precision, device=self.device, capacity=capacity)
        total = torch.cuda.get_device_properties(self.device).total_memory
        self.budget = hbm_budget * total
        self.keep_vorticity = keep_vorticity

    def prepare(self, cases):
        """Build the spectral bases of every grid size in `cases` ahead of time
        (the one-time host eigendecomposition is not charged to a request)."""
        for c in cases:
            self.ens._bases_for(c)

    def _estimate_bytes(self, case):
        esize = self.ens.dtype.itemsize
        cells = case.nr * case.nz
        per_case = cells * (6 * esize + 2 * esize) + cells * 4 * (2 + 4 if self.ens.tensor_cores
                                                                  else 0)
        key = (case.nr, case.nz, case.dx)
        bases = 0 if key in self.ens._bases else 8 * 4 * (case.nr ** 2 + case.nz ** 2) * 3
        return per_case + bases

    def run(self, requests, max_wall_s=None):
        """Serve `requests` (arrival times in seconds from now) to completion."""
        ens = self.ens
        pending = sorted(requests, key=lambda r: r.arrival)
        active = {}                 # CaseState -> [request, steps done, admitted time]
        report = ServerReport(completions=[])
        t0 = time.perf_counter()
        while pending or active:
            now = time.perf_counter() - t0
            if max_wall_s is not None and now > max_wall_s:
                break
            admitted = False
            while pending and pending[0].arrival <= now:
                req = pending[0]
                need = self._estimate_bytes(req.case)
                if active and torch.cuda.memory_allocated(self.device) + need > self.budget:
                    break       # head of the queue waits for memory to free up
                pending.pop(0)
                m = ens._admit(req.case)
                active[m] = [req, 0, now]
                admitted = True
            if admitted:
                ens._replan()
            if not active:
                if pending:
                    time.sleep(max(0.0, pending[0].arrival - (time.perf_counter() - t0)))
                continue
            report.max_active = max(report.max_active, len(active))
            ts = time.perf_counter()
            ens.step(1)
            torch.cuda.synchronize(self.device)
            te = time.perf_counter()
            report.step_latency_s.append(te - ts)
            report.peak_bytes = max(report.peak_bytes, torch.cuda.memory_allocated(self.device))
            done = []
            for m, rec in active.items():
                rec[1] += 1
                report.cell_updates += m.case.nr * m.case.nz
                if rec[1] >= rec[0].steps:
                    done.append(m)
            for m in done:
                req, steps, admitted_at = active.pop(m)
                report.completions.append(Completion(
                    id=req.id, steps=steps, arrival=req.arrival, admitted=admitted_at,
                    finished=te - t0, state=ens.state_arena[m.slot].cpu().numpy().copy(),
                    vorticity=(m.fields["omega"].detach().cpu().clone()
                               if self.keep_vorticity else None)))
                ens.members.remove(m)
                ens._free.append(m.slot)
                m.fields = None
            if done:
                ens._replan()
        report.wall_s = time.perf_counter() - t0
        return report


def poisson_requests(n, rate_per_s=20.0, seed=5, sizes=(256, 512, 1024, 2048),
                     steps=(500, 5000), re_range=(10.0, 500.0), step_scale=1.0):
    """Seeded synthetic request stream: Poisson arrivals, grids nz x nz/2 on
    z in [0, 2], r in [0, 1], a rigid sphere, torus or spheroid (aspect ratio
    uniform in [0.5, 2]) in a uniform stream, Re log-uniform."""
    rng = np.random.default_rng(seed)
    t = 0.0
    out = []
    for k in range(n):
        t += rng.exponential(1.0 / rate_per_s)
        nz = int(rng.choice(sizes))
        body = str(rng.choice(["sphere", "torus", "spheroid"]))
        radius = float(rng.uniform(0.04, 0.1))
        case = RigidBodyCase(
            nz=nz, nr=nz // 2, dx=2.0 / nz, z_cm=0.5, r_sphere=radius,
            Re=float(np.exp(rng.uniform(np.log(re_range[0]), np.log(re_range[1])))),
            body=body, aspect=float(rng.uniform(0.5, 2.0)),
            torus_R=(0.2 if body == "torus" else 0.0), seed=10_000 + k)
        n_steps = max(1, int(round(rng.integers(steps[0], steps[1] + 1) * step_scale)))
        out.append(SimulationRequest(id=k, case=case, steps=n_steps, arrival=t))
    return out
