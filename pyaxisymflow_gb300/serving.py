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

Reported: cell-updates/s over the run, per-step latency percentiles (device
time of one step of the whole batch, CUDA events), completion latency
percentiles (arrival to the end of the last step), the cost of the re-plans
and how the admission's memory estimate compares with what it allocated.
"""
import time
from dataclasses import dataclass, field

import numpy as np
import torch

from .engine import TILE_NR, TILE_NZ, RigidBodyCase, RigidEnsemble


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
    step_latency_s: list = field(default_factory=list)   # device time of each batch step
    step_interval_s: list = field(default_factory=list)  # host launch-to-launch interval
    replan_s: list = field(default_factory=list)         # wall time of each re-plan
    admissions: list = field(default_factory=list)       # (estimated, allocated) bytes
    cell_updates: int = 0
    wall_s: float = 0.0
    max_active: int = 0
    peak_bytes: int = 0

    def summary(self):
        lat = np.array(self.step_latency_s) if self.step_latency_s else np.zeros(1)
        comp = np.array([c.finished - c.arrival for c in self.completions]) \
            if self.completions else np.zeros(1)
        replan = np.array(self.replan_s) if self.replan_s else np.zeros(1)
        est = [(e, a) for e, a in self.admissions if a > 0]
        ratio = np.array([e / a for e, a in est]) if est else np.ones(1)
        return {
            "requests": len(self.completions),
            "cell_updates_per_s": self.cell_updates / self.wall_s if self.wall_s else 0.0,
            "step_p50_ms": float(np.percentile(lat, 50) * 1e3),
            "step_p99_ms": float(np.percentile(lat, 99) * 1e3),
            "completion_p50_s": float(np.percentile(comp, 50)),
            "completion_p99_s": float(np.percentile(comp, 99)),
            "replans": len(self.replan_s),
            "replan_p50_ms": float(np.percentile(replan, 50) * 1e3),
            "replan_p99_ms": float(np.percentile(replan, 99) * 1e3),
            "replan_share_of_wall": float(replan.sum() / self.wall_s) if self.wall_s else 0.0,
            "memory_estimate_over_allocated": {"min": float(ratio.min()),
                                               "max": float(ratio.max())},
            "max_active_cases": self.max_active,
            "peak_device_bytes": self.peak_bytes,
            "wall_s": self.wall_s,
        }


class SimulationServer:
    """Admits requests against a device-memory budget and steps every active
    case together.

    The host keeps `depth` steps in flight: it launches a step, does the
    book-keeping of the next one (admissions, retirements, re-plans) while the
    GPU runs, and waits only for the step `depth` launches back. A retiring
    case's state block (and, with keep_vorticity, its vorticity) is copied
    out on the stream right after its last step; its completion time is taken
    when the host sees that step finish."""

    def __init__(self, precision="f32", device="cuda", hbm_budget=0.8, capacity=1024,
                 keep_vorticity=False, depth=2):
        self.device = torch.device(device)
        self.ens = RigidEnsemble([], precision=precision, device=self.device, capacity=capacity)
        total = torch.cuda.get_device_properties(self.device).total_memory
        self.budget = hbm_budget * total
        self.keep_vorticity = keep_vorticity
        self.depth = max(1, int(depth))
        # pinned rows for the state blocks of retiring cases, used round robin:
        # a row is read back within `depth` steps, and at most `capacity` cases
        # retire per step, so (depth + 2) * capacity rows are never overwritten
        # before they are read
        self._rows = torch.empty(((self.depth + 2) * capacity,
                                  self.ens.state_arena.shape[1]), dtype=torch.float64,
                                 pin_memory=True)
        self._next_row = 0

    def prepare(self, cases):
        """Build the spectral bases of every grid size in `cases` ahead of time
        (the one-time host eigendecomposition is not charged to a request)."""
        for c in cases:
            self.ens._bases_for(c)

    def _estimate_bytes(self, case):
        """Device bytes an admission allocates: the case's fields (as
        engine.CaseState makes them) and, for a new grid size, its bases."""
        ens = self.ens
        es = ens.dtype.itemsize
        nr, nz = case.nr, case.nz
        cells = nr * nz
        # the caching allocator hands out multiples of 512 bytes
        blk = lambda b: -(-b // 512) * 512  # noqa: E731
        n = 5 * blk(cells * es) + blk(2 * cells * es)   # omega psi u_z u_r chi, gemm_work
        if ens.tensor_cores:
            n += 4 * blk(cells * 4)                      # tensor-core work fields
            if not ens.dct:
                n += 2 * blk(cells * 4)                  # omega's TF32 operand pair
        if ens.refine:
            n += blk(cells * 4)                          # psi_lo
        tiles = -(-nr // TILE_NR) * -(-nz // TILE_NZ)
        n += (blk(3 * case.kill_width * 8) + blk(nr * 8) + blk(nz * 8) + 3 * blk(nr * es)
              + blk(nz * es) + blk((2 * tiles + 8) * 8))
        key = (case.nr, case.nz, case.dx)
        if key not in ens._bases:
            n += 8 * 4 * (case.nr ** 2 + case.nz ** 2) * 3
        return n

    def run(self, requests, max_wall_s=None):
        """Serve `requests` (arrival times in seconds from now) to completion."""
        ens = self.ens
        pending = sorted(requests, key=lambda r: r.arrival)
        active = {}                 # CaseState -> [request, steps launched, admitted time]
        inflight = []               # (start event, end event, retiring cases' copies)
        report = ServerReport(completions=[])
        stream = torch.cuda.current_stream(self.device)
        t0 = time.perf_counter()
        last_launch = None

        def replan():
            ts = time.perf_counter()
            ens._replan(pack=False)
            report.replan_s.append(time.perf_counter() - ts)

        def retire_done(block):
            # handle finished steps in launch order; wait while more than
            # `block` steps are in flight
            while inflight and (len(inflight) > block or inflight[0][1].query()):
                ev_s, ev_e, fin = inflight.pop(0)
                ev_e.synchronize()
                tdone = time.perf_counter() - t0
                report.step_latency_s.append(ev_s.elapsed_time(ev_e) / 1e3)
                for req, admitted_at, state_host, vort in fin:
                    report.completions.append(Completion(
                        id=req.id, steps=req.steps, arrival=req.arrival, admitted=admitted_at,
                        finished=tdone, state=state_host.numpy().copy(),
                        vorticity=vort.cpu() if vort is not None else None))

        while pending or active or inflight:
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
                before = torch.cuda.memory_allocated(self.device)
                m = ens._admit(req.case)
                report.admissions.append((need, torch.cuda.memory_allocated(self.device)
                                          - before))
                active[m] = [req, 0, now]
                admitted = True
            if admitted:
                replan()
            if not active:
                retire_done(0)
                last_launch = None
                if pending:
                    time.sleep(max(0.0, pending[0].arrival - (time.perf_counter() - t0)))
                continue
            report.max_active = max(report.max_active, len(active))
            ev_s = torch.cuda.Event(enable_timing=True)
            ev_e = torch.cuda.Event(enable_timing=True)
            ev_s.record(stream)
            ens.step(1)
            ev_e.record(stream)
            tl = time.perf_counter()
            if last_launch is not None:
                report.step_interval_s.append(tl - last_launch)
            last_launch = tl
            fin, done = [], []
            for m, rec in active.items():
                rec[1] += 1
                report.cell_updates += m.case.nr * m.case.nz
                if rec[1] >= rec[0].steps:
                    done.append(m)
            for m in done:
                req, steps, admitted_at = active.pop(m)
                state_host = self._rows[self._next_row]
                self._next_row = (self._next_row + 1) % self._rows.shape[0]
                state_host.copy_(ens.state_arena[m.slot], non_blocking=True)
                vort = m.fields["omega"].detach().clone() if self.keep_vorticity else None
                fin.append((req, admitted_at, state_host, vort))
                ens.members.remove(m)
                ens._free.append(m.slot)
                m.fields = None
            inflight.append((ev_s, ev_e, fin))
            if done:
                replan()
            retire_done(self.depth)
            report.peak_bytes = max(report.peak_bytes, torch.cuda.memory_allocated(self.device))
        retire_done(0)
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
