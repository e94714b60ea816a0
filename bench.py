"""Benchmark of the per-timestep hot path on GB300 (one JSON line on stdout).

python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference]
                [--workload ensemble64|sphere512] [--precision f32|f64]

A "step" advances every case of the workload by one timestep (the loop body
of examples/FlowPastSphere/flow_past_sphere.py:107-188). value = cell-updates
per second over the whole job (all ranks): cells of all cases x steps / time.

Workloads (synthetic, seeded; there is no dataset):
  ensemble64  64 freely sedimenting rigid spheres, nz in {256, 512, 768, 1024},
              nr = nz / 2, z in [0, 2], r in [0, 1], Re log-uniform in
              [10, 1000] (velocity scale 1), sphere radius uniform in
              [0.04, 0.12], density ratio uniform in [1.5, 4], seed 4
  sphere512   one 512 x 256 rigid sphere, Re 100, radius 0.0625 at z = 0.5
  poisson2048 isolated streamfunction solves, 2048 x 1024, periodic z, a sum
              of 32 Gaussian vortex rings (seed 3); FP32 tensor-core solve +
              one FP64 refinement step vs plain FP64
  serve       continuous-batching server on a Poisson request stream
  remesh      vorticity advection by remeshed particles (MP4), 2048 x 1024

--impl reference times the reference's CPU path restated by the oracle
(numpy FP64, all host cores for BLAS) on a bounded sample of the same
workload; it never touches the GPU.
"""
import argparse
import json
import math
import os
import subprocess
import sys
import threading
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)

METRIC = "cell-updates/s on 1 GB300, batched FP32 vs plain FP64 at <=1e-5 L2; p50/p99 lat"
UNIT = "cell-updates/s"
PHASES = ("kill", "transform", "vel_max", "penalise", "advect_diffuse")
# Algorithmic fields moved per cell by each stencil phase (reads + writes):
# vel_max psi; penalise psi chi omega -> u_z u_r and the penalised omega
# (staged in the work buffer; + psi_lo with the refinement step);
# advect_diffuse staged omega, u_z, u_r -> omega (+ omega's TF32 hi / lo
# operand copy on the dense tensor-core path, + the rebuilt mask of
# sedimenting bodies).
PHASE_FIELDS = {"vel_max": 1, "penalise": 6, "advect_diffuse": 4}
# the same in the FP64 engine (sedimenting bodies: + the rebuilt mask)
PHASE_FIELDS_F64 = {"vel_max": 1, "penalise": 6, "advect_diffuse": 5}


# DRAM bytes (dram__bytes_read.sum + dram__bytes_write.sum) of each step
# kernel's launches in one step (both plan groups; the z transforms and the
# radial products: both launches of each group together), ensemble64 FP32
# engine, from the ncu capture summarised in profiles/dram_traffic_ensemble64.md
NCU_TRAFFIC = {
    ("ensemble64", "f32", "kill"): 5.9e6,
    ("ensemble64", "f32", "z_transforms"): 461.1e6,
    ("ensemble64", "f32", "r_products"): 523.9e6,
    ("ensemble64", "f32", "vel_max"): 74.0e6,
    ("ensemble64", "f32", "penalise"): 444.4e6,
    ("ensemble64", "f32", "advect_diffuse"): 295.7e6,
}
# remeshing (2048 x 1024 cells, 4.19 M particles): FP64 instructions per
# particle of the two kernels together (80 + 48) and their DRAM bytes per call
FP64_INSTR_PER_PARTICLE = 128.0
FP64_PEAK_GINSTR = 625.0
P2M_TRAFFIC = 673.2e6


def ensemble_cases(workload, seed=4):
    from pyaxisymflow_gb300.engine import RigidBodyCase
    if workload == "sphere512":
        return [RigidBodyCase()]
    rng = np.random.default_rng(seed)
    cases = []
    for k in range(64):
        nz = int(rng.choice([256, 512, 768, 1024]))
        Re = float(np.exp(rng.uniform(np.log(10.0), np.log(1000.0))))
        radius = float(rng.uniform(0.04, 0.12))
        ratio = float(rng.uniform(1.5, 4.0))
        cases.append(RigidBodyCase(nz=nz, nr=nz // 2, dx=2.0 / nz, r_sphere=radius, Re=Re,
                                   z_cm=1.5, U0=0.0, ramp=False, sediment=True, rho_s=ratio,
                                   seed=1000 + k))
    return cases


def peaks():
    path = os.path.join(HERE, "MEASURED_PEAKS.json")
    if os.path.exists(path):
        with open(path) as f:
            p = json.load(f)
        return p.get("hbm_gbs", 6800.0), p.get("bf16_tflops", 1900.0), "measured"
    return 6800.0, 1900.0, "fallback"


class ClockSampler:
    """nvidia-smi clocks / throttle reasons sampled during the timed region."""

    QUERY = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index, interval_ms=50):
        self.gpu = gpu_index
        self.interval_ms = interval_ms
        self.samples = []
        self._proc = None
        self.t0 = self.t1 = 0.0
        self._thread = threading.Thread(target=self._run, daemon=True)

    def _run(self):
        # one nvidia-smi process sampling every interval_ms (a new process per
        # sample takes longer than the interval)
        try:
            self._proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.gpu}", f"--query-gpu={self.QUERY}",
                 "--format=csv,noheader,nounits", f"-lms={self.interval_ms}"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            for line in self._proc.stdout:
                line = line.strip()
                if line:
                    self.samples.append((time.perf_counter(), [x.strip() for x in line.split(",")]))
        except Exception:
            pass

    def __enter__(self):
        self._thread.start()
        time.sleep(0.2)  # let the sampler start before the timed region
        self.t0 = time.perf_counter()
        return self

    def __exit__(self, *exc):
        self.t1 = time.perf_counter()
        time.sleep(2 * self.interval_ms / 1000.0)
        if self._proc is not None:
            self._proc.terminate()  # the process this sampler started
            try:
                self._proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self._proc.kill()
        self._thread.join(timeout=10)

    def summary(self):
        """Median SM clock and the throttle reasons of the samples taken while
        the timed region ran (all samples when none fell inside it)."""
        inside = [f for t, f in self.samples
                  if self.t0 <= t <= self.t1 + self.interval_ms / 1000.0]
        picked = inside or [f for _, f in self.samples]
        if not picked:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        sm = [float(s[1]) for s in picked if s[1].replace(".", "").isdigit()]
        mx = [float(s[2]) for s in picked if s[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[k] for s in picked for k in range(4)
                          if len(s) > 5 + k and s[5 + k].lower() == "active"})
        return {"sm_mhz": float(np.median(sm)) if sm else None,
                "sm_max_mhz": max(mx) if mx else None, "reasons": reasons,
                "samples": len(picked), "interval_ms": self.interval_ms}


def dist_setup(args):
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("gloo")
    return world, rank, local


def barrier(world):
    if world > 1:
        import torch.distributed as dist
        dist.barrier()


def max_over_ranks(world, x):
    if world == 1:
        return x
    import torch
    import torch.distributed as dist
    t = torch.tensor([x], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def case_params(cases):
    """The fields of each case that the oracle needs, as plain values."""
    return [dict(nz=c.nz, nr=c.nr, dx=c.dx, z_cm=c.z_cm, r_sphere=c.r_sphere, U0=c.U0, Re=c.Re,
                 nu=c.nu, lam=c.lam, cfl=c.cfl, kill_width=c.kill_width, ramp=c.ramp,
                 noise=c.noise, seed=c.seed, sediment=c.sediment, rho_f=c.rho_f,
                 rho_s=c.rho_s, gravity=c.gravity) for c in cases]


def host_cores():
    return len(os.sched_getaffinity(0)) if hasattr(os, "sched_getaffinity") else os.cpu_count()


def cpu_run(cases, threads, seconds, warmup=1, max_rounds=1000, kind="cport", dump=None):
    """The oracle timed on the host (oracle/cpu_baseline.py) in a child
    process, so that its BLAS and OpenMP thread counts are set before numpy
    loads; one round advances every case one timestep. Returns the child's
    JSON record."""
    import tempfile
    with tempfile.TemporaryDirectory() as d:
        path = os.path.join(d, "cases.json")
        with open(path, "w") as f:
            json.dump(case_params(cases), f)
        env = dict(os.environ, OMP_NUM_THREADS=str(threads),
                   OPENBLAS_NUM_THREADS=str(threads), OPENBLAS_THREAD_TIMEOUT="4",
                   PYTHONDONTWRITEBYTECODE="1")
        cmd = [sys.executable, "-m", "oracle.cpu_baseline", path, "--kind", kind,
               "--seconds", str(seconds), "--warmup", str(warmup),
               "--max-rounds", str(max_rounds)]
        if dump:
            cmd += ["--dump", dump]
        r = subprocess.run(cmd, cwd=HERE, env=env, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"CPU baseline run failed: {r.stderr[-2000:]}")
        return json.loads(r.stdout.strip().splitlines()[-1])


def cpu_baseline_record(cases):
    """The GPU line's cpu_baseline: the C + OpenMP oracle on every host core
    over the whole workload (about 20 s of rounds), one core on a sample of
    two cases per grid size, and the oracle's reproducibility across BLAS
    thread counts (the 512 x 256 rigid sphere, 100 steps, 1 thread vs all)."""
    cores = host_cores()
    full = cpu_run(cases, cores, seconds=20.0)
    by_size = {}
    for c in cases:
        by_size.setdefault(c.nz, [])
        if len(by_size[c.nz]) < 2:
            by_size[c.nz].append(c)
    sample = [c for nz in sorted(by_size) for c in by_size[nz]]
    one = cpu_run(sample, 1, seconds=8.0, warmup=0)
    import tempfile

    from pyaxisymflow_gb300.engine import RigidBodyCase
    with tempfile.TemporaryDirectory() as d:
        dumps = []
        for th in (1, cores):
            path = os.path.join(d, f"w{th}.npz")
            cpu_run([RigidBodyCase()], th, seconds=1e9, warmup=0, max_rounds=100, dump=path)
            dumps.append(path)
        a = np.load(dumps[0])["arr_0"]
        b = np.load(dumps[1])["arr_0"]
        floor = float(np.linalg.norm(a - b) / np.linalg.norm(a))
    return {
        "value": full["value"], "unit": UNIT, "cores": cores, "kind": "port",
        "sample": (f"all {full['cases']} cases of the workload, {full['rounds']} timesteps each "
                   f"({full['seconds']:.1f} s): the oracle with its grid kernels in C + OpenMP "
                   f"({full['omp_threads']} threads; ENO3 as the reference's pystencils C with "
                   f"OpenMP, the rest as its numba loops), spectral solve by numpy / OpenBLAS "
                   f"({full['blas_threads']} threads), FP64"),
        "cpu_model": full["cpu_model"], "machine": full["machine"],
        "omp_threads": full["omp_threads"], "blas_threads": full["blas_threads"],
        "one_core": {"value": one["value"], "unit": UNIT,
                     "sample": f"{one['cases']} cases (two per grid size), {one['rounds']} "
                               f"timestep(s) each, 1 OpenMP + 1 BLAS thread"},
        "per_core_scaling": full["value"] / one["value"],
        "blas_thread_floor": {"rel_l2_omega": floor,
                              "case": "512 x 256 rigid sphere, 100 steps, OpenBLAS 1 thread vs "
                                      f"{cores}"},
    }


def accuracy_cases(cases):
    """Indices of the hardest cases of the seeded ensemble per grid size: the
    highest Reynolds number and the smallest sphere."""
    idx = []
    for nz in sorted({c.nz for c in cases}):
        group = [k for k, c in enumerate(cases) if c.nz == nz]
        for k in (max(group, key=lambda q: cases[q].Re),
                  min(group, key=lambda q: cases[q].r_sphere)):
            if k not in idx:
                idx.append(k)
    return idx


def fp32_accuracy(cases, dev, steps):
    """Relative L2 error of the FP32 engine against the FP64 engine (within
    1e-12 of the FP64 oracle) on the hardest cases, at checkpoints up to
    `steps`, with two FP64 controls run the same way: the initial vorticity
    moved by one double ulp (does the flow amplify round-off?) and the sphere
    radius moved by one float ulp at the same viscosity (how far does a
    float-sized change of the problem itself move the fields?)."""
    import dataclasses

    import torch

    from pyaxisymflow_gb300.engine import ST_UBODY, ST_ZCM, RigidEnsemble
    idx = accuracy_cases(cases)
    sel = [cases[k] for k in idx]
    w0 = [c.noise * np.random.default_rng(c.seed).standard_normal((c.nr, c.nz)) for c in sel]
    ulp = 2.0 ** -24
    wider = [dataclasses.replace(c, r_sphere=c.r_sphere * (1 + ulp), Re=c.Re * (1 + ulp))
             for c in sel]
    checkpoints = sorted({steps // 4, steps // 2, steps})
    fields = ("omega", "psi", "u_z", "u_r")

    def snaps(ens):
        out = {}
        for s in range(1, steps + 1):
            ens.step(1)
            if s in checkpoints:
                rows = []
                for m in ens.members:
                    f = {n: m.fields[n].double().clone() for n in fields}
                    if "psi_lo" in m.fields:
                        f["psi"] += m.fields["psi_lo"].double()
                    rows.append(f)
                out[s] = (rows, ens.state.cpu().numpy().copy())
        torch.cuda.synchronize(dev)
        return out

    ref = snaps(RigidEnsemble(sel, precision="f64", device=dev, initial_vorticity=w0))
    runs = {
        "fp32": snaps(RigidEnsemble(sel, precision="f32", device=dev, initial_vorticity=w0)),
        "fp64_double_ulp_noise": snaps(RigidEnsemble(
            sel, precision="f64", device=dev,
            initial_vorticity=[np.nextafter(w, np.inf) for w in w0])),
        "fp64_radius_float_ulp": snaps(RigidEnsemble(wider, precision="f64", device=dev,
                                                     initial_vorticity=w0)),
    }
    per_case = []
    for q, c in enumerate(sel):
        row = {"case": idx[q], "grid": f"{c.nz}x{c.nr}", "Re": c.Re, "radius": c.r_sphere,
               "density_ratio": c.rho_s}
        for name, sn in runs.items():
            row[name] = {}
            for s in checkpoints:
                a, sa = sn[s]
                b, sb = ref[s]
                e = {n: float(torch.linalg.norm(a[q][n] - b[q][n]) / torch.linalg.norm(b[q][n]))
                     for n in fields}
                e["z_body"] = float(abs(sa[q, ST_ZCM] - sb[q, ST_ZCM]) / abs(sb[q, ST_ZCM]))
                e["U_body"] = float(abs(sa[q, ST_UBODY] - sb[q, ST_UBODY])
                                    / max(abs(sb[q, ST_UBODY]), 1e-300))
                row[name][str(s)] = e
        per_case.append(row)
    last = str(steps)
    summary = {name: {n: max(r[name][last][n] for r in per_case) for n in fields}
               for name in runs}
    # the same error over all cells of the selected cases together
    agg = {}
    for name, sn in runs.items():
        a, _ = sn[steps]
        b, _ = ref[steps]
        agg[name] = {n: float(np.sqrt(sum(float(torch.linalg.norm(a[q][n] - b[q][n])) ** 2
                                          for q in range(len(sel)))
                                      / sum(float(torch.linalg.norm(b[q][n])) ** 2
                                            for q in range(len(sel)))))
                     for n in fields}
    return {"steps": steps, "checkpoints": checkpoints, "cases": idx,
            "max_rel_l2_at_end": summary, "rel_l2_over_all_selected_cells_at_end": agg,
            "per_case": per_case}


def run_reference(args, world, rank):
    """The reference's CPU implementation of the path on the host cores: the
    oracle with its grid kernels in C + OpenMP on every core and the
    spectral solve on OpenBLAS; a step advances every case of the workload
    one timestep (the GPU arm's step); the steps stop after about two minutes
    of stepping."""
    if rank != 0:
        return
    if args.workload == "soft1024":
        rec = soft_cpu_record(soft_case(), seconds=120.0)
        line = {"impl": "reference", "metric": "cell-updates/s, soft-sphere streaming loop (FP64)",
                "value": rec["value"], "unit": UNIT, "n_gpus": args.gpus, "steps": args.steps,
                "warmup": args.warmup, "higher_is_better": True, "scaling": "weak",
                "vs_baseline": None, "dtype": "f64", "data": "synthetic",
                "config": {"workload": "soft1024", "sample": rec["sample"]},
                "cpu_baseline": rec,
                "e2e": {"value": rec["value"], "unit": UNIT, "h2d_bytes_per_step": 0,
                        "d2h_bytes_per_step": 0}}
        print(json.dumps(line), flush=True)
        return
    cases = ensemble_cases(args.workload)
    cores = host_cores()
    rec = cpu_run(cases, cores, seconds=120.0, warmup=min(args.warmup, 1),
                  max_rounds=args.steps)
    value = rec["value"]
    desc = (f"all {len(cases)} cases, 1 timestep each per step, {rec['rounds']} of "
            f"{args.steps} steps timed ({rec['seconds']:.1f} s), oracle with C + OpenMP grid "
            f"kernels ({rec['omp_threads']} threads) and OpenBLAS solve "
            f"({rec['blas_threads']} threads), FP64, {rec['cpu_model']}")
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus,
        "steps": rec["rounds"], "warmup": args.warmup,
        "ms_per_step": float(1000.0 * rec["seconds"] / rec["rounds"]),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic",
        "config": {"workload": args.workload, "cases": len(cases),
                   "cells_per_step": rec["cells_per_round"], "sample": desc},
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": cores, "kind": "port",
                         "sample": desc, "cpu_model": rec["cpu_model"]},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def phase_times(ens, ids, rounds, stream):
    """Device time (ms) of each phase in `ids` over all cases, as it runs in a
    step: each phase captured as a CUDA graph of its own (the plan groups'
    launches on forked streams, as in the step graph), `rounds` rounds of the
    phases in order replayed behind a backlog of whole steps, so the host
    never leaves the device idle between the events. Runs the phases (the
    cases advance)."""
    import torch
    dev = ens.device
    graphs = []
    torch.cuda.synchronize(dev)
    for ph in ids:
        g = torch.cuda.CUDAGraph()
        s = torch.cuda.Stream(dev)
        with torch.cuda.stream(s):
            with torch.cuda.graph(g, stream=s):
                ens.phase(ph, stream=s)
        graphs.append(g)
    torch.cuda.synchronize(dev)
    evs = [[(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
            for _ in ids] for _ in range(rounds)]
    if ens.graph is not None:
        for _ in range(5):
            ens.replay()
    else:
        ens.step(1)
    for r in range(rounds):
        for q, g in enumerate(graphs):
            evs[r][q][0].record(stream)
            g.replay()
            evs[r][q][1].record(stream)
    torch.cuda.synchronize(dev)
    return [sum(evs[r][q][0].elapsed_time(evs[r][q][1]) for r in range(rounds)) / rounds
            for q in range(len(ids))]


def run_gb300(args, world, rank, local):
    import torch
    from pyaxisymflow_gb300 import _native
    from pyaxisymflow_gb300.engine import ST_CD, ST_DT, ST_WORDS, HostPipeline, RigidEnsemble
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    _native.lib()
    cases = ensemble_cases(args.workload)
    zopt = {} if args.z_transform == "default" else {"dct": args.z_transform == "dct"}
    ens = RigidEnsemble(cases, precision=args.precision, device=dev, **zopt)
    cells = ens.cells()
    stream = torch.cuda.current_stream(dev)
    # launch choices for this grid-size mix, measured before the timed region
    # (scheduling only: the results are the same for every choice)
    from pyaxisymflow_gb300.autotune import Autotuner
    tuner = Autotuner()
    tuning = None
    if not args.no_tune:
        tuner.tune(ens)
        tuning = dict(tuner.last)
    ens.capture(1)
    for _ in range(args.warmup):
        ens.replay()
    torch.cuda.synchronize(dev)
    barrier(world)
    # ---- timed region: K graph replays, device time by CUDA events ------------
    with ClockSampler(local) as clocks:
        torch.cuda.synchronize(dev)
        barrier(world)
        evs_t = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps + 1)]
        evs_t[0].record(stream)
        for k in range(args.steps):
            ens.replay()
            evs_t[k + 1].record(stream)
        torch.cuda.synchronize(dev)
        barrier(world)
    step_ms = [evs_t[k].elapsed_time(evs_t[k + 1]) for k in range(args.steps)]
    ms = evs_t[0].elapsed_time(evs_t[-1])
    ms = max_over_ranks(world, ms)
    ms_per_step = ms / args.steps
    value = cells * world / (ms_per_step / 1000.0)
    status = ens.status()
    n_plans = ens.n_plans
    uses_tc = ens.tensor_cores
    # ---- per-phase device times (same stream, same step sequence) -------------
    ph_ms = {p: 0.0 for p in PHASES}
    nph = max(3, min(args.steps, 10))
    ph_list = phase_times(ens, list(range(len(PHASES))), nph, stream)
    for k, p in enumerate(PHASES):
        ph_ms[p] = ph_list[k]
    # the four launches of the transform one at a time (phase ids 5..8)
    part_ms = phase_times(ens, [5, 6, 7, 8], nph, stream)
    uses_dct = ens.dct
    uses_refine = ens.refine
    # ---- end to end through the public API with host buffers ------------------
    # every case's vorticity in pinned host memory; each step copies it in,
    # advances every case and copies it and the state blocks (dt, Cd) back.
    # The cases run as groups (--e2e-groups), each step of a group one CUDA graph on the
    # group's stream (its H2D copy, its launches, its D2H copies), so the
    # transfers of one group overlap the computation of the others, within a
    # step and across steps; the host reads each step's state blocks (two
    # pinned buffers in turn) while the next step runs.
    pipe = HostPipeline(cases, groups=args.e2e_groups, precision=args.precision, device=dev,
                        **zopt)
    if not args.no_tune:
        for sub in pipe.ensembles:
            tuner.tune(sub)
    host_w = pipe.host_buffer()
    host_states = [torch.empty((len(cases), ST_WORDS), dtype=torch.float64, pin_memory=True)
                   for _ in range(2)]
    for _ in range(2):
        pipe.step(host_w, host_states[0])
        pipe.synchronize()
    pipe.capture_pipelined(host_w, host_states)
    for k in range(2):
        pipe.replay_step(k)
        pipe.wait_step(k)
    field_bytes = host_w.numel() * host_w.element_size()
    h2d = field_bytes
    d2h = field_bytes + host_states[0].numel() * 8
    barrier(world)
    t0 = time.perf_counter()
    for k in range(args.steps):
        pipe.replay_step(k)
        if k:
            hs = host_states[pipe.wait_step(k - 1)]
            _ = float(hs[0, ST_CD]) + float(hs[0, ST_DT])
    hs = host_states[pipe.wait_step(args.steps - 1)]
    _ = float(hs[0, ST_CD]) + float(hs[0, ST_DT])
    pipe.synchronize()
    e2e_s = (time.perf_counter() - t0) / args.steps
    e2e_s = max_over_ranks(world, e2e_s)
    e2e_value = cells * world / e2e_s
    # ---- plain FP64 GPU path on the same workload, and the FP32 error -------------
    fp64 = None
    if args.precision == "f32" and not args.no_fp64_compare:
        del ens
        torch.cuda.empty_cache()
        fp64 = {}
        for variant, dct in (("dct", True), ("dense", False)):
            e64 = RigidEnsemble(cases, precision="f64", device=dev, dct=dct)
            e64.step(1)
            torch.cuda.synchronize(dev)
            f0 = torch.cuda.Event(enable_timing=True)
            f1 = torch.cuda.Event(enable_timing=True)
            nf = 3
            f0.record(stream)
            e64.step(nf)
            f1.record(stream)
            torch.cuda.synchronize(dev)
            ms64 = f0.elapsed_time(f1) / nf
            entry = {"value": cells * world / (ms64 / 1000.0), "ms_per_step": ms64,
                     "speedup_fp32_over_fp64": ms64 / ms_per_step,
                     "z_transform": "FP64 DCT" if dct else "dense FP64 products"}
            if dct:
                # per-phase device times of the FP64 step, and its stencil passes'
                # algorithmic bytes (FP64 fields) over their time
                p64 = dict(zip(PHASES, phase_times(e64, list(range(len(PHASES))), 3, stream)))
                entry["phase_ms"] = p64
                b64 = sum(sum(PHASE_FIELDS_F64.values()) * 8 * c.nr * c.nz for c in cases)
                entry["stencil_hbm_gbs"] = b64 / (sum(p64[p] for p in PHASE_FIELDS_F64)
                                                   / 1000.0) / 1e9
            fp64[variant] = entry
            del e64
            torch.cuda.empty_cache()
        fp64["speedup_fp32_over_fp64"] = fp64["dct"]["speedup_fp32_over_fp64"]
        if not args.no_accuracy:
            try:
                fp64["accuracy"] = fp32_accuracy(cases, dev, args.accuracy_steps)
            except Exception as exc:  # noqa: BLE001
                fp64["accuracy"] = {"error": f"{type(exc).__name__}: {exc}"[:500]}
    # ---- roofline of the dominant kernel ---------------------------------------
    hbm, bf16, src = peaks()
    esize = 8 if args.precision == "f64" else 4
    if uses_tc and not uses_dct:
        PHASE_FIELDS["advect_diffuse"] += 2   # omega's TF32 operand pair
    if any(c.sediment for c in cases):
        PHASE_FIELDS["advect_diffuse"] += 1   # the rebuilt mask
    if uses_refine:
        PHASE_FIELDS["penalise"] += 1         # psi_lo
    zname = "z_transforms" if uses_dct else "z_products"
    kern_ms = {"kill": ph_ms["kill"], zname: part_ms[0] + part_ms[2],
               "r_products": part_ms[1] + part_ms[3], "vel_max": ph_ms["vel_max"],
               "penalise": ph_ms["penalise"], "advect_diffuse": ph_ms["advect_diffuse"]}
    dom = max(kern_ms, key=kern_ms.get)
    if dom in ("r_products", "z_products"):
        # useful FLOPs: two products of 2 n^2 m each per case
        flops = sum(4.0 * (c.nr * c.nr * c.nz if dom == "r_products" else c.nz * c.nz * c.nr)
                    for c in cases)
        achieved = flops / (kern_ms[dom] / 1000.0) / 1e12
        if args.precision == "f64" or not uses_tc:
            roof = {"bound": "fp64" if args.precision == "f64" else "fp32",
                    "achieved": achieved, "peak": 1.25 if args.precision == "f64" else 73.0,
                    "unit": "TFLOP/s",
                    "peak_source": "nominal GB300 FP64 (DFMA probe on this pool: 1.0)"
                    if args.precision == "f64" else "nominal GB300 FP32"}
        else:
            # 3xTF32: three tensor products per useful product; the TF32 dense
            # rate is half the BF16 rate
            roof = {"bound": "tensor", "achieved": 3 * achieved, "peak": bf16 / 2,
                    "unit": "TFLOP/s", "useful_tflops": achieved,
                    "peak_source": f"{src} bf16 / 2 (TF32 dense rate)"}
    elif dom == "z_transforms":
        # forward: read the rows (4 B; with the refinement step also psi and
        # psi_lo, 8 B more, for the residual), write the TF32 pair (8 B);
        # inverse: read the rows and the spectral factor (4 + 4 B), write the
        # pair (8 B)
        per_cell = 36.0 if uses_refine else 28.0
        nbytes = sum(per_cell * c.nr * c.nz for c in cases)
        achieved = nbytes / (kern_ms[dom] / 1000.0) / 1e9
        roof = {"bound": "hbm", "achieved": achieved, "peak": hbm, "unit": "GB/s",
                "peak_source": f"{src} hbm"}
    else:
        nbytes = sum(PHASE_FIELDS.get(dom, 0) * esize * c.nr * c.nz for c in cases)
        achieved = nbytes / (kern_ms[dom] / 1000.0) / 1e9
        roof = {"bound": "hbm", "achieved": achieved, "peak": hbm, "unit": "GB/s",
                "peak_source": f"{src} hbm"}
    roof["kernel"] = dom
    roof["frac"] = roof["achieved"] / roof["peak"]
    roof["kernel_ms"] = kern_ms[dom]
    # DRAM bytes (read + write) of the dominant kernel's launches in one step,
    # from the ncu capture summarised in profiles/ (same workload and kernels)
    roof["traffic"] = NCU_TRAFFIC.get((args.workload, args.precision, dom))
    roof["traffic_unit"] = "bytes per step of the kernel's launches (ncu dram read + write)"
    stencil_bytes = sum(sum(PHASE_FIELDS.values()) * esize * c.nr * c.nz for c in cases)
    stencil_ms = sum(ph_ms[p] for p in PHASE_FIELDS)
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms_per_step, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": args.precision,
        "data": "synthetic",
        "config": {"workload": args.workload, "cases": len(cases), "cells_per_step": cells,
                   "precision": args.precision, "l2": "working set > L2 (129 MB)",
                   "parallelism": f"case-parallel replicas x{world}"},
        "roofline": roof,
        "phase_ms": ph_ms,
        "kernel_ms": kern_ms,
        "transform": "z DCT + radial tensor-core products" if uses_dct
                     else ("tensor-core products" if uses_tc else "SIMT products"),
        "step_latency_ms": {"p50": float(np.percentile(step_ms, 50)),
                            "p99": float(np.percentile(step_ms, 99))},
        "plain_fp64": fp64,
        "tuning": tuning,
        "stencil_hbm_gbs": stencil_bytes / (stencil_ms / 1000.0) / 1e9,
        "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": h2d,
                "d2h_bytes_per_step": d2h, "groups": len(pipe.ensembles),
                "pipelined": "per-group step graphs, state read one step behind"},
        "gpu_launches": None,
        "clocks": clocks.summary(),
        "status_ok": bool(np.all(status == 0)),
    }
    # kill_reset, 4 spectral products (2 transforms + 2 products on the DCT
    # path), vel_max (which also computes dt), penalise, advect_diffuse; per
    # plan group
    n_launch = (1 + 4 + 3) * n_plans
    line["gpu_launches"] = n_launch * args.steps
    line["config"]["plan_groups"] = n_plans
    # ---- continuous-batching serving leg (config 5) ----------------------------
    # (a failure of a secondary leg is recorded in the line, not allowed to
    # lose the measurement above)
    if not args.no_serve:
        try:
            line["serving"] = serve_leg(args, dev)
        except Exception as exc:  # noqa: BLE001
            line["serving"] = {"error": f"{type(exc).__name__}: {exc}"[:500]}
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        try:
            line["cpu_baseline"] = cpu_baseline_record(cases)
        except Exception as exc:  # noqa: BLE001
            line["cpu_baseline"] = {"error": f"{type(exc).__name__}: {exc}"[:500]}
    if rank == 0:
        print(json.dumps(line), flush=True)


def vortex_rings(nr, nz, dx, seed=3, n=32):
    """Seeded sum of axisymmetric Gaussian vortex rings: centres z ~ U(0, Lz),
    r ~ U(0.1, 0.9) Lr, radii U[0.02, 0.2], strengths N(0, 1)."""
    rng = np.random.default_rng(seed)
    z = (np.arange(nz) + 0.5) * dx
    r = (np.arange(nr) + 0.5) * dx
    Z, R = np.meshgrid(z, r)
    w = np.zeros((nr, nz))
    for _ in range(n):
        zc, rc = rng.uniform(0, nz * dx), rng.uniform(0.1, 0.9) * nr * dx
        rad, st = rng.uniform(0.02, 0.2), rng.standard_normal()
        w += st * np.exp(-((Z - zc) ** 2 + (R - rc) ** 2) / rad ** 2)
    return w, Z, R


def run_poisson(args, world, rank, local):
    """Isolated streamfunction solves, 2048 x 1024 (nz x nr), periodic z,
    Neumann r: FP32 tensor-core solve + one FP64-residual refinement vs the
    plain FP64 solve, with errors of psi and velocity."""
    import torch
    from pyaxisymflow_gb300.kernels.compute_velocity_from_psi import \
        compute_velocity_from_psi_unb
    from pyaxisymflow_gb300.kernels.FastDiagonalisationStokesSolver import \
        FastDiagonalisationStokesSolver
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    nz, nr = 2048, 1024
    dx = 1.0 / nr
    bc = "homogenous_neumann_along_r_and_periodic_along_z"
    w, Z, R = vortex_rings(nr, nz, dx)
    tw = torch.tensor(w, dtype=torch.float64, device=dev)
    tR = torch.tensor(R, dtype=torch.float64, device=dev)
    s64 = FastDiagonalisationStokesSolver(nr, nz, dx, bc_type=bc, device=dev)
    s32 = FastDiagonalisationStokesSolver(nr, nz, dx, bc_type=bc, device=dev,
                                          real_dtype=np.float32, refine=1)
    psi64, psi32 = torch.zeros_like(tw), torch.zeros_like(tw)
    stream = torch.cuda.current_stream(dev)

    def timed(fn, k):
        for _ in range(args.warmup):
            fn()
        torch.cuda.synchronize(dev)
        ev = [torch.cuda.Event(enable_timing=True) for _ in range(k + 1)]
        ev[0].record(stream)
        for q in range(k):
            fn()
            ev[q + 1].record(stream)
        torch.cuda.synchronize(dev)
        return [ev[q].elapsed_time(ev[q + 1]) for q in range(k)]

    with ClockSampler(local) as clocks:
        t32 = timed(lambda: s32.solve(psi32, tw), args.steps)
    t64 = timed(lambda: s64.solve(psi64, tw), max(3, args.steps // 4))
    tc_ms = timed(lambda: s32.engine._tc_run(ctypes_stream(stream)), args.steps)
    uz64, ur64 = (torch.zeros_like(tw) for _ in range(2))
    compute_velocity_from_psi_unb(uz64, ur64, psi64, tR, dx)
    # velocity by the FP32 stencil from psi as a float pair hi + lo (the
    # fused engine's representation), summed in float
    f32 = dict(dtype=torch.float32, device=dev)
    hi = psi32.float()
    lo = (psi32 - hi.double()).float()
    tRf = tR.float()
    parts = []
    for part in (hi, lo):
        u = [torch.zeros((nr, nz), **f32) for _ in range(2)]
        compute_velocity_from_psi_unb(u[0], u[1], part, tRf, dx)
        parts.append(u)
    uz32 = (parts[0][0] + parts[1][0]).double()
    ur32 = (parts[0][1] + parts[1][1]).double()

    def rel(a, b):
        return float(torch.linalg.norm(a - b) / torch.linalg.norm(b))

    s_norefine = FastDiagonalisationStokesSolver(nr, nz, dx, bc_type=bc, device=dev,
                                                 real_dtype=np.float32, refine=0)
    p0 = torch.zeros_like(tw)
    s_norefine.solve(p0, tw)
    cells = nr * nz
    ms32 = float(np.mean(t32))
    ms64 = float(np.mean(t64))
    flops = 4.0 * nr * nz * (nr + nz)
    tcm = float(np.mean(tc_ms))
    hbm, bf16, src = peaks()
    # e2e: host rhs in (pinned), solve, psi out
    host_in = torch.tensor(w, dtype=torch.float64).pin_memory()
    host_out = torch.empty_like(host_in).pin_memory()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        tw.copy_(host_in, non_blocking=True)
        s32.solve(psi32, tw)
        host_out.copy_(psi32, non_blocking=True)
        torch.cuda.synchronize(dev)
    e2e_s = (time.perf_counter() - t0) / args.steps
    line = {
        "metric": METRIC, "value": cells / (ms32 / 1000.0), "unit": UNIT, "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms32,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic",
        "config": {"workload": "poisson2048", "grid": "nz 2048 x nr 1024", "bc": bc,
                   "rhs": "32 Gaussian vortex rings, seed 3", "step": "one streamfunction solve",
                   "refinement_steps": 1},
        "roofline": {"bound": "tensor", "kernel": "tf32x3_gemm (4 products)",
                     "achieved": 3 * flops / (tcm / 1000.0) / 1e12, "peak": bf16 / 2,
                     "unit": "TFLOP/s", "useful_tflops": flops / (tcm / 1000.0) / 1e12,
                     "peak_source": f"{src} bf16 / 2 (TF32 dense rate)", "traffic": None},
        "step_latency_ms": {"p50": float(np.percentile(t32, 50)),
                            "p99": float(np.percentile(t32, 99))},
        "plain_fp64": {"value": cells / (ms64 / 1000.0), "ms_per_step": ms64,
                       "speedup_fp32_over_fp64": ms64 / ms32},
        "rel_l2_vs_fp64": {"psi": rel(psi32, psi64), "u_z": rel(uz32, uz64),
                           "u_r": rel(ur32, ur64), "psi_without_refinement": rel(p0, psi64)},
        "e2e": {"value": cells / e2e_s, "unit": UNIT, "h2d_bytes_per_step": cells * 8,
                "d2h_bytes_per_step": cells * 8},
        "gpu_launches": args.steps * (2 + 4 + 4 + 3),
        "clocks": clocks.summary(),
        "status_ok": s32.engine.tc_status() == 0,
    }
    if rank == 0:
        print(json.dumps(line), flush=True)


def soft_case():
    """Config 2: a soft neo-Hookean sphere (radius 0.1, G = 1e-3, density
    ratio 1) in oscillatory streaming, U(t) = 0.1 cos(2 pi t) on the
    penalised forcing region, 1024 x 512 cells on z in [0, 1], r in [0, 0.5]
    (the example's domain, dx = 1 / nz), the example's viscosity ratio and
    Brinkman factor."""
    from pyaxisymflow_gb300.simulation import SoftCase
    omega = 2 * math.pi
    e = 0.1 / (0.1 * omega)
    return SoftCase(nz=1024, nr=512, dx=1.0 / 1024, z_cm=0.5, r_ball=0.1, freq=1.0, e=e,
                    cauchy=e * (0.1 * omega) ** 2 / 1e-3)


def run_soft(args, world, rank, local):
    """Config 2 on the device: the soft-sphere loop with dt and t resident
    on the GPU (SoftSphereEngine), one CUDA graph per step, FP64."""
    import torch

    from pyaxisymflow_gb300.simulation import SOFT_WORDS, SoftSphereEngine
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    case = soft_case()
    cells = case.nr * case.nz
    eng = SoftSphereEngine(case, device=dev)
    stream = torch.cuda.current_stream(dev)
    eng.capture(1)
    for _ in range(args.warmup):
        eng.replay()
    torch.cuda.synchronize(dev)
    barrier(world)
    with ClockSampler(local) as clocks:
        torch.cuda.synchronize(dev)
        barrier(world)
        ev = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps + 1)]
        ev[0].record(stream)
        for k in range(args.steps):
            eng.replay()
            ev[k + 1].record(stream)
        torch.cuda.synchronize(dev)
        barrier(world)
    step_ms = [ev[k].elapsed_time(ev[k + 1]) for k in range(args.steps)]
    ms = max_over_ranks(world, ev[0].elapsed_time(ev[-1])) / args.steps
    status = eng.status()
    # device time of each launch group of a step
    nph = max(3, min(args.steps, 10))
    pev = [[(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
            for _ in eng.PARTS] for _ in range(nph)]
    for q in range(nph):
        for k in range(len(eng.PARTS)):
            pev[q][k][0].record(stream)
            eng.phase(k)
            pev[q][k][1].record(stream)
    torch.cuda.synchronize(dev)
    part_ms = {name: sum(pev[q][k][0].elapsed_time(pev[q][k][1]) for q in range(nph)) / nph
               for k, name in enumerate(eng.PARTS)}
    dom = max(part_ms, key=part_ms.get)
    hbm, _, src = peaks()
    if dom == "solve_velocity_dt":
        # the four FP64 products of the spectral solve: 2 n m k flops each
        flops = 4.0 * (case.nr * case.nz * case.nz + case.nr * case.nr * case.nz)
        achieved = flops / (part_ms[dom] / 1e3) / 1e12
        roof = {"bound": "fp64", "achieved": achieved, "peak": 1.25, "unit": "TFLOP/s",
                "peak_source": "nominal GB300 FP64 (dense products; no FP64 tensor path)"}
    else:
        # FP64 fields read + written per cell by the group (algorithmic)
        fields = {"advect_pin_mask": 23, "extrapolate": 12, "solid_stress": 17,
                  "tether_penalise_diffuse": 19}[dom]
        achieved = fields * 8.0 * cells / (part_ms[dom] / 1e3) / 1e9
        roof = {"bound": "hbm", "achieved": achieved, "peak": hbm, "unit": "GB/s",
                "peak_source": f"{src} hbm"}
    roof.update({"kernel": dom, "frac": roof["achieved"] / roof["peak"],
                 "kernel_ms": part_ms[dom], "traffic": None})
    # end to end: omega in from pinned host memory, one step, omega / eta1 /
    # eta2 and the state block back, every step
    host_w = torch.empty((case.nr, case.nz), dtype=torch.float64, pin_memory=True)
    host_w.copy_(eng.vorticity)
    host_out = torch.empty((3, case.nr, case.nz), dtype=torch.float64, pin_memory=True)
    host_state = torch.empty(SOFT_WORDS, dtype=torch.float64, pin_memory=True)
    torch.cuda.synchronize(dev)
    t0 = time.perf_counter()
    for _ in range(args.steps):
        eng.vorticity.copy_(host_w, non_blocking=True)
        eng.replay()
        host_out[0].copy_(eng.vorticity, non_blocking=True)
        host_out[1].copy_(eng.eta1, non_blocking=True)
        host_out[2].copy_(eng.eta2, non_blocking=True)
        host_state.copy_(eng.state, non_blocking=True)
        torch.cuda.synchronize(dev)
        host_w.copy_(host_out[0])
    e2e_s = max_over_ranks(world, (time.perf_counter() - t0) / args.steps)
    line = {
        "metric": "cell-updates/s, soft-sphere streaming loop (FP64)", "value": cells * world
        / (ms / 1e3), "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": "soft1024", "grid": "nz 1024 x nr 512, dx = 1/1024",
                   "body": "soft neo-Hookean sphere r 0.1, G 1e-3, density ratio 1",
                   "forcing": "U(t) = 0.1 cos(2 pi t)", "nu": case.nu, "lam": case.lam,
                   "dt": eng.dt, "l2": "each step touches > L2 (about 40 FP64 fields)"},
        "roofline": roof,
        "phase_ms": part_ms,
        "step_latency_ms": {"p50": float(np.percentile(step_ms, 50)),
                            "p99": float(np.percentile(step_ms, 99))},
        "extrapolation_sweeps_max": float(eng.state[4]),
        "e2e": {"value": cells * world / e2e_s, "unit": UNIT,
                "h2d_bytes_per_step": host_w.numel() * 8,
                "d2h_bytes_per_step": host_out.numel() * 8 + SOFT_WORDS * 8},
        "gpu_launches": eng.LAUNCHES_PER_STEP * args.steps,
        "clocks": clocks.summary(),
        "status_ok": status == 0,
    }
    # the same loop with the z products of the solve as FP64 DCTs (psi within
    # ~1e-11 of the dense eigenvector products)
    del eng
    torch.cuda.empty_cache()
    eng2 = SoftSphereEngine(case, device=dev, dct=True)
    eng2.capture(1)
    for _ in range(args.warmup):
        eng2.replay()
    torch.cuda.synchronize(dev)
    d0 = torch.cuda.Event(enable_timing=True)
    d1 = torch.cuda.Event(enable_timing=True)
    d0.record(stream)
    for _ in range(args.steps):
        eng2.replay()
    d1.record(stream)
    torch.cuda.synchronize(dev)
    ms2 = d0.elapsed_time(d1) / args.steps
    line["dct_variant"] = {"value": cells * world / (ms2 / 1e3), "ms_per_step": ms2,
                           "speedup_over_dense": ms / ms2, "status_ok": eng2.status() == 0,
                           "z_transform": "FP64 DCT-II / DCT-III rows, dense radial products"}
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        line["cpu_baseline"] = soft_cpu_record(case, seconds=12.0)
    if rank == 0:
        print(json.dumps(line), flush=True)


def soft_cpu_record(case, seconds):
    """The numpy oracle's soft loop on the host (its least-squares sweeps and
    ENO3 in numpy, slower than the reference's C++ and pystencils C), a
    bounded sample of steps of the same case."""
    from oracle import kernels as K
    from oracle import simulation as osim
    st, coords = osim.soft_sphere_init(case, K)
    solver = K.FastDiagonalisationStokesSolver(case.nr, case.nz, case.dx)
    aw = K.gen_advect_vorticity_via_eno3(case.dx, case.nr, case.nz)
    ae = K.gen_advect_refmap_via_eno3(case.dx, case.nr, case.nz)
    osim.soft_sphere_step(case, st, coords, solver, aw, ae, K)
    n, t0 = 0, time.perf_counter()
    while n < 1 or time.perf_counter() - t0 < seconds:
        osim.soft_sphere_step(case, st, coords, solver, aw, ae, K)
        n += 1
    secs = time.perf_counter() - t0
    return {"value": case.nr * case.nz * n / secs, "unit": UNIT, "cores": host_cores(),
            "kind": "port",
            "sample": f"{case.nz} x {case.nr}, {n} steps of the numpy oracle's soft loop "
                      f"({secs:.1f} s; BLAS on all cores, elementwise work, ENO3 and the "
                      "least-squares sweeps in numpy)"}


def ctypes_stream(stream):
    import ctypes
    return ctypes.c_void_p(stream.cuda_stream)


def serve_leg(args, dev, clocks=None):
    """Continuous batching on a Poisson stream of requests (mean 20/s): grids
    256 x 128 .. 2048 x 1024, sphere / torus / spheroid, 500-5000 steps, Re
    log-uniform in [10, 500], 80% HBM budget; and the same requests run one
    after another on the plain FP64 engine (per-size step time of one case
    alone, times the steps asked)."""
    import torch

    from pyaxisymflow_gb300.engine import RigidEnsemble
    from pyaxisymflow_gb300.serving import SimulationServer, poisson_requests
    reqs = poisson_requests(args.requests, rate_per_s=20.0, seed=5)
    server = SimulationServer(precision=args.precision, device=dev, hbm_budget=0.8)
    server.prepare([r.case for r in reqs])
    report = server.run(reqs)
    summ = report.summary()
    del server
    torch.cuda.empty_cache()
    per_size = {}
    for r in reqs:
        key = (r.case.nz, r.case.nr)
        if key in per_size:
            continue
        e = RigidEnsemble([r.case], precision="f64", device=dev)
        e.step(2)
        torch.cuda.synchronize(dev)
        t0 = time.perf_counter()
        e.step(5)
        torch.cuda.synchronize(dev)
        per_size[key] = (time.perf_counter() - t0) / 5
        del e
    seq_s = sum(per_size[(r.case.nz, r.case.nr)] * r.steps for r in reqs)
    seq_cells = sum(r.case.nz * r.case.nr * r.steps for r in reqs)
    return {
        "config": {"requests": len(reqs), "arrival_rate_per_s": 20.0,
                   "grids": "nz in {256, 512, 1024, 2048}, nr = nz / 2",
                   "bodies": "sphere / torus / spheroid (aspect U[0.5, 2])",
                   "steps_per_request": "U{500..5000}", "hbm_budget": 0.8, "seed": 5,
                   "precision": args.precision, "steps_in_flight": 2},
        "summary": summ,
        "steps": len(report.step_latency_s),
        "plain_fp64_sequential": {"value": seq_cells / seq_s, "wall_s_estimate": seq_s,
                                  "speedup_served_over_sequential_fp64":
                                      summ["cell_updates_per_s"] / (seq_cells / seq_s)},
    }


def run_serve(args, world, rank, local):
    """The serving workload alone (config: Poisson arrivals, mixed grids and
    bodies, HBM-budget admission)."""
    import torch
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    with ClockSampler(local) as clocks:
        leg = serve_leg(args, dev)
    summ = leg["summary"]
    line = {
        "metric": METRIC, "value": summ["cell_updates_per_s"], "unit": UNIT, "n_gpus": world,
        "steps": leg["steps"], "warmup": 0,
        "ms_per_step": summ["step_p50_ms"], "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": args.precision, "data": "synthetic",
        "config": dict(leg["config"], workload="serve"),
        "serving": summ,
        "plain_fp64_sequential": leg["plain_fp64_sequential"],
        "clocks": clocks.summary(),
        "gpu_launches": 8 * leg["steps"],
    }
    if rank == 0:
        print(json.dumps(line), flush=True)


def run_remesh(args, world, rank, local):
    """Vorticity advection by remeshed particles (kernels/advect_particle.py),
    2048 x 1024 (nz x nr) cells, particles on the (2048, 2048) mirrored domain:
    one step = particle update + MP4 particle-to-mesh + reset, FP64, through
    the drop-in advect_vorticity_via_particles. Synthetic seeded vorticity and
    velocity with |u| dt <= 0.5 dx."""
    import torch
    from pyaxisymflow_gb300 import _native as N
    from pyaxisymflow_gb300.kernels.advect_particle import advect_vorticity_via_particles
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    nz, nr = 2048, 1024
    dx = 1.0 / nz
    rng = np.random.default_rng(7)
    f64 = dict(dtype=torch.float64, device=dev)
    Zd, Rd = np.meshgrid((np.arange(nz) + 0.5) * dx, (np.arange(2 * nr) + 0.5) * dx)
    Zt, Rt = torch.tensor(Zd, **f64), torch.tensor(Rd, **f64)
    zp, rp, vp = Zt.clone(), Rt.clone(), torch.zeros_like(Zt)
    w0 = rng.standard_normal((nr, nz))
    w = torch.tensor(w0, **f64)
    uz = torch.tensor(rng.uniform(-1, 1, (nr, nz)), **f64)
    ur = torch.tensor(rng.uniform(-1, 1, (nr, nz)), **f64)
    dt = 0.5 * dx
    stream = torch.cuda.current_stream(dev)
    step = lambda: advect_vorticity_via_particles(zp, rp, vp, w, Zt, Rt, nr, uz, ur, dx, dt)  # noqa
    for _ in range(args.warmup):
        step()
    torch.cuda.synchronize(dev)
    with ClockSampler(local) as clocks:
        t0 = time.perf_counter()
        for _ in range(args.steps):
            step()
        torch.cuda.synchronize(dev)
        wall = (time.perf_counter() - t0) / args.steps
    # device time of the particle-to-mesh kernels alone (CUDA events)
    work = torch.empty(int(N.lib().axi_p2m_mp4_work_bytes(2 * nr, nz)), dtype=torch.uint8,
                       device=dev)
    out = torch.empty_like(Zt)
    ev = [torch.cuda.Event(enable_timing=True) for _ in range(2)]
    k = max(10, args.steps // 4)
    ev[0].record(stream)
    for _ in range(k):
        N.call("axi_particles_to_mesh_2d_mp4_f64", N.ptr(Zt), N.ptr(Rt), N.ptr(vp), N.ptr(out),
               2 * nr, nz, dx, dx, 0, N.ptr(work), N.stream_of(out))
    ev[1].record(stream)
    torch.cuda.synchronize(dev)
    p2m_ms = ev[0].elapsed_time(ev[1]) / k
    hbm, _, src = peaks()
    n_part = 2 * nr * nz
    alg = 32.0 * n_part  # positions x, y, values in; mesh values out (FP64)
    line = {
        "metric": "cell-updates/s, vorticity advection by remeshed particles (FP64)",
        "value": nr * nz / wall, "unit": UNIT, "n_gpus": 1, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": wall * 1e3, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": "remesh", "grid": f"nz {nz} x nr {nr}",
                   "particles": n_part, "kernel": "MP4, unbounded",
                   "timing": "wall clock per call of the drop-in (it synchronises to check "
                             "particle displacement)"},
        # bit-exact with the reference's sequential FP64 sums, the two kernels
        # are FP64-pipe bound: 80 FP64 instructions per particle (two IEEE
        # divisions, eight MP4 weights) and 48 per mesh point (16 weight
        # products, multiplies and adds), counted by ncu on this workload
        "roofline": {"bound": "fp64", "kernel": "particles_to_mesh (stencil + gather)",
                     "achieved": FP64_INSTR_PER_PARTICLE * n_part / (p2m_ms / 1e3) / 1e9,
                     "peak": FP64_PEAK_GINSTR, "unit": "G FP64 instructions/s",
                     "frac": FP64_INSTR_PER_PARTICLE * n_part / (p2m_ms / 1e3) / 1e9
                     / FP64_PEAK_GINSTR,
                     "traffic": P2M_TRAFFIC, "traffic_unit": "bytes per call (ncu dram read + write)",
                     "peak_source": "nominal GB300 FP64, 1.25 TFLOP/s = 625 G DFMA/s",
                     "p2m_ms": p2m_ms,
                     "hbm_frac": alg / (p2m_ms / 1e3) / 1e9 / hbm,
                     "algorithmic_bytes": "32 B per particle"},
        "gpu_launches": 3 * args.steps,
        "clocks": clocks.summary(),
    }
    if not args.no_cpu_baseline:
        # the oracle (numpy, the reference's algorithm) on a 256 x 128 sample
        snr, snz = 128, 256
        sdx = 1.0 / snz
        sZ, sR = np.meshgrid((np.arange(snz) + 0.5) * sdx, (np.arange(2 * snr) + 0.5) * sdx)
        from oracle import kernels as K
        sw = rng.standard_normal((snr, snz))
        suz, sur = rng.uniform(-1, 1, (snr, snz)), rng.uniform(-1, 1, (snr, snz))
        szp, srp, svp = sZ.copy(), sR.copy(), np.zeros_like(sZ)
        n, t0 = 0, time.perf_counter()
        while time.perf_counter() - t0 < 10.0:
            K.advect_vorticity_via_particles(szp, srp, svp, sw, sZ, sR, snr, suz, sur, sdx,
                                             0.5 * sdx)
            n += 1
        secs = time.perf_counter() - t0
        line["cpu_baseline"] = {"value": snr * snz * n / secs, "unit": UNIT, "cores": 1,
                                "kind": "port",
                                "sample": f"{snz} x {snr} cells, {n} steps, numpy oracle, "
                                          f"{secs:.1f} s"}
    print(json.dumps(line), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=400)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--workload", default="ensemble64",
                    choices=["ensemble64", "sphere512", "poisson2048", "serve", "remesh",
                             "soft1024"])
    ap.add_argument("--requests", type=int, default=40)
    ap.add_argument("--precision", default="f32", choices=["f32", "f64"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-fp64-compare", action="store_true")
    ap.add_argument("--no-serve", action="store_true",
                    help="skip the continuous-batching serving leg of the default line")
    ap.add_argument("--no-tune", action="store_true",
                    help="keep the default launch choices (no autotuning)")
    ap.add_argument("--no-accuracy", action="store_true",
                    help="skip the FP32-vs-FP64 comparison over --accuracy-steps steps")
    ap.add_argument("--accuracy-steps", type=int, default=2000)
    ap.add_argument("--e2e-groups", type=int, default=2,
                    help="case groups of the end-to-end host pipeline")
    ap.add_argument("--z-transform", default="default", choices=["default", "dense", "dct"],
                    help="FP32 engine: z products as dense tensor-core GEMMs or as DCTs")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    world, rank, local = dist_setup(args)
    if args.impl == "reference":
        run_reference(args, world, rank)
    elif args.workload == "poisson2048":
        run_poisson(args, world, rank, local)
    elif args.workload == "serve":
        run_serve(args, world, rank, local)
    elif args.workload == "remesh":
        run_remesh(args, world, rank, local)
    elif args.workload == "soft1024":
        run_soft(args, world, rank, local)
    else:
        run_gb300(args, world, rank, local)


if __name__ == "__main__":
    main()
