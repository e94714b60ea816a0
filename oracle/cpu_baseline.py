"""CPU baseline runner. MEASUREMENT INFRASTRUCTURE ONLY: it times the oracle
(the reference's algorithm on the host) for bench.py; the GPU product never
runs it.

Run as a child process (``python -m oracle.cpu_baseline CASES.json ...``) so
that the BLAS and OpenMP thread counts are fixed before numpy loads:
OMP_NUM_THREADS and OPENBLAS_NUM_THREADS set the threads, and
OPENBLAS_THREAD_TIMEOUT lets the BLAS threads sleep right after each spectral
solve instead of spinning on the cores the OpenMP kernels run on next.

kind "cport": the loop with its grid kernels in C + OpenMP (oracle/cstep.c,
the analogue of the reference's numba loops and pystencils C / OpenMP ENO3);
kind "numpy": the numpy oracle itself. A round advances every case one
timestep; rounds continue until `--seconds` have passed (at least one,
at most `--max-rounds`). Prints one JSON line.
"""
import argparse
import json
import os
import platform
import time

import numpy as np

from . import cport
from . import kernels as K
from . import simulation as sim


def cpu_model():
    """Model name of the host CPU (lscpu's or /proc/cpuinfo's field)."""
    try:
        with open("/proc/cpuinfo") as f:
            for line in f:
                if line.lower().startswith("model name"):
                    return line.split(":", 1)[1].strip()
    except OSError:
        pass
    try:
        import subprocess
        out = subprocess.run(["lscpu"], capture_output=True, text=True, timeout=10).stdout
        for line in out.splitlines():
            if line.startswith("Model name"):
                return line.split(":", 1)[1].strip()
    except (OSError, ValueError):
        pass
    return platform.processor() or platform.machine()


class Runs:
    """The oracle set up for a list of case parameter dicts (the fields of
    the engine's RigidBodyCase); solvers and advection closures are shared by
    cases of the same grid."""

    def __init__(self, params, kind):
        self.kind = kind
        self.runs = []
        solvers, advects = {}, {}
        for p in params:
            if p["sediment"]:
                oc = sim.SedimentingCase(nz=p["nz"], nr=p["nr"], dx=p["dx"], z_cm=p["z_cm"],
                                         r_sphere=p["r_sphere"], rho_f=p["rho_f"],
                                         rho_s=p["rho_s"], nu=p["nu"], lam=p["lam"],
                                         cfl=p["cfl"], kill_width=p["kill_width"],
                                         gravity=p["gravity"])
                w0 = p["noise"] * np.random.default_rng(p["seed"]).standard_normal(
                    (p["nr"], p["nz"]))
                st, coords = sim.sedimenting_init(oc, K, vorticity=w0)
            else:
                oc = sim.RigidSphereCase(nz=p["nz"], nr=p["nr"], dx=p["dx"], z_cm=p["z_cm"],
                                         r_sphere=p["r_sphere"], U0=p["U0"], Re=p["Re"],
                                         lam=p["lam"], cfl=p["cfl"],
                                         kill_width=p["kill_width"], ramp=p["ramp"],
                                         noise=p["noise"], seed=p["seed"])
                st, coords = sim.rigid_sphere_init(oc, K)
            key = (oc.nr, oc.nz, oc.dx)
            if key not in solvers:
                solvers[key] = K.FastDiagonalisationStokesSolver(oc.nr, oc.nz, oc.dx)
                advects[key] = K.gen_advect_vorticity_via_eno3(oc.dx, oc.nr, oc.nz)
            ex = cport.CStepScratch(coords[3]) if kind == "cport" else None
            self.runs.append((p["sediment"], oc, st, coords, solvers[key], advects[key], ex))
        self.cells = sum(r[1].nr * r[1].nz for r in self.runs)

    def round(self):
        t0 = time.perf_counter()
        for sed, oc, st, coords, solver, adv, ex in self.runs:
            if self.kind == "cport":
                (cport.sedimenting_step if sed else cport.rigid_sphere_step)(
                    oc, st, coords, solver, ex)
            else:
                (sim.sedimenting_step if sed else sim.rigid_sphere_step)(
                    oc, st, coords, solver, adv, K)
        return time.perf_counter() - t0


def main(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("cases", help="JSON file: a list of case parameter dicts")
    ap.add_argument("--kind", default="cport", choices=["cport", "numpy"])
    ap.add_argument("--seconds", type=float, default=20.0)
    ap.add_argument("--warmup", type=int, default=1)
    ap.add_argument("--max-rounds", type=int, default=1000)
    ap.add_argument("--dump", default=None,
                    help="write the final vorticity of every case to this .npz")
    args = ap.parse_args(argv)
    with open(args.cases) as f:
        params = json.load(f)
    runs = Runs(params, args.kind)
    threads = cport.threads() if args.kind == "cport" else 1
    for _ in range(args.warmup):
        runs.round()
    secs, rounds, times = 0.0, 0, []
    while rounds < 1 or (secs < args.seconds and rounds < args.max_rounds):
        t = runs.round()
        times.append(t)
        secs += t
        rounds += 1
    if args.dump:
        np.savez(args.dump, *[r[2].vorticity for r in runs.runs])
    out = {
        "value": runs.cells * rounds / secs, "unit": "cell-updates/s", "kind": args.kind,
        "cases": len(params), "cells_per_round": runs.cells, "rounds": rounds,
        "seconds": secs, "round_ms": [1e3 * t for t in times],
        "omp_threads": threads,
        "blas_threads": os.environ.get("OPENBLAS_NUM_THREADS", "library default"),
        "cpu_model": cpu_model(), "host_cpus": os.cpu_count(),
        "machine": platform.machine(),
    }
    print(json.dumps(out), flush=True)


if __name__ == "__main__":
    main()
