"""Launch autotuner of the fused engine (RigidEnsemble).

The reference specialises its pystencils kernels per grid at generation time
(pyst_kernels/advection_flux.py:9-21: fixed_grid_size, num_threads); here the
kernels are compiled once, and what depends on the mix of grid sizes in an
ensemble is how the work is scheduled: into how many plans the cases are
split (each stepped on a stream of its own), how many blocks of each stencil kernel
stay resident per SM, how far ahead they prefetch their tiles into L2, how
many persistent CTAs run the tensor-core products and in which order they
take their tiles, and in which order the z-transform items run. Every choice
gives bit-identical results (include/axisym_gb300.h: axi_tuning).

The tuner times whole steps with CUDA events for each candidate, one choice
at a time (coordinate descent from the defaults, keeping a change only when
it is faster by more than `min_gain`), restores the ensemble's state after
measuring, applies the best choices and caches them keyed by the ensemble's
grid-size mix, so ensembles of the same mix reuse them without measuring.
"""
import json
import os

import numpy as np
import torch

# candidate values per choice; the first is the default
CANDIDATES = {
    "tc_ctas_percent": (0, 75, 50),
    "tc_tile_order": (0, 1),
    "dct_item_order": (0, 1, 2),
    "prefetch_waves": (0, 2, -1),
    "vel_max_blocks": (0, 2, 4),
    "penalise_blocks": (0, 2, 3),
    "advect_blocks": (0, 2, 3),
    "plan_groups": (0, 1, 2, 3),
}


def mix_key(ens):
    """Cache key: precision, plan flags and the multiset of (nr, nz, body kind)."""
    sizes = sorted((c.nr, c.nz, "sediment" if c.sediment else "stream") for c in ens.cases)
    counts = {}
    for s in sizes:
        counts[s] = counts.get(s, 0) + 1
    mix = ";".join(f"{nr}x{nz}:{kind}*{n}" for (nr, nz, kind), n in sorted(counts.items()))
    return f"{ens.precision}|tc{int(ens.tensor_cores)}|dct{int(ens.dct)}|" \
           f"refine{int(ens.refine)}|{mix}"


def applicable(ens, name):
    if name in ("tc_ctas_percent", "tc_tile_order"):
        return ens.tensor_cores
    if name == "plan_groups":
        return ens.n_cases > 1
    if name == "dct_item_order":
        return ens.dct and ens.tensor_cores
    return True


def _save(ens):
    fields = []
    for m in ens.members:
        f = {}
        for k, v in m.fields.items():
            f[k] = [x.clone() for x in v] if isinstance(v, list) else v.clone()
        fields.append((f, None if m.history is None else m.history.clone()))
    return fields, ens.state_arena.clone()


def _restore(ens, saved):
    fields, state = saved
    for m, (f, h) in zip(ens.members, fields):
        for k, v in f.items():
            if isinstance(v, list):
                for dst, src in zip(m.fields[k], v):
                    dst.copy_(src)
            else:
                m.fields[k].copy_(v)
        if h is not None:
            m.history.copy_(h)
    ens.state_arena.copy_(state)
    torch.cuda.synchronize(ens.device)


class Autotuner:
    """Picks the launch choices of an ensemble by measurement (see the module
    docstring). `cache_path`: optional JSON file the choices persist in."""

    def __init__(self, cache_path=None, reps=5, steps_per_rep=2, min_gain=0.01):
        self.cache_path = cache_path
        self.reps = reps
        self.steps_per_rep = steps_per_rep
        self.min_gain = min_gain
        self.cache = {}
        self.measurements = 0
        self.last = None
        if cache_path and os.path.exists(cache_path):
            with open(cache_path) as f:
                self.cache = json.load(f)

    def step_ms(self, ens):
        """Median device time (ms) of one step of `ens` with its current choices."""
        stream = torch.cuda.current_stream(ens.device)
        ens.step(1)
        times = []
        for _ in range(self.reps):
            a = torch.cuda.Event(enable_timing=True)
            b = torch.cuda.Event(enable_timing=True)
            a.record(stream)
            ens.step(self.steps_per_rep)
            b.record(stream)
            b.synchronize()
            times.append(a.elapsed_time(b) / self.steps_per_rep)
        self.measurements += 1
        return float(np.median(times))

    def tune(self, ens):
        """Applies the best launch choices to `ens` (measured, or from the
        cache for the same grid-size mix) and returns them. The ensemble's
        fields and state are as before the call."""
        key = mix_key(ens)
        if key in self.cache:
            ens.set_tuning(self.cache[key])
            self.last = {"key": key, "cached": True, "choices": dict(self.cache[key])}
            return dict(self.cache[key])
        saved = _save(ens)
        best = {}
        ens.set_tuning(best)
        t_default = t_best = self.step_ms(ens)
        trials = {"default": t_default}
        for name, values in CANDIDATES.items():
            if not applicable(ens, name):
                continue
            for v in values[1:]:
                trial = dict(best)
                trial[name] = v
                ens.set_tuning(trial)
                t = self.step_ms(ens)
                trials[f"{name}={v}"] = t
                if t < t_best * (1.0 - self.min_gain):
                    best, t_best = trial, t
        _restore(ens, saved)
        ens.set_tuning(best)
        self.cache[key] = best
        if self.cache_path:
            os.makedirs(os.path.dirname(os.path.abspath(self.cache_path)), exist_ok=True)
            with open(self.cache_path, "w") as f:
                json.dump(self.cache, f, indent=1, sort_keys=True)
        self.last = {"key": key, "cached": False, "choices": dict(best),
                     "default_ms": t_default, "tuned_ms": t_best, "trials_ms": trials}
        return dict(best)
