"""Checkpoint and restore of a RigidEnsemble as one .npz file.

The reference's drivers save result fields with np.savez and pickle
(examples/TorusStreaming/torus_streaming.py:163-165) but cannot resume a
run. A snapshot here holds what the next step depends on, so a restored
ensemble continues bit-identically: per case its parameters (the
RigidBodyCase fields as JSON), omega, the body mask chi (rebuilt each step for
a sedimenting sphere), the state block (time, dt, drag, body position and
velocity, step count, ...) and the (dt, Cd) history, plus the engine options
(precision, tensor cores, z transform, refinement). psi is saved, and with
refinement its low part psi_lo too: the refined solve starts from the pair.
u_z and u_r are saved for post-processing; the next step recomputes them.
"""
import dataclasses
import json

import numpy as np

FORMAT = "pyaxisymflow-gb300 rigid ensemble snapshot 1"
FIELDS = ("omega", "psi", "u_z", "u_r", "chi")
REFINE_FIELDS = ("psi_lo",)


def _fields(refine):
    return FIELDS + (REFINE_FIELDS if refine else ())


def ensemble_snapshot(ens):
    """Host copy of everything a restore needs (waits for the device)."""
    import torch
    torch.cuda.synchronize(ens.device)
    snap = {
        "format": FORMAT,
        "precision": ens.precision,
        "tensor_cores": bool(ens.tensor_cores),
        "dct": bool(ens.dct),
        "refine": bool(ens.refine),
        "cases": [dataclasses.asdict(c) for c in ens.cases],
        "state": ens.state.cpu().numpy().copy(),
        "fields": [{n: m.fields[n].cpu().numpy().copy() for n in _fields(ens.refine)}
                   for m in ens.members],
        "history": [None if m.history is None else m.history.cpu().numpy().copy()
                    for m in ens.members],
    }
    return snap


def write_snapshot(path, snap):
    """Writes a snapshot dict as .npz (arrays stored as they are)."""
    meta = {k: snap[k] for k in ("format", "precision", "tensor_cores", "dct", "cases")}
    meta["refine"] = bool(snap.get("refine", False))
    meta["history_steps"] = [0 if h is None else int(h.shape[0]) for h in snap["history"]]
    arrays = {"meta": np.array(json.dumps(meta)), "state": snap["state"]}
    for k, f in enumerate(snap["fields"]):
        for n in _fields(meta["refine"]):
            arrays[f"{n}_{k}"] = f[n]
    for k, h in enumerate(snap["history"]):
        if h is not None:
            arrays[f"history_{k}"] = h
    np.savez(path, **arrays)


def read_snapshot(path):
    """Inverse of write_snapshot."""
    with np.load(path, allow_pickle=False) as z:
        meta = json.loads(str(z["meta"]))
        if meta.get("format") != FORMAT:
            raise ValueError(f"{path}: not a rigid ensemble snapshot")
        n = len(meta["cases"])
        snap = {k: meta[k] for k in ("format", "precision", "tensor_cores", "dct", "cases")}
        snap["refine"] = bool(meta.get("refine", False))
        snap["state"] = z["state"].copy()
        snap["fields"] = [{f: z[f"{f}_{k}"].copy() for f in _fields(snap["refine"])}
                          for k in range(n)]
        snap["history"] = [z[f"history_{k}"].copy() if meta["history_steps"][k] else None
                           for k in range(n)]
    return snap


def restore_ensemble(snap, device="cuda"):
    """A RigidEnsemble in the snapshot's state, on `device`."""
    import torch

    from ..engine import ST_WORDS, RigidBodyCase, RigidEnsemble
    cases = [RigidBodyCase(**c) for c in snap["cases"]]
    steps = {0 if h is None else h.shape[0] for h in snap["history"]}
    if len(steps) > 1:
        raise ValueError("cases with different history lengths")
    ens = RigidEnsemble(cases, precision=snap["precision"], device=device,
                        history_steps=steps.pop() if steps else 0,
                        initial_vorticity=[f["omega"] for f in snap["fields"]],
                        tensor_cores=snap["tensor_cores"], dct=snap["dct"],
                        refine=bool(snap.get("refine", False)))
    state = np.asarray(snap["state"], dtype=np.float64)
    if state.shape != (len(cases), ST_WORDS):
        raise ValueError("state block shape does not match the cases")
    for k, m in enumerate(ens.members):
        for n in _fields(ens.refine):
            m.fields[n].copy_(torch.as_tensor(snap["fields"][k][n]).to(m.fields[n].dtype))
        if m.history is not None:
            m.history.copy_(torch.as_tensor(snap["history"][k]))
        ens.state_arena[m.slot].copy_(torch.as_tensor(state[k]))
    ens.refresh_operands()
    torch.cuda.synchronize(ens.device)
    return ens


def save_checkpoint(ens, path):
    """Writes `ens` to `path` (.npz)."""
    write_snapshot(path, ensemble_snapshot(ens))


def load_checkpoint(path, device="cuda"):
    """A RigidEnsemble restored from a file written by save_checkpoint."""
    return restore_ensemble(read_snapshot(path), device)
