"""Autotuner of the 2-D step's kernel variants, with an on-disk cache.

For a plan (grid, fields, components, precision) on a given GPU it times each
variant the plan has -- TMA-fed persistent row passes or one CTA per line,
TMA-fed persistent column passes or one CTA per tile -- over a few steps of
the caller's own field and operator (on a scratch copy), keeps the fastest,
and records it in a JSON cache (NLSE_AUTOTUNE_CACHE, default
~/.cache/nlse_gb300/autotune.json, rewritten under an exclusive file lock).
The variants compute the same arithmetic (up to rounding: the compiler fuses
multiply-adds differently in different kernels); only their speed differs.

NLSE_AUTOTUNE=0 turns tuning off (the library's default variant is used),
NLSE_AUTOTUNE=1 tunes every 2-D plan; by default plans of at least 2^18
points per field are tuned, where the choice matters.
"""

from __future__ import annotations

import fcntl
import json
import os

import torch

from . import engine

MIN_POINTS = 1 << 18


def cache_path() -> str:
    return os.environ.get("NLSE_AUTOTUNE_CACHE") or os.path.join(
        os.path.expanduser("~"), ".cache", "nlse_gb300", "autotune.json")


def plan_key(plan) -> str:
    gpu = torch.cuda.get_device_name(plan.device)
    shape = "x".join(str(s) for s in plan.shape)
    return f"{gpu}|{plan.ndim}d|{shape}|fields={plan.nfields}|comps={plan.comps}|dtype={plan.dtype}"


def _read(path: str) -> dict:
    try:
        with open(path) as f:
            return json.load(f)
    except (OSError, ValueError):
        return {}


def _store(key: str, rec: dict) -> None:
    path = cache_path()
    os.makedirs(os.path.dirname(path) or ".", exist_ok=True)
    with open(path + ".lock", "w") as lk:
        fcntl.flock(lk, fcntl.LOCK_EX)
        data = _read(path)
        data[key] = rec
        tmp = f"{path}.{os.getpid()}.tmp"
        with open(tmp, "w") as f:
            json.dump(data, f, indent=1, sort_keys=True)
        os.replace(tmp, path)


def variants(plan) -> list:
    rows, cols, rows_ok, cols_ok = plan.get_kernels()
    return [(r, c) for r in ((True, False) if rows_ok else (False,))
            for c in ((True, False) if cols_ok else (False,))]


def tune(plan, A: torch.Tensor, op, steps: int = 3, reps: int = 3, force: bool = False) -> dict:
    """Pick (and cache) the fastest variant of `plan` for field A and operator op."""
    key = plan_key(plan)
    rec = None if force else _read(cache_path()).get(key)
    if rec is not None and tuple(rec["variant"]) in {tuple(v) for v in variants(plan)}:
        plan.set_kernels(*rec["variant"])
        return rec
    scratch = A.clone()
    a = torch.cuda.Event(enable_timing=True)
    b = torch.cuda.Event(enable_timing=True)
    timing = {}
    for v in variants(plan):
        plan.set_kernels(*v)
        engine.propagate(plan, scratch, op, steps)  # warm-up
        ts = []
        for _ in range(reps):
            a.record()
            engine.propagate(plan, scratch, op, steps)
            b.record()
            torch.cuda.synchronize(A.device)
            ts.append(a.elapsed_time(b) / steps)
        plan.status()
        timing[v] = sorted(ts)[len(ts) // 2]
    best = min(timing, key=timing.get)
    plan.set_kernels(*best)
    rec = {"variant": [bool(best[0]), bool(best[1])],
           "ms_per_step": {f"rows_tma={int(r)},cols_tma={int(c)}": t
                           for (r, c), t in timing.items()}}
    _store(key, rec)
    return rec


def maybe_tune(plan, A: torch.Tensor, op) -> None:
    """Tune a plan once per process, where the policy above asks for it."""
    if getattr(plan, "_tuned", False):
        return
    plan._tuned = True
    mode = os.environ.get("NLSE_AUTOTUNE", "")
    if mode == "0" or plan.ndim != 2:
        return
    if mode != "1" and plan.shape[0] * plan.shape[1] < MIN_POINTS:
        return
    tune(plan, A, op)
