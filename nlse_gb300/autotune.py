"""Autotuner of the 2-D step's kernel variants and launch shapes, with an
on-disk cache (the role VkFFTApp(tune=True) plays for the reference's FFT
plan, NLSE/nlse.py:216).

For a plan (grid, fields, components, precision) on a given GPU it times,
over a few steps of the caller's own field and operator (on a scratch copy):
  1. every pair of available pass variants -- row pass: one CTA per line,
     TMA-fed persistent, TMA-fed persistent on line pairs in packed FP32;
     column pass: one CTA per tile, persistent bulk-copy ring, the ring on
     column pairs in packed FP32;
  2. for the fastest pair, the persistent passes' CTAs per SM (the grid is
     SMs x CTAs per SM): all that fit, or 1, 2, 3, 4 (row pass) and 1, 2
     (column pass);
keeps the fastest, and records it in a JSON cache (NLSE_AUTOTUNE_CACHE,
default ~/.cache/nlse_gb300/autotune.json, rewritten under an exclusive file
lock).  The variants compute the same arithmetic up to rounding (the
kernels contract multiply-adds differently; the pair kernels refine the
hardware reciprocal by one Newton step); only their speed differs.

NLSE_AUTOTUNE=0 turns tuning off (the plan's default variant is used),
NLSE_AUTOTUNE=1 tunes every 2-D plan; by default plans of at least 2^18
points per field are tuned, where the choice matters.
"""

from __future__ import annotations

import fcntl
import json
import os

import torch

from . import _lib, engine

MIN_POINTS = 1 << 18


def cache_path() -> str:
    return os.environ.get("NLSE_AUTOTUNE_CACHE") or os.path.join(
        os.path.expanduser("~"), ".cache", "nlse_gb300", "autotune.json")


def plan_key(plan) -> str:
    gpu = torch.cuda.get_device_name(plan.device)
    shape = "x".join(str(s) for s in plan.shape)
    return (f"v2|{gpu}|{plan.ndim}d|{shape}|fields={plan.nfields}|comps={plan.comps}"
            f"|dtype={plan.dtype}")


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


ROW_CAPS = (1, 2, 3, 4)
COL_CAPS = (1, 2)


def variants(plan) -> list:
    """(rows, cols) variant codes the plan has."""
    v = plan.get_variant()
    return [(r, c) for r in v["rows_avail"] for c in v["cols_avail"]]


def _key(cfg) -> str:
    r, c, rc, cc = cfg
    return f"rows={r},cols={c},rows_cap={rc},cols_cap={cc}"


def tune(plan, A: torch.Tensor, op, steps: int = 3, reps: int = 3, force: bool = False) -> dict:
    """Pick (and cache) the fastest variant and launch shape of `plan` for field A
    and operator op; returns the cache record."""
    key = plan_key(plan)
    rec = None if force else _read(cache_path()).get(key)
    if rec is not None and isinstance(rec.get("variant"), dict):
        v = rec["variant"]
        if (v["rows"], v["cols"]) in set(variants(plan)):
            plan.set_variant(v["rows"], v["cols"], v["rows_cap"], v["cols_cap"])
            return rec
    scratch = A.clone()
    a = torch.cuda.Event(enable_timing=True)
    b = torch.cuda.Event(enable_timing=True)
    timing = {}

    def measure(cfg):
        if cfg in timing:
            return
        plan.set_variant(*cfg)
        engine.propagate(plan, scratch, op, steps)  # warm-up
        ts = []
        for _ in range(reps):
            a.record()
            engine.propagate(plan, scratch, op, steps)
            b.record()
            torch.cuda.synchronize(A.device)
            ts.append(a.elapsed_time(b) / steps)
        plan.status()
        timing[cfg] = sorted(ts)[len(ts) // 2]

    for r, c in variants(plan):
        measure((r, c, 0, 0))
    r, c, _, _ = min(timing, key=timing.get)
    if r != _lib.ROWS_LINE:
        for cap in ROW_CAPS:
            measure((r, c, cap, 0))
    rc = min((k for k in timing if k[0] == r and k[1] == c and k[3] == 0), key=timing.get)[2]
    if c != _lib.COLS_TILE:
        for cap in COL_CAPS:
            measure((r, c, rc, cap))
    best = min(timing, key=timing.get)
    plan.set_variant(*best)
    rec = {"variant": dict(zip(("rows", "cols", "rows_cap", "cols_cap"), best)),
           "ms_per_step": {_key(k): t for k, t in timing.items()}}
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
