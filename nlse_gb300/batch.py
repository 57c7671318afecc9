"""Several simulations advanced together: out_fields.

The reference runs one out_field per NLSE instance; a mixed batch (fields of
different grid sizes, powers, n2 and potentials) is several instances.
out_fields takes such a list and advances every instance's z-loop in one
CUDA graph (nlse_group_propagate): for one-component complex64 grids of
256..2048 points per axis, two launches per step for the whole batch (one
column pass over every instance's tiles, one row pass over every instance's
lines); otherwise one concurrent branch of the graph per instance.  Each instance keeps its own plan (scratch) for
this.  Callbacks are not available here (use out_field per instance).
"""

from __future__ import annotations

import ctypes as ct

import numpy as np
import torch

from . import _lib, autotune, engine
from .engine import Plan
from .nlse import count_steps


class _Group:
    def __init__(self):
        self.lib = _lib.load()
        h = ct.c_void_p()
        _lib.check(self.lib.nlse_group_create(ct.byref(h)), "group")
        self.handle = h

    def __del__(self):
        h = getattr(self, "handle", None)
        if h is not None and h.value:
            try:
                self.lib.nlse_group_destroy(h)
            except Exception:
                pass


_group = None
# whether the last out_fields ran the whole batch as two launches per step
last_fused = False


def _own_plan(simu, A: torch.Tensor) -> Plan:
    """A plan private to this simulation (concurrent branches must not share scratch)."""
    lead = simu._lead_shape(tuple(A.shape))
    na = len(simu._last_axes)
    key = (tuple(A.shape[-na:]), int(np.prod(lead)) if lead else 1, engine.dtype_code(A),
           str(A.device))
    cached = getattr(simu, "_group_plan", None)
    if cached is not None and cached[0] == key:
        return cached[1]
    plan = Plan(na, key[0], key[1], simu._comps, key[2], A.device)
    simu._group_plan = (key, plan)
    return plan


def out_fields(jobs, z: float, precision: str = "single", normalize: bool = True) -> list:
    """Propagate several (simulation, E_in) pairs over z together.

    Returns the fields in the order given, each as out_field would return it.
    """
    global _group
    if _group is None:
        _group = _Group()
    prepared = []
    try:
        for simu, E_in in jobs:
            assert tuple(E_in.shape[simu._last_axes[0]:]) == tuple(
                simu.XX.shape[simu._last_axes[0]:]), "Shape mismatch"
            if simu.propagator is None:
                simu.propagator = simu._build_propagator()
            simu._send_arrays_to_gpu()
            V = None if simu.V is None else simu.V.clone()
            A, _ = simu._prepare_output_array(E_in, normalize)
            plan = _own_plan(simu, A)
            n2_old = simu.n2
            if z > simu.L:
                simu.n2 = 0
            op = simu._operator(A, V, simu.propagator, precision, None, plan)
            # the same kernel variant as out_field on this geometry (shared tuning cache)
            autotune.maybe_tune(plan, A, op)
            prepared.append((simu, E_in, A, plan, op, count_steps(z, simu.delta_z), n2_old))
        n = len(prepared)
        plans = (ct.c_void_p * n)(*[p[3].handle.value for p in prepared])
        fields = (ct.c_void_p * n)(*[p[2].data_ptr() for p in prepared])
        ops = (_lib.Operator * n)(*[p[4].struct() for p in prepared])
        steps = (ct.c_int64 * n)(*[p[5] for p in prepared])
        dev = prepared[0][2].device
        with torch.cuda.device(dev):
            _lib.check(_group.lib.nlse_group_propagate(_group.handle, n, plans, fields, ops, steps,
                                                       engine.stream_handle(dev)),
                       "group propagate")
        global last_fused
        last_fused = bool(_group.lib.nlse_group_fused(_group.handle))
    finally:
        for item in prepared:
            item[0].n2 = item[6]
    out = []
    for simu, E_in, A, *_ in prepared:
        simu._retrieve_arrays_from_gpu()
        if isinstance(E_in, np.ndarray):
            out.append(engine.to_host(A).numpy())
        elif isinstance(E_in, torch.Tensor) and not E_in.is_cuda:
            out.append(engine.to_host(A))
        else:
            out.append(A)
    return out
