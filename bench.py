#!/usr/bin/env python
"""Split-step throughput of nlse_gb300 on GB300, one JSON line on stdout.

Workload: the NLSE 2-D beam at NX = NY = 2048, complex64, "single" scheme
(power 1.05 W, waist 2.23 mm, window 4 waist, n2 = -1.6e-9 m^2/W,
Isat = 1e5 W/m^2, alpha = 20 /m, potential -1e-4 exp(-r^2/(70 um)^2),
E_0 (1 + 0.01 (a + ib)) with seeded normal a, b, dz = 2e-5 m).  A batch of
8 such fields (256 MiB of complex64, more than the 129 MB L2) advances
together, so every step streams from HBM; no L2 flush is needed.

Metric: field-steps/s = fields x split steps / s (one split step of one
2048^2 field is one "step").  `value` times nlse_propagate on resident
device fields (the whole loop replayed from a CUDA graph); `e2e` times the
public API, NLSE.out_field, from pinned host memory to host memory.

--impl reference: the reference's CPU path restated by the oracle
(reference CPU kernels: scipy FFT on all host cores + the numba kernels'
arithmetic in NumPy), timed on one field per step.

Multi-GPU (torchrun): every rank advances its own batch of fields (weak
scaling, no collective on the data path); timing is the max over ranks.
"""

from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import tempfile
import threading
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

N = 2048
BATCH = 8
DZ = 2e-5
WAIST, WAIST2, POWER, N2, ISAT, ALPHA, L = 2.23e-3, 70e-6, 1.05, -1.6e-9, 1e5, 20, 10e-3
METRIC = "steps/s at 2048^2 c64 (field-steps/s, 8-field batch)"
UNIT = "field-steps/s"
# algorithmic bytes per grid point per step (complex64 field, real f32 potential)
B_ROW = 16 + 4   # inverse+forward row pass: read A, write A, read V
B_COL = 16       # column pass: read A, write A (propagator L2-resident, shared by the batch)


SUR_TRAIN, SUR_TEST, SUR_EPOCHS, SUR_COARSE, SUR_EVERY = 20480, 4096, 4, 5, 16


def surrogate_leg(dev, n_train=SUR_TRAIN, n_test=SUR_TEST, epochs=SUR_EPOCHS):
    """Surrogate vs solver on 256^2 fields (the 164-field distributions restricted to
    256^2): train on solver pairs, then time, from device-resident inputs, the plain
    batched solver and the surrogate (coarse Strang solve + network + judge with a
    1-in-16 re-solved sample) on held-out fields."""
    import torch

    from nlse_gb300 import surrogate as sg

    def T():
        torch.cuda.synchronize()
        return time.perf_counter()

    t0 = T()
    train = sg.sample_inputs(n_train, seed=21, device=dev)
    Ef = sg.solve(train)
    t1 = T()
    Ec = sg.solve(train, SUR_COARSE)
    s = sg.Surrogate(dev, seed=0, coarse=SUR_COARSE)
    s.fit(train, Ef, epochs=epochs, batch=32, lr=2e-3, E_c=Ec)
    t2 = T()
    s.net.check_status()
    del train, Ef, Ec
    test = sg.sample_inputs(n_test, seed=22, device=dev)
    warm = sg.subset(test, slice(0, 64))
    sg.solve(warm)
    s.judge(warm, s.predict(warm), every=SUR_EVERY)
    ta = T()
    ref = sg.solve(test)
    tb = T()
    P, Ec = s.predict(test, with_coarse=True)
    tc = T()
    out, rep = s.judge(test, P, every=SUR_EVERY, seed=23)
    td = T()
    xin, xs, _ = s.features(test, Ec)
    tn0 = T()
    s.net.predict(xin, xs)
    tn1 = T()
    q = [0.5, 0.9, 0.99, 1.0]
    e_c, e_p, e_o = (sg.rel_l2(x, ref).cpu().numpy() for x in (Ec, P, out))

    def stats(e):
        return {"quantiles_50_90_99_max": [float(v) for v in np.quantile(e, q)],
                "pass_1e-2": float((e <= 1e-2).mean())}

    return {"workload": "256^2 c64 fields, 164-field distributions, L=10 mm (201 solver steps)",
            "fields": n_test, "solver_fields_per_s": n_test / (tb - ta),
            "surrogate_fields_per_s": n_test / (td - tb),
            "surrogate_without_judge_fields_per_s": n_test / (tc - tb),
            "network_only_fields_per_s": n_test / (tn1 - tn0),
            "speedup_vs_solver": (tb - ta) / (td - tb),
            "coarse_strang_steps": SUR_COARSE, "judge_sample": f"1 in {SUR_EVERY}",
            "rel_l2_vs_solver": {"coarse_alone": stats(e_c), "coarse_plus_network": stats(e_p),
                                 "after_judge": stats(e_o)},
            "judge": rep,
            "train": {"pairs": n_train, "epochs": epochs, "batch": 32, "data_s": t1 - t0,
                      "train_s": t2 - t1, "final_loss": float(np.mean(s.history[-50:]))}}


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=200)
    ap.add_argument("--warmup", type=int, default=20)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--batch", type=int, default=BATCH)
    ap.add_argument("--no-surrogate", action="store_true",
                    help="leave out the surrogate-vs-solver leg (about a minute)")
    ap.add_argument("--mixed-only", action="store_true",
                    help="only time the 164-field mixed batch (--steps steps per call; for "
                         "profiling)")
    ap.add_argument("--cnlse-only", type=int, default=0, metavar="STEPS",
                    help="only run the CNLSE 1024^2 nonlocal configuration: three out_field "
                         "calls of STEPS steps, the last one timed (for profiling)")
    ap.add_argument("--network-only", type=int, default=0, metavar="FIELDS",
                    help="only time the surrogate network's inference on FIELDS random "
                         "256^2 inputs (--steps passes after one warm-up; for profiling)")
    return ap.parse_args()


def fields(XX, YY, batch, seed):
    rng = np.random.default_rng(seed)
    E = np.exp(-(XX**2 + YY**2) / WAIST**2)
    a = rng.standard_normal((batch, *XX.shape))
    b = rng.standard_normal((batch, *XX.shape))
    return (E * (1 + 0.01 * (a + 1j * b))).astype(np.complex64)


def potential(XX, YY):
    return (-1e-4 * np.exp(-(XX**2 + YY**2) / WAIST2**2)).astype(np.complex64)


def peaks():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi samples during the timed region (read only)."""

    Q = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.proc = None
        self.path = Path(tempfile.mkstemp(prefix="clocks_", suffix=".csv")[1])

    def start(self):
        try:
            self.f = open(self.path, "w")
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.Q}",
                 "--format=csv,noheader,nounits", "-lms", "100"], stdout=self.f,
                stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None
        time.sleep(0.3)

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        self.proc.wait(timeout=10)
        self.f.close()
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in self.path.read_text().splitlines():
            parts = [p.strip() for p in line.split(",")]
            if len(parts) < 7:
                continue
            try:
                sm.append(float(parts[0]))
                mx = float(parts[1])
            except ValueError:
                continue
            for nm, v in zip(names, parts[3:7]):
                if v.lower().startswith("active"):
                    reasons.add(nm)
        self.path.unlink(missing_ok=True)
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": mx,
                "reasons": sorted(reasons), "samples": len(sm)}


def load_traffic():
    """DRAM bytes per launch of the column pass from the committed ncu summary, if any."""
    p = ROOT / "profiles" / "traffic.json"
    if p.exists():
        try:
            return json.loads(p.read_text())
        except Exception:
            return None
    return None


# ---------------------------------------------------------------------------
# reference CPU path (oracle restatement), bounded sample
# ---------------------------------------------------------------------------
def cpu_reference(steps_per_sample: int, reps: int, warmup: int):
    from oracle import nlse_oracle as orc

    cores = os.cpu_count() or 1
    orc.WORKERS = cores
    o = orc.OracleNLSE(ALPHA, POWER, 4 * WAIST, N2, None, L, NX=N, NY=N, Isat=ISAT,
                       cpu_kernels=True)
    o.delta_z = DZ
    V = potential(o.XX, o.YY)
    A = o.prepare(fields(o.XX, o.YY, 1, 0)[0], True)
    prop = o.build_propagator()
    for _ in range(warmup):
        o.split_step(A, V, prop, "single")
    times = []
    for _ in range(reps):
        t0 = time.perf_counter()
        for _ in range(steps_per_sample):
            o.split_step(A, V, prop, "single")
        times.append(time.perf_counter() - t0)
    t = float(np.sum(times))
    return {"value": reps * steps_per_sample / t, "unit": UNIT, "cores": cores,
            "kind": "port",
            "sample": f"{reps * steps_per_sample} split steps of one 2048^2 complex64 field, "
                      "reference CPU-path arithmetic (kernels_cpu) with scipy.fft on all "
                      "host threads"}, t


def run_reference(args):
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    cb, _ = cpu_reference(1, args.steps, max(0, min(args.warmup, 3)))
    line = {"metric": METRIC, "value": cb["value"], "unit": UNIT, "impl": "reference",
            "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": 1e3 / cb["value"], "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "c64", "data": "synthetic (seeded)",
            "config": {"workload": "NLSE 2-D 2048^2 complex64 single scheme, dz=2e-5 m, "
                                   "potential well, noisy Gaussian beam; one field per step",
                       "l2": "CPU run"},
            "cpu_baseline": cb,
            "e2e": {"value": cb["value"], "unit": UNIT, "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


# ---------------------------------------------------------------------------
# GB300 path
# ---------------------------------------------------------------------------
def gpu_stand_in(dev, E_host, V, sim, plan, op, steps=20, warmup=3):
    """The reference's GPU-path step, measured as a stand-in for its VkFFT path.

    The reference's GPU path needs cupy and pyvkfft, which are not installed,
    so its arithmetic is restated here on torch.fft (cuFFT) and torch
    elementwise operations, step by step as NLSE.split_step "single" runs it
    (nlse.py:372-487): forward 2-D FFT, times the propagator, inverse FFT
    (normalised), square_mod (kernels_gpu.py:179-190: |A|**2), nl_prop
    (kernels_gpu.py:4-37).  Baseline only; the product never uses cuFFT.  The
    elementwise part is unfused here (cupy fuses it into one kernel), so the
    FFT + propagator part is also reported alone as a bound the reference
    cannot beat.  A cross-check compares its field with the product's after
    the same steps."""
    import torch
    from scipy.constants import c, epsilon_0

    from nlse_gb300 import engine

    A0 = torch.from_numpy(E_host).to(dev)
    P = sim.propagator
    P = (P if isinstance(P, torch.Tensor) else torch.from_numpy(np.asarray(P))).to(dev)
    Vk = torch.from_numpy(np.asarray(sim.k / 2 * V)).to(dev)
    g = sim.k / 2 * N2 * c * epsilon_0
    isat = 2 * ISAT / (epsilon_0 * c)
    a2 = ALPHA / 2

    def step(A):
        A = torch.fft.ifft2(torch.fft.fft2(A).mul_(P))
        A_sq = torch.abs(A) ** 2
        sat = 1 / (1 + A_sq / isat)
        arg = 1j * g * A_sq * sat
        arg = arg - a2 * sat
        arg = arg + 1j * Vk
        arg = arg * DZ
        return A.mul_(torch.exp(arg))

    def fft_part(A):
        return torch.fft.ifft2(torch.fft.fft2(A).mul_(P))

    def timed(f):
        A = A0.clone()
        for _ in range(warmup):
            A = f(A)
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        a.record()
        for _ in range(steps):
            A = f(A)
        b.record()
        torch.cuda.synchronize()
        return a.elapsed_time(b) / 1e3 / steps

    t_step, t_fft = timed(step), timed(fft_part)
    # the same steps on the product, from the same field
    A = A0.clone()
    for _ in range(steps):
        A0 = step(A0)
    engine.propagate(plan, A, op, steps, 0, graph=False)
    torch.cuda.synchronize()
    err = float(torch.linalg.vector_norm(A - A0) / torch.linalg.vector_norm(A0))
    nf = E_host.shape[0]
    return {"field_steps_per_s": nf / t_step, "fft_and_propagator_only_field_steps_per_s": nf / t_fft,
            "rel_l2_vs_product_after_steps": err, "steps_compared": steps,
            "note": "reference VkFFT GPU path unavailable (cupy and pyvkfft are not installed); "
                    "stand-in: the reference's split_step arithmetic on torch.fft (cuFFT) and "
                    "unfused torch elementwise ops, same 8-field 2048^2 workload, device-resident"}


def run_gb300(args):
    import torch

    import nlse_gb300 as ng
    from nlse_gb300 import _build, _lib, engine

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    dist = None
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl", device_id=dev)
    _build.build()
    B = args.batch

    sim = ng.NLSE(ALPHA, POWER, 4 * WAIST, N2, None, L, NX=N, NY=N, Isat=ISAT)
    sim.delta_z = DZ
    V = potential(sim.XX, sim.YY)
    sim.V = V
    # weak scaling: the job is world x B whole fields; this rank owns one block
    from nlse_gb300.shard import field_block

    blk = field_block(world * B, rank, world)
    E_host = fields(sim.XX, sim.YY, blk.stop - blk.start, 1000 + blk.start)
    A = torch.from_numpy(E_host).to(dev)
    sim.propagator = sim._build_propagator()
    plan = sim._build_fft_plan(A)[0]
    op = sim._operator(A, torch.from_numpy(V).to(dev), sim.propagator, "single")

    # kernel variants picked by the autotuner (cached per GPU and geometry)
    from nlse_gb300 import autotune

    tuned = autotune.tune(plan, A.clone(), op)
    # warm-up (also captures and instantiates the graph)
    engine.propagate(plan, A, op, args.warmup, 0, graph=True)
    torch.cuda.synchronize()

    sampler = ClockSampler(local)
    sampler.start()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    e0.record()
    engine.propagate(plan, A, op, args.steps, 0, graph=True)
    e1.record()
    torch.cuda.synchronize()
    if dist:
        dist.barrier()
    clocks = sampler.stop()
    t = e0.elapsed_time(e1) / 1e3
    if dist:
        tt = torch.tensor([t], device=dev)
        dist.all_reduce(tt, op=dist.ReduceOp.MAX)
        t = float(tt.item())
    value = world * B * args.steps / t
    launches = 1 + 2 * args.steps

    # per-kernel durations on the launching stream (torch's current stream),
    # inside the same (column pass, row pass) sequence the loop runs: an event
    # after every launch.  (A pass repeated on its own runs at other speeds:
    # the row pass 230-275 us instead of ~214 us, as its L2 contents differ.)
    def time_passes(reps=20):
        engine.run_pass(plan, A, op, _lib.PASS_FORWARD)
        for _ in range(3):
            engine.run_pass(plan, A, op, _lib.PASS_LINEAR)
            engine.run_pass(plan, A, op, _lib.PASS_INV_NL_FWD)
        torch.cuda.synchronize()
        evs = [torch.cuda.Event(enable_timing=True) for _ in range(2 * reps + 1)]
        evs[0].record()
        for i in range(reps):
            engine.run_pass(plan, A, op, _lib.PASS_LINEAR)
            evs[2 * i + 1].record()
            engine.run_pass(plan, A, op, _lib.PASS_INV_NL_FWD)
            evs[2 * i + 2].record()
        engine.run_pass(plan, A, op, _lib.PASS_LINEAR)
        engine.run_pass(plan, A, op, _lib.PASS_INV_NL)
        torch.cuda.synchronize()
        col = sum(evs[2 * i].elapsed_time(evs[2 * i + 1]) for i in range(reps)) / reps
        row = sum(evs[2 * i + 1].elapsed_time(evs[2 * i + 2]) for i in range(reps)) / reps
        return col / 1e3, row / 1e3

    t_col, t_row = time_passes()
    npix = N * N * B
    peak, peak_kind = peaks()
    kern = {
        "column_pass": {"s": t_col, "bytes": B_COL * npix},
        "row_pass_inv_nl_fwd": {"s": t_row, "bytes": B_ROW * npix},
    }
    dom = max(kern, key=lambda k: kern[k]["s"])
    ach = kern[dom]["bytes"] / kern[dom]["s"] / 1e9
    traffic = load_traffic()
    roof = {"bound": "hbm", "kernel": dom, "achieved": round(ach, 1), "peak": peak,
            "peak_kind": f"{peak_kind} hbm_gbs", "unit": "GB/s", "frac": round(ach / peak, 4),
            "traffic": (traffic or {}).get(dom),
            "algorithmic_bytes_per_launch": kern[dom]["bytes"],
            "launch_ms": round(kern[dom]["s"] * 1e3, 4),
            "other_kernels": {k: {"launch_ms": round(v["s"] * 1e3, 4),
                                  "achieved_gbs": round(v["bytes"] / v["s"] / 1e9, 1)}
                              for k, v in kern.items() if k != dom}}
    step_model_gbs = 52 * N * N * B * args.steps / t / 1e9 / world

    # e2e through the public API: pinned host field -> out_field -> host field
    e2e = None
    cpu_base = None
    if True:
        Eh = torch.from_numpy(E_host).pin_memory()
        sim2 = ng.NLSE(ALPHA, POWER, 4 * WAIST, N2, None, L, NX=N, NY=N, Isat=ISAT)
        sim2.delta_z = DZ
        sim2.V = V
        z = (args.steps - 0.5) * DZ
        nst = ng.count_steps(z, DZ)
        sim2.out_field(Eh, z, verbose=False)  # warm-up (plan, graph)
        torch.cuda.synchronize()
        if dist:
            dist.barrier()
        tes = []
        for _ in range(5):
            t0 = time.perf_counter()
            out = sim2.out_field(Eh, z, verbose=False)
            torch.cuda.synchronize()
            tes.append(time.perf_counter() - t0)
        te = float(np.median(tes))
        if dist:
            tt = torch.tensor([te], device=dev)
            dist.all_reduce(tt, op=dist.ReduceOp.MAX)
            te = float(tt.item())
        h2d = E_host.nbytes + V.nbytes + sim2.propagator.nbytes
        e2e = {"value": world * B * nst / te, "unit": UNIT,
               "h2d_bytes_per_step": int(h2d / nst), "d2h_bytes_per_step": int(out.numpy().nbytes / nst),
               "steps_per_call": nst, "calls": len(tes),
               "note": "out_field calls from pinned host memory to a new host tensor, median "
                       "of 5 calls (loops of at most 100 steps go through out_field's "
                       "copy/compute pipeline: the first and the last field alone, the others "
                       "together, uploads and downloads overlapping the propagation; longer "
                       "loops run unsplit); "
                       "h2d/d2h bytes per call divided by its steps"}
        # single 2048^2 field, the configuration's own 501-step loop (L2-resident)
        s1 = ng.NLSE(ALPHA, POWER, 4 * WAIST, N2, None, L, NX=N, NY=N, Isat=ISAT)
        s1.delta_z = DZ
        s1.V = V
        E1 = torch.from_numpy(E_host[0]).to(dev)
        s1.out_field(E1, L, verbose=False)
        torch.cuda.synchronize()
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        flush = torch.empty(256 * 2**20, dtype=torch.uint8, device=dev)
        ts = []
        for _ in range(3):
            flush.fill_(1)  # evict L2 between timed loops
            a.record()
            s1.out_field(E1, L, verbose=False)
            b.record()
            torch.cuda.synchronize()
            ts.append(a.elapsed_time(b) / 1e3)
        single = {"steps": ng.count_steps(L, DZ), "steps_per_s": ng.count_steps(L, DZ) / min(ts),
                  "note": "one 2048^2 field, 501-step out_field loop from device memory, "
                          "L2 flushed between loops (the field itself fits in L2)"}

        def loop_time(sim, E, z, reps=3):
            sim.out_field(E, z, verbose=False)
            torch.cuda.synchronize()
            best = None
            for _ in range(reps):
                flush.fill_(1)
                a.record()
                sim.out_field(E, z, verbose=False)
                b.record()
                torch.cuda.synchronize()
                t_ = a.elapsed_time(b) / 1e3
                best = t_ if best is None else min(best, t_)
            return best

        # the same loop in complex128 (the configuration's FP64 run); real FP32 potential:
        # 3 sweeps x 2 x 16 B + 4 B per point and step
        E1d = torch.from_numpy(E_host[0].astype(np.complex128)).to(dev)
        td = loop_time(s1, E1d, L)
        nst1 = ng.count_steps(L, DZ)
        single_c128 = {"steps": nst1, "steps_per_s": nst1 / td,
                       "gbs_100B_per_pt": round(100 * N * N * nst1 / td / 1e9, 1),
                       "note": "one 2048^2 complex128 field, 501-step out_field loop from "
                               "device memory, L2 flushed between loops"}
        # the coupled 1024^2 configuration: CNLSE, both components, Gaussian nonlocal
        # kernel (sigma 100 um on a 67^2 support), L = 20 mm at dz = 5e-5 (400 steps)
        s3, E3, LC = cnlse_setup(dev)
        tc = loop_time(s3, E3, LC)
        nst3 = ng.count_steps(LC, 5e-5)
        cnlse = {"steps": nst3, "steps_per_s": nst3 / tc,
                 "note": "CNLSE 1024^2 complex64, two components, Gaussian nonlocal kernel "
                         "(linear convolution on a zero-padded 2048^2 grid every step), "
                         "400-step out_field loop from device memory, L2 flushed between loops"}
    mixed = mixed_batch_leg(args.steps, dev, rank, world, dist)
    stand_in = None
    if rank == 0:
        stand_in = gpu_stand_in(dev, E_host, V, sim, plan, op)
    sur = None
    if rank == 0 and not args.no_surrogate:
        sur = surrogate_leg(dev)
    if rank == 0:
        cb, _ = cpu_reference(4, 3, 1)
        cpu_base = cb
        line = {"metric": METRIC, "value": round(value, 2), "unit": UNIT, "n_gpus": world,
                "steps": args.steps, "warmup": args.warmup,
                "ms_per_step": round(t / args.steps * 1e3, 5), "higher_is_better": True,
                "scaling": "weak", "vs_baseline": None, "dtype": "c64",
                "data": "synthetic (seeded noisy Gaussian beams)",
                "config": {"workload": "NLSE 2-D 2048^2 complex64 single scheme, dz=2e-5 m, "
                                       "potential well, noisy Gaussian beam (the 2048^2 "
                                       "configuration), batch of fields per GPU",
                           "fields_per_gpu": B, "grid": [N, N], "scheme": "single",
                           "l2": "inputs larger than L2 (256 MiB per GPU)",
                           "step_model_gbs_52B_per_pt": round(step_model_gbs, 1),
                           "kernel_variant": tuned,
                           "single_field_loop": single, "single_field_loop_c128": single_c128,
                           "cnlse_1024_nonlocal": cnlse, "mixed_batch_164": mixed,
                           "reference_gpu_stand_in": stand_in,
                           "surrogate_256": sur},
                "roofline": roof, "cpu_baseline": cpu_base, "e2e": e2e,
                "gpu_launches": launches, "clocks": clocks}
        print(json.dumps(line), flush=True)
    if dist:
        dist.destroy_process_group()


MIXED_GROUPS = [(96, 256), (48, 512), (16, 1024), (4, 2048)]


def mixed_batch_leg(steps, dev, rank=0, world=1, dist=None):
    """The 164-field mixed batch (96 @ 256^2, 48 @ 512^2, 16 @ 1024^2, 4 @ 2048^2)
    through out_fields, inputs resident on the device: median of 7 calls of
    `steps` steps, and the loop's own rate from calls of steps and 3 x steps
    (the difference removes the per-call set-up)."""
    import torch

    import nlse_gb300 as ng
    from nlse_gb300 import batch as ngb
    from tests import cases

    jobs = cases.mixed_batch(MIXED_GROUPS, seed=11 + rank)
    for sim, _ in jobs:
        # the per-field potentials and the propagators stay on the device
        sim.V = torch.from_numpy(sim.V).to(dev)
        sim.propagator = torch.from_numpy(sim._build_propagator()).to(dev)
    jobs = [(sim, torch.from_numpy(E).to(dev)) for sim, E in jobs]
    nf = sum(n for n, _ in MIXED_GROUPS)

    def calls(nsteps, reps=7):
        z = (nsteps - 0.5) * 5e-5
        ng.out_fields(jobs, z)
        torch.cuda.synchronize()
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        if dist:
            dist.barrier()
        ts = []
        for _ in range(reps):
            a.record()
            ng.out_fields(jobs, z)
            b.record()
            torch.cuda.synchronize()
            ts.append(a.elapsed_time(b) / 1e3)
        t = float(np.median(ts))
        if dist:
            tt = torch.tensor([t], device=dev)
            dist.all_reduce(tt, op=dist.ReduceOp.MAX)
            t = float(tt.item())
        return ng.count_steps(z, 5e-5), t, ts

    nb, tb, tbs = calls(steps)
    nb3, tb3, _ = calls(3 * steps)
    loop = (tb3 - tb) / (nb3 - nb)
    rates = sorted(world * nf * nb / x for x in tbs)
    return {"fields": nf, "steps": nb, "field_steps_per_s": world * nf * nb / tb,
            "replays": len(tbs), "field_steps_per_s_min_max": [rates[0], rates[-1]],
            "loop_field_steps_per_s": world * nf / loop, "loop_ms_per_step": loop * 1e3,
            "call_setup_ms": (tb - nb * loop) * 1e3,
            "fused": ngb.last_fused, "launches_per_step": 2 if ngb.last_fused else None,
            "note": "96@256^2 + 48@512^2 + 16@1024^2 + 4@2048^2 complex64, per-field power, n2 "
                    "and potentials, fields and potentials device-resident; out_fields (one "
                    "CUDA graph: one column pass and one row pass per step over every grid "
                    "size when fused); field_steps_per_s: median of 7 calls of `steps` steps "
                    "including each call's set-up (parameter blocks, normalisation, graph "
                    "update, first forward pass); loop_*: per step, from the difference "
                    f"between calls of {3 * steps} and {steps} steps"}


def mixed_only(args):
    """Only the mixed-batch leg (for profiling its kernels)."""
    import torch

    from nlse_gb300 import _build

    _build.build()
    dev = torch.device("cuda", 0)
    torch.cuda.set_device(dev)
    print(json.dumps({"mixed_batch_164": mixed_batch_leg(args.steps, dev)}))


def cnlse_setup(dev):
    """The coupled 1024^2 configuration: CNLSE, both components, Gaussian nonlocal
    kernel (sigma 100 um on a 67^2 support), L = 20 mm at dz = 5e-5 (400 steps)."""
    import torch

    import nlse_gb300 as ng

    NC, LC = 1024, 20e-3
    s3 = ng.CNLSE(ALPHA, 0.5, 4 * WAIST, N2, -0.8e-9, None, LC, NX=NC, NY=NC, Isat=ISAT,
                  nl_length=100e-6)
    s3.delta_z, s3.power2, s3.n22 = 5e-5, 0.05, N2
    dxc = 4 * WAIST / NC
    rr = np.arange(-33, 34) * dxc
    kern = np.exp(-(rr[:, None] ** 2 + rr[None, :] ** 2) / (2 * (100e-6) ** 2))
    s3.nl_profile = kern / kern.sum()
    E3 = np.array([np.exp(-(s3.XX**2 + s3.YY**2) / w**2) for w in (1.5e-3, 0.5e-3)])
    return s3, torch.from_numpy(E3.astype(np.complex64)).to(dev), LC


def cnlse_only(args):
    """Three out_field calls of the CNLSE nonlocal configuration (the last one timed)."""
    import torch

    from nlse_gb300 import _build

    _build.build()
    dev = torch.device("cuda", 0)
    s3, E3, _ = cnlse_setup(dev)
    z = (args.cnlse_only - 0.5) * 5e-5
    for _ in range(2):
        s3.out_field(E3, z, verbose=False)
    a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    a.record()
    s3.out_field(E3, z, verbose=False)
    b.record()
    torch.cuda.synchronize()
    t = a.elapsed_time(b) / 1e3
    print(json.dumps({"cnlse_1024_nonlocal_only": {"steps": args.cnlse_only,
                                                   "steps_per_s": round(args.cnlse_only / t, 1)}}))


def network_only(args):
    """Inference throughput of an initialised surrogate network on random inputs."""
    import torch

    from nlse_gb300 import _build
    from nlse_gb300.fno import FNO, N as FN

    _build.build()
    nf = args.network_only
    net = FNO("cuda")
    g = torch.Generator(device="cuda").manual_seed(0)
    xin = torch.randn((nf, FN, FN, 3), device="cuda", generator=g) * 0.3
    xs = torch.randn((nf, 2), device="cuda", generator=g)
    net.predict(xin, xs, chunk=nf)
    a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    a.record()
    for _ in range(args.steps):
        net.predict(xin, xs, chunk=nf)
    b.record()
    torch.cuda.synchronize()
    net.check_status()
    t = a.elapsed_time(b) / 1e3 / args.steps
    print(json.dumps({"surrogate_network_only": {"fields": nf, "passes": args.steps,
                                                 "ms_per_pass": round(t * 1e3, 3),
                                                 "fields_per_s": round(nf / t, 1)}}))


def main():
    args = parse()
    if args.network_only:
        network_only(args)
    elif args.cnlse_only:
        cnlse_only(args)
    elif args.mixed_only:
        mixed_only(args)
    elif args.impl == "reference":
        run_reference(args)
    else:
        run_gb300(args)


if __name__ == "__main__":
    main()
