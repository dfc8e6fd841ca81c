"""Benchmark of the fused time-step kernel on the headline workload.

Workload (the reference's headline plain-method case at full size): the
focused-beam app on a 4096 (axial) x 2048 (lateral) FP32 grid, 24 cells per
wavelength, aperture 1024 cells, focus 3000 cells, Mach 5e-3 reached over 5
periods, beta 3.5, dissipation 5e-5, CFL 0.9. Synthetic: the state starts at
rest and the source drives it; no dataset is involved.

One bench step = one accepted time step of the whole grid (boundary hook,
y and x sweeps, CFL reduction and dt control, diffusion).

  value : Gcell-updates/s over K back-to-back steps, device-timed with CUDA
          events on the solver's stream, state resident in HBM.
  e2e   : the same metric through the C ABI a user calls, with host buffers:
          fv_set_state from pinned host memory, K synchronous fv_run(1)
          calls (each returns the step's stats: dt, T, CFL, status), and
          fv_get_state back to pinned host memory, all inside the timed
          region.
  roofline : the step kernel against the measured HBM copy bandwidth, with
          24 algorithmic bytes per cell-update (3 FP32 fields read once and
          written once) over the step kernel's own duration (CUDA events
          between an attempt's launches); `issue` carries the kernel's
          issue-slot figures from the committed ncu summary.
  cpu_baseline : the oracle's CPU restatement (FP32, OpenMP over rows, all
          host cores) on a bounded sample of the same grid.

`--impl reference` times that CPU restatement alone (the reference's GPU
code cannot be built with current toolkits; its arithmetic runs on the host
through the restatement) and prints the same line with "impl": "reference".
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

ALG_BYTES_PER_CELL = 24  # 3 FP32 fields read + 3 written
L2_BYTES = 129 * 1024 * 1024
PROFILE_TRAFFIC = os.path.join(ROOT, "profiles", "step_kernel_focused_beam_4096x2048.traffic.json")


def workload_params(exact: bool):
    from fivonagi_gb300 import FV_APP_FOCUSED_BEAM, default_params
    return default_params(FV_APP_FOCUSED_BEAM).replace(exact=1 if exact else 0)


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


def max_over_ranks(x: float, device) -> float:
    """The largest of every rank's x (the job's time is its slowest rank's)."""
    import torch
    import torch.distributed as dist

    t = torch.tensor([float(x)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def replica_throughput(cells: int, steps_per_rank: int, world: int, ms: float) -> float:
    """Gcell-updates/s of the whole job: every rank advances its own replica
    by steps_per_rank steps; ms is the slowest rank's time."""
    return cells * steps_per_rank * world / (ms * 1e-3) / 1e9


class ClockSampler:
    """nvidia-smi clock and throttle-reason samples during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int):
        self.gpu = gpu_index
        self.proc = None
        self.lines = []
        self.thread = None

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.gpu}", f"--query-gpu={self.FIELDS}",
                 "--format=csv,noheader,nounits", "-lms", "100"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except (FileNotFoundError, OSError):
            self.proc = None
            return
        self.thread = threading.Thread(target=self._read, daemon=True)
        self.thread.start()

    def _read(self):
        for ln in self.proc.stdout:
            self.lines.append(ln.strip())

    def stop(self) -> dict:
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        if self.thread:
            self.thread.join(timeout=2)
        sm, smax, reasons, power = [], [], set(), []
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [x.strip() for x in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax.append(float(parts[2]))
                power.append(float(parts[3]))
            except ValueError:
                continue
            for name, val in zip(names, parts[5:9]):
                if val.lower() == "active":
                    reasons.add(name)
        return {
            "sm_mhz": statistics.median(sm) if sm else None,
            "sm_max_mhz": max(smax) if smax else None,
            "power_w_max": max(power) if power else None,
            "samples": len(sm),
            "reasons": sorted(reasons),
        }


def measured_peak():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(path) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    except (OSError, KeyError, ValueError):
        return 6800.0, "fallback"


def profiled_figures():
    """DRAM bytes per launch and issue figures of the step kernel from the
    committed ncu summary (profiles/), or None."""
    try:
        with open(PROFILE_TRAFFIC) as f:
            return json.load(f)
    except (OSError, ValueError):
        return None


def cpu_sample(params, seconds: float, max_steps: int):
    """The oracle (FP32 CPU restatement) on the full grid, bounded in time."""
    import numpy as np

    from oracle import oracle
    threads = os.cpu_count() or 1
    oracle.set_threads(threads)
    sim = oracle.OracleSim(params, np.float32, math="fvm")
    sim.init_state()
    sim.run(1)  # warm-up: first touch of the scratch grids
    steps = 0
    t0 = time.perf_counter()
    while steps < max_steps and time.perf_counter() - t0 < seconds:
        sim.run(1)
        steps += 1
    dt = time.perf_counter() - t0
    sim.close()
    cells = params.nx * params.ny
    return {
        "value": cells * steps / dt / 1e9,
        "unit": "Gcell-updates/s",
        "cores": threads,
        "kind": "port",
        "sample": f"{steps} accepted steps of the full {params.nx}x{params.ny} grid from rest "
                  f"({dt:.1f} s, FP32, OpenMP over rows)",
    }


def run_reference(args):
    rank, world, _ = dist_env()
    if rank != 0:
        return 0
    params = workload_params(exact=True)
    res = cpu_sample(params, seconds=25.0, max_steps=max(1, args.steps))
    line = {
        "impl": "reference",
        "metric": "Gcell-updates/s",
        "value": res["value"],
        "unit": "Gcell-updates/s",
        "n_gpus": args.gpus,
        "steps": args.steps,
        "warmup": args.warmup,
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f32",
        "data": "synthetic",
        "config": {"workload": "focused-beam 4096x2048 FP32 (plain method, full size)",
                   "nx": params.nx, "ny": params.ny, "runs": "CPU restatement of the reference "
                   "arithmetic on the host cores (the reference's CUDA does not build on current toolkits)"},
        "cpu_baseline": {"kind": res["kind"], "cores": res["cores"], "sample": res["sample"],
                         "value": res["value"], "unit": res["unit"]},
        "e2e": {"value": res["value"], "unit": "Gcell-updates/s", "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line))
    return 0


def run_gpu(args):
    import ctypes as C

    import numpy as np
    import torch

    from fivonagi_gb300 import Simulation, _abi, autotune

    rank, world, local = dist_env()
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", init_method="env://")
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    exact = not args.fast
    params = workload_params(exact)
    cells = params.nx * params.ny

    # ---- launch shape and division from the autotuner (cached; outside every
    # timed region), or as given (--blocks/--division: few launches before a
    # profiler's capture)
    DIVISIONS = {"default": _abi.FV_DIVISION_DEFAULT, "fma": _abi.FV_DIVISION_FMA, "exact": _abi.FV_DIVISION_EXACT}
    if args.blocks > 0:
        blocks, division = args.blocks, DIVISIONS[args.division]
    else:
        blocks, division = autotune.tune(params)
        if args.division != "default":
            division = DIVISIONS[args.division]

    # ---- device-timed throughput (state resident in HBM)
    sim = Simulation(params)
    sim.set_launch(blocks)
    sim.set_division(division)
    division_used = "exact" if sim.get_division() == _abi.FV_DIVISION_EXACT else "fma"
    sim.init_state()
    stream = torch.cuda.Stream(device=dev)
    sim.set_stream(stream.cuda_stream)
    if args.warmup:
        sim.run(args.warmup)
    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    sampler = ClockSampler(local)
    sampler.start()
    ev0 = torch.cuda.Event(enable_timing=True)
    ev1 = torch.cuda.Event(enable_timing=True)
    ev0.record(stream)
    sim.launch_attempts(args.steps)
    ev1.record(stream)
    stream.synchronize()
    st = sim.sync()
    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    clocks = sampler.stop()
    ms = ev0.elapsed_time(ev1)
    if world > 1:
        ms = max_over_ranks(ms, dev)
    accepted = int(st["accepted"])
    value = replica_throughput(cells, accepted, world, ms)
    per_launch_ms = ms / max(1, accepted + int(st["rejected"]))

    # ---- one step timed alone after an L2 flush, as a cross-check
    flush = torch.empty(2 * L2_BYTES // 4, dtype=torch.float32, device=dev)
    flushed = []
    for _ in range(5):
        with torch.cuda.stream(stream):
            flush.fill_(1.0)
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        sim.launch_attempts(1)
        e1.record(stream)
        stream.synchronize()
        flushed.append(e0.elapsed_time(e1))
    sim.sync()
    del flush
    flushed_ms = statistics.median(flushed)

    # ---- the step kernel alone: attempts launched one at a time with CUDA
    # events on the solver's stream between their launches (the inputs are
    # the 201 MB state, larger than L2)
    step_kernel_ms, attempt_unfused_ms = sim.time_attempts(min(200, max(1, args.steps)))
    sim.close()

    # ---- end to end through the C ABI with pinned host buffers
    sim = Simulation(params)
    sim.set_launch(blocks)
    sim.set_division(division)
    sim.set_stream(stream.cuda_stream)
    u0 = torch.zeros((3, params.ny, params.nx), dtype=torch.float32, pin_memory=True)
    u_out = torch.empty((3, params.ny, params.nx), dtype=torch.float32, pin_memory=True)
    lib = sim.lib
    stats = _abi.FvRunStats()
    e2e_steps = min(args.steps, args.e2e_steps)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    _abi.check(lib.fv_set_state(sim.h, u0[0].data_ptr(), u0[1].data_ptr(), u0[2].data_ptr(), 0), "set_state")
    for _ in range(e2e_steps):
        _abi.check(lib.fv_run(sim.h, 1, C.byref(stats)), "fv_run")
    _abi.check(lib.fv_get_state(sim.h, u_out[0].data_ptr(), u_out[1].data_ptr(), u_out[2].data_ptr(), 0),
               "get_state")
    t1 = time.perf_counter()
    sim.close()
    e2e_s = t1 - t0
    if world > 1:
        e2e_s = max_over_ranks(e2e_s, dev)
    state_bytes = 3 * cells * 4
    ctrl_bytes = C.sizeof(_abi.FvRunStats)
    e2e = {
        "value": replica_throughput(cells, e2e_steps, world, e2e_s * 1e3),
        "unit": "Gcell-updates/s",
        "steps": e2e_steps,
        "h2d_bytes_per_step": state_bytes / e2e_steps,
        "d2h_bytes_per_step": state_bytes / e2e_steps + 88,
        "calls": "fv_set_state(pinned host) + steps x fv_run(1) (sync, stats read back) + fv_get_state(pinned host)",
    }
    del ctrl_bytes

    peak, peak_kind = measured_peak()
    alg_bytes = ALG_BYTES_PER_CELL * cells
    achieved = alg_bytes / (step_kernel_ms * 1e-3) / 1e9
    prof = profiled_figures() or {}
    roofline = {
        "bound": "hbm",
        "achieved": achieved,
        "peak": peak,
        "unit": "GB/s",
        "frac": achieved / peak,
        "peak_source": f"hbm_gbs, {peak_kind} (MEASURED_PEAKS.json); of measured",
        "traffic": prof.get("bytes_per_launch"),
        "kernel": "step_kernel (fused y/x sweeps, CFL, diffusion)",
        "bytes_per_launch": alg_bytes,
        "launch_ms": step_kernel_ms,
        "launch_timing": "step kernel alone, CUDA events between an attempt's launches on the solver's stream",
        "attempt_ms": per_launch_ms,
        "attempt_ms_unfused": attempt_unfused_ms,
        "attempt_ms_l2_flushed": flushed_ms,
        "issue": {"bound": "instruction issue (the bound that applies to this kernel)",
                  "ipc": prof.get("ipc_active"), "ipc_peak": prof.get("ipc_peak"),
                  "issue_slots_busy": prof.get("issue_slots_busy"),
                  "warp_instructions_per_launch": prof.get("warp_instructions_per_launch"),
                  "source": "ncu --set full, profiles/step_kernel_focused_beam_4096x2048.md"},
    }

    line = {
        "metric": "Gcell-updates/s",
        "value": value,
        "unit": "Gcell-updates/s",
        "n_gpus": world,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": ms / max(1, accepted),
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f32",
        "data": "synthetic",
        "config": {
            "workload": "focused-beam 4096x2048 FP32 (plain method, full size)",
            "nx": params.nx, "ny": params.ny, "cells": cells,
            "variant": "exact (no FMA contraction; bit-identical to the oracle)" if exact else "fast (FMA)",
            "cfl_target": params.cflwhish, "accepted": accepted, "rejected": int(st["rejected"]),
            "T_end": st["T"],
            "l2": "inputs larger than L2: each step reads one 100.7 MB state buffer and writes the "
                  "other, 201 MB per step > 129 MB L2; attempt_ms_l2_flushed is one step after "
                  "writing 258 MB",
            "parallelism": "replicas" if world > 1 else "single GPU",
            "ctas_per_launch": blocks,
            "step_division": division_used,
        },
        "roofline": roofline,
        "e2e": e2e,
        # per attempt: ghost-frame pre-pass, step, fix-up, finalize
        "gpu_launches": 4 * (accepted + int(st["rejected"])),
        "clocks": clocks,
    }
    if rank == 0 and not args.no_cpu:
        line["cpu_baseline"] = cpu_sample(params, seconds=args.cpu_seconds, max_steps=50)
    if world > 1:
        torch.distributed.destroy_process_group()
    if rank == 0:
        print(json.dumps(line))
    return 0


def run_batched(args):
    """Config 3: n focused-beam simulations of uneven sizes and physics,
    stepped by the batched launch, against the same simulations run one at a
    time with the plain path. Both legs are device-timed with CUDA events."""
    import torch

    from fivonagi_gb300 import Batch, Simulation, autotune, configs

    rank, world, local = dist_env()
    torch.cuda.set_device(local)
    plist = configs.batched(args.instances, seed=args.seed, exact=0 if args.fast else 1)
    cells = [p.nx * p.ny for p in plist]
    steps = args.steps
    stream = torch.cuda.Stream()

    # ---- batched: one launch per attempt of every simulation
    b = Batch(plist)
    b.set_stream(stream.cuda_stream)
    b.init_state()
    b.run(max(args.warmup, 3))
    torch.cuda.synchronize()
    sampler = ClockSampler(local)
    sampler.start()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    b.launch_attempts(steps)
    e1.record(stream)
    stream.synchronize()
    clocks = sampler.stop()
    st = b.sync()
    ms_batch = e0.elapsed_time(e1)
    acc = [s["accepted"] for s in st]
    b.close()
    batched_rate = sum(c * a for c, a in zip(cells, acc)) / (ms_batch * 1e-3) / 1e9

    # ---- sequential: each simulation alone with the plain path, same steps
    ms_seq = 0.0
    acc_seq = 0
    for p in plist:
        sim = Simulation(p)
        b, m = autotune.tune(p, steps=20)
        sim.set_launch(b)
        sim.set_division(m)
        sim.set_stream(stream.cuda_stream)
        sim.init_state()
        sim.run(max(args.warmup, 3))
        e0.record(stream)
        sim.launch_attempts(steps)
        e1.record(stream)
        stream.synchronize()
        s1 = sim.sync()
        ms_seq += e0.elapsed_time(e1)
        acc_seq += p.nx * p.ny * s1["accepted"]
        sim.close()
    seq_rate = acc_seq / (ms_seq * 1e-3) / 1e9
    line = {
        "metric": "Gcell-updates/s (batched, aggregate)",
        "value": batched_rate,
        "unit": "Gcell-updates/s",
        "n_gpus": 1,
        "steps": steps,
        "warmup": args.warmup,
        "ms_per_step": ms_batch / steps,
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f32",
        "data": "synthetic",
        "config": {"workload": f"{len(plist)} focused-beam simulations, sides from {list(configs.SIDES)}, "
                               f"seed {args.seed}", "cells_per_step": sum(cells),
                   "variant": "fast (FMA)" if args.fast else "exact"},
        "sequential_plain_path": {"value": seq_rate, "unit": "Gcell-updates/s", "ms_total": ms_seq},
        "batched_over_sequential": batched_rate / seq_rate,
        "clocks": clocks,
        # per attempt: ghost-frame pre-pass, batch step, batch fix-up, batch finalize
        "gpu_launches": 4 * steps,
    }
    print(json.dumps(line))
    return 0


def _adjoint_case(p, target, nsteps, seed):
    """Weights and loss window of one design: amplitudes ~ U[0.5, 1.5]
    AMPL and phases ~ U[0, 2 pi) (seeded), a 32x32 window centred on
    `target`, the last 500 steps."""
    import numpy as np

    from fivonagi_gb300.adjoint import loss_window

    rng = np.random.default_rng(seed)
    amp = (rng.uniform(0.5, 1.5, p.array_elems) * p.ampl).astype(np.float32)
    ph = rng.uniform(0.0, 2 * np.pi, p.array_elems).astype(np.float32)
    i, j = target
    win = loss_window(i - 16, j - 16, 32, 32, max(1, nsteps - 499), nsteps)
    return amp, ph, win


def _device_mem_used():
    import torch

    free, total = torch.cuda.mem_get_info()
    return total - free


def _time_design(p, amp, ph, win, nsteps, fd_params=0):
    """Plain forward, recorded forward and backward of one design (wall
    clock around synchronous calls), and optionally a central-difference
    check of a few amplitude gradients on the recorded dt schedule."""
    import numpy as np
    import torch

    from fivonagi_gb300 import Simulation
    from fivonagi_gb300.adjoint import Adjoint

    sim = Simulation(p)
    sim.set_array_weights(amp, ph)
    sim.init_state()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    sim.run(nsteps)
    t_plain = time.perf_counter() - t0
    sim.close()
    mem0 = _device_mem_used()
    adj = Adjoint(p, win, nsteps)
    t0 = time.perf_counter()
    loss = adj.forward(amp, ph)
    t_fwd = time.perf_counter() - t0
    t0 = time.perf_counter()
    ga, gp = adj.backward()
    t_bwd = time.perf_counter() - t0
    mem = _device_mem_used() - mem0
    checks = []
    order = np.argsort(-np.abs(ga))
    for k in order[:fd_params]:
        h = 1e-2 * abs(float(amp[k]))
        a = amp.astype(np.float64).copy()
        a[k] += h
        lp = adj.replay(a.astype(np.float32), ph)
        a[k] -= 2 * h
        lm = adj.replay(a.astype(np.float32), ph)
        hk = (np.float32(amp[k] + h) - np.float32(amp[k] - h)) / 2.0
        fd = (lp - lm) / (2.0 * float(hk))
        checks.append({"param": f"amp[{int(k)}]", "adjoint": float(ga[k]), "central_difference": fd,
                       "rel_diff": abs(float(ga[k]) - fd) / max(abs(fd), 1e-300)})
    adj.close()
    return dict(loss=loss, t_plain=t_plain, t_fwd=t_fwd, t_bwd=t_bwd, mem=mem, ga=ga, gp=gp, checks=checks)


def run_adjoint(args):
    """Config 4: the phased array (1024x1024, 128 elements of 8 cells),
    gradient of the mean u1^2 over a 32x32 window at (700, 512) and steps
    3501-4000 with respect to the 256 element weights, dt schedule frozen."""
    from fivonagi_gb300 import _abi

    p = _abi.default_params("phased-array")
    nsteps = args.adjoint_steps or 4000
    warm = min(200, nsteps)
    _time_design(p, *_adjoint_case(p, (700, 512), warm, args.seed), warm)  # warm-up: first launches
    amp, ph, win = _adjoint_case(p, (700, 512), nsteps, args.seed)
    r = _time_design(p, amp, ph, win, nsteps, fd_params=2)
    cells = p.nx * p.ny
    bytes_bwd = 96.0 * cells * nsteps  # algorithmic bytes per cell-step of the adjoint
    peak, kind = measured_peak()
    achieved = bytes_bwd / r["t_bwd"] / 1e9
    line = {
        "metric": "adjoint/forward time ratio",
        "value": r["t_bwd"] / r["t_plain"],
        "unit": "ratio",
        "n_gpus": 1,
        "steps": nsteps,
        "warmup": warm,
        "higher_is_better": False,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f32",
        "data": "synthetic",
        "config": {"workload": "phased array 1024x1024, 128 elements x (amplitude, phase), loss window 32x32 "
                               f"at (700, 512) over steps {max(1, nsteps - 499)}-{nsteps}, checkpoint every "
                               "ceil(sqrt(N)) steps",
                   "seed": args.seed},
        "forward_plain_s": r["t_plain"],
        "forward_recorded_s": r["t_fwd"],
        "backward_s": r["t_bwd"],
        "gradients_per_s": 1.0 / (r["t_fwd"] + r["t_bwd"]),
        "loss": r["loss"],
        "adjoint_memory_gb": r["mem"] / 1e9,
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                     "frac": achieved / peak, "peak_source": f"hbm_gbs, {kind} (MEASURED_PEAKS.json)",
                     "traffic": None, "kernel": "backward pass (96 B per cell-step)"},
        "gradient_check": r["checks"],
    }
    print(json.dumps(line))
    return 0


def run_designs(args):
    """Config 5: designs of the phased array on 2048x1024 (6000 steps), each
    with its own random weights and a focal target from an 8x8 grid in the
    right half (a seeded permutation).

    The throughput runs `--concurrent` designs at a time from host threads,
    each on its own adjoint handle and non-blocking stream (the library's
    calls release the GIL): the kernels of one design fill the gaps that the
    small per-step launches of another leave. The backward/forward ratio is
    timed on the first designs run alone."""
    from concurrent.futures import ThreadPoolExecutor

    import numpy as np
    import torch

    from fivonagi_gb300 import _abi
    from fivonagi_gb300.adjoint import Adjoint

    base = _abi.default_params("phased-array")
    p = base.replace(nx=2048, ny=1024, xmax=2047 / 24, ymax=1023 / 24, center=512.0)
    nsteps = args.adjoint_steps or 6000
    warm = min(200, nsteps)
    rng = np.random.default_rng(args.seed)
    targets = [(1024 + 128 * (k % 8) + 64, 128 * (k // 8) + 64) for k in rng.permutation(64)]
    cases = [_adjoint_case(p, targets[d], nsteps, args.seed + 1000 + d) for d in range(args.designs)]
    # ---- alone: the backward/forward ratio and a gradient check
    _time_design(p, *_adjoint_case(p, targets[0], warm, args.seed), warm)  # warm-up
    alone = [_time_design(p, *cases[d], nsteps, fd_params=1 if d == 0 else 0)
             for d in range(min(args.designs, args.ratio_designs))]

    # ---- throughput: every design, `concurrent` at a time
    def gradient(d):
        amp, ph, win = cases[d]
        adj = Adjoint(p, win, nsteps)
        try:
            adj.forward(amp, ph)
            return adj.backward()
        finally:
            adj.close()

    conc = max(1, args.concurrent)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    with ThreadPoolExecutor(conc) as ex:
        grads = list(ex.map(gradient, range(args.designs)))
    torch.cuda.synchronize()
    t_all = time.perf_counter() - t0
    # the concurrent runs give the gradients of the runs alone, bit for bit
    same = all(np.array_equal(grads[d][0], alone[d]["ga"]) and np.array_equal(grads[d][1], alone[d]["gp"])
               for d in range(len(alone)))
    line = {
        "metric": "gradients/s",
        "value": args.designs / t_all,
        "unit": "gradients/s",
        "n_gpus": 1,
        "steps": nsteps,
        "warmup": warm,
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f32",
        "data": "synthetic",
        "config": {"workload": f"{args.designs} phased-array designs 2048x1024, {nsteps} steps, 256 weights each, "
                               "32x32 focal windows from an 8x8 grid in the right half", "seed": args.seed,
                   "concurrent_designs": conc},
        "gradients_per_s_alone": len(alone) / sum(r["t_fwd"] + r["t_bwd"] for r in alone),
        "adjoint_forward_ratio_mean": float(np.mean([r["t_bwd"] / r["t_plain"] for r in alone])),
        "ratio_designs": len(alone),
        "concurrent_gradients_equal_alone": bool(same),
        "adjoint_memory_gb_max": max(r["mem"] for r in alone) / 1e9,
        "gradient_check": alone[0]["checks"],
    }
    print(json.dumps(line))
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=4000)
    ap.add_argument("--warmup", type=int, default=100)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--fast", action="store_true", help="FMA-contracted variant instead of exact")
    ap.add_argument("--e2e-steps", type=int, default=1000)
    ap.add_argument("--cpu-seconds", type=float, default=20.0)
    ap.add_argument("--no-cpu", action="store_true", help="leave out the CPU-baseline leg")
    ap.add_argument("--workload", choices=["plain", "batched", "adjoint", "designs"], default="plain",
                    help="plain: focused beam 4096x2048; batched: config-3 batch vs sequential; "
                         "adjoint: config-4 gradient; designs: config-5 gradients")
    ap.add_argument("--instances", type=int, default=64)
    ap.add_argument("--designs", type=int, default=32)
    ap.add_argument("--concurrent", type=int, default=4,
                    help="designs workload: designs run at a time, each on its own stream")
    ap.add_argument("--ratio-designs", type=int, default=4,
                    help="designs workload: designs timed alone for the backward/forward ratio")
    ap.add_argument("--adjoint-steps", type=int, default=0,
                    help="adjoint and designs workloads: steps instead of the configuration's (a small "
                         "case for a profiler's launch list)")
    ap.add_argument("--blocks", type=int, default=0,
                    help="plain workload: CTAs per step launch instead of the autotuner's choice")
    ap.add_argument("--division", choices=["default", "fma", "exact"], default="default",
                    help="plain workload: the step kernel's division instead of the autotuner's (or, with "
                         "--blocks, the library default's) choice")
    ap.add_argument("--seed", type=int, default=0)
    args = ap.parse_args()
    if args.warmup < 3 and args.impl == "ours":
        args.warmup = 3
    if args.impl == "reference":
        return run_reference(args)
    if args.workload == "batched":
        return run_batched(args)
    if args.workload == "adjoint":
        return run_adjoint(args)
    if args.workload == "designs":
        return run_designs(args)
    return run_gpu(args)


if __name__ == "__main__":
    sys.exit(main())
