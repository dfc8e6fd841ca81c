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
          fv_set_state from pinned host memory, K attempts through
          fv_steps_async / fv_step_wait (each attempt's stats -- accepted,
          dt, T, CFL, status -- read back to the host, the next block of 32
          attempts enqueued before the current block is read), and
          fv_get_state back to pinned host memory, all inside the timed
          region.
  roofline : the step kernel against the measured HBM copy bandwidth, with
          24 algorithmic bytes per cell-update (3 FP32 fields read once and
          written once) over the step kernel's own duration (CUDA events
          between an attempt's launches); `issue` carries the kernel's
          issue-slot figures from the committed ncu summary.
  cpu_baseline : the oracle's CPU restatement (FP32, OpenMP over rows, all
          host cores) on a bounded sample of the same grid.

  error : relative L2 distance per field (u1, u2, u3) after the first
          `--error-steps` steps from rest (500 by default): the exact GPU
          path against the FP32 oracle evaluating the hooks' sin with the
          library's correctly rounded functions (bit-identical: 0), against
          the FP32 oracle with the host libm (the mode pinned to the
          reference's own build), and against the FP64 oracle; the fast
          variant against FP64.
  batched, adjoint, fast : the other parts of the metric on the same run:
          the config-3 batch against its simulations run one at a time
          (`--steps` attempts each), the config-4 gradient cost (recorded
          forward + backward over a plain forward, 4000 steps), and the FMA
          variant at the headline size.
  clocks : SM clock and throttle reasons sampled through NVML every
          millisecond inside the timed region, with the whole run's samples
          beside them.

`--impl reference` times that CPU restatement alone (the reference's GPU
code cannot be built with current toolkits; its arithmetic runs on the host
through the restatement) and prints the same line with "impl": "reference".
It loads none of this library: its parameter block is built in Python
(`headline_params`, checked against the library's defaults by a CPU test).
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

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

ALG_BYTES_PER_CELL = 24  # 3 FP32 fields read + 3 written
L2_BYTES = 129 * 1024 * 1024
PROFILE_TRAFFIC = os.path.join(ROOT, "profiles", "step_kernel_focused_beam_4096x2048.traffic.json")


def headline_params(exact: bool = True):
    """The focused-beam app's parameter block at 4096 x 2048, as
    fv_default_params(FV_APP_FOCUSED_BEAM) gives it, built without loading
    the library (the reference arm runs no product code)."""
    from fivonagi_gb300._abi import FV_APP_FOCUSED_BEAM, FvParams

    p = FvParams()
    p.app = FV_APP_FOCUSED_BEAM
    p.cfl_even_only, p.exact, p.max_retries = 1, 1 if exact else 0, 64
    p.cflmax, p.cflwhish = 1.0, float(np.float32(90 / 100.0))
    p.dtini = float(np.float32(0.005))
    p.nx, p.ny = 4096, 2048
    p.xmax, p.ymax = 4095.0 / 24.0, 2047.0 / 24.0
    p.beta, p.diffdelta, p.ampl, p.frec = 3.5, 5e-5, 5e-3, 1.0
    p.isp_f, p.aperture, p.center, p.ramp_periods, p.tide = 3000.0, 1024.0, 1024.0, 5.0, 0.0
    return p


def headline_config(params) -> dict:
    """The `config` object of both arms' lines (identical keys and values)."""
    return {
        "workload": "focused-beam 4096x2048 FP32 (plain method, full size)",
        "nx": params.nx, "ny": params.ny, "cells": params.nx * params.ny,
        "source": "left edge, aperture 1024 cells centred on j=1024, focus 3000 cells, 24 cells per "
                  "wavelength, Mach 5e-3 over a 5-period ramp",
        "physics": "beta 3.5, dissipation 5e-5, CFL 0.9",
        "start": "medium at rest",
        "l2": "inputs larger than L2: each step reads one 100.7 MB state buffer and writes the other, "
              "201 MB per step > 129 MB L2",
    }


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
    """SM clock, power and throttle reasons of one GPU, read through NVML
    (libnvidia-ml, read-only queries) every millisecond from a thread, so
    that even a few-millisecond timed region gets samples; falls back to
    nvidia-smi every 100 ms where NVML cannot be loaded. `begin()`/`end()`
    bracket the timed region; samples outside it describe the whole run."""

    # nvmlClocksEventReasons bits (NVML's public header)
    REASONS = {0x4: "sw_power_cap", 0x8: "hw_slowdown", 0x20: "sw_thermal_slowdown",
               0x40: "hw_thermal_slowdown", 0x80: "hw_power_brake_slowdown"}
    SMI_FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
                  "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
                  "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device_index: int, uuid: str | None = None, interval_s: float = 0.001):
        self.index = device_index
        self.uuid = uuid
        self.interval = interval_s
        self.samples = []  # (timed, sm_mhz, max_mhz, power_w, reasons bitmask or names)
        self.timed = False
        self.stop_flag = threading.Event()
        self.thread = None
        self.proc = None
        self.source = None

    def _nvml(self):
        import ctypes as C
        lib = C.CDLL("libnvidia-ml.so.1")
        if lib.nvmlInit_v2() != 0:
            raise OSError("nvmlInit failed")
        h = C.c_void_p()
        rc = -1
        if self.uuid:
            u = self.uuid if self.uuid.startswith("GPU-") else "GPU-" + self.uuid
            rc = lib.nvmlDeviceGetHandleByUUID(u.encode(), C.byref(h))
        if rc != 0:
            rc = lib.nvmlDeviceGetHandleByIndex_v2(C.c_uint(self.index), C.byref(h))
        if rc != 0:
            raise OSError("no NVML handle")
        get_reasons = getattr(lib, "nvmlDeviceGetCurrentClocksEventReasons", None) or \
            lib.nvmlDeviceGetCurrentClocksThrottleReasons
        return lib, h, get_reasons

    def _run_nvml(self, lib, h, get_reasons):
        import ctypes as C
        clk, mx, pw, rs = C.c_uint(), C.c_uint(), C.c_uint(), C.c_ulonglong()
        lib.nvmlDeviceGetMaxClockInfo(h, 1, C.byref(mx))  # NVML_CLOCK_SM
        while not self.stop_flag.is_set():
            ok = lib.nvmlDeviceGetClockInfo(h, 1, C.byref(clk)) == 0
            lib.nvmlDeviceGetPowerUsage(h, C.byref(pw))
            get_reasons(h, C.byref(rs))
            if ok:
                self.samples.append((self.timed, float(clk.value), float(mx.value), pw.value / 1000.0,
                                     int(rs.value)))
            time.sleep(self.interval)

    def _run_smi(self):
        for ln in self.proc.stdout:
            parts = [x.strip() for x in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm, smax, pw = float(parts[1]), float(parts[2]), float(parts[3])
            except ValueError:
                continue
            names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
            reasons = {n for n, v in zip(names, parts[5:9]) if v.lower() == "active"}
            self.samples.append((self.timed, sm, smax, pw, reasons))

    def start(self):
        try:
            lib, h, get_reasons = self._nvml()
            self.source = "nvml, 1 ms"
            self.thread = threading.Thread(target=self._run_nvml, args=(lib, h, get_reasons), daemon=True)
        except (OSError, AttributeError):
            try:
                self.proc = subprocess.Popen(
                    ["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.SMI_FIELDS}",
                     "--format=csv,noheader,nounits", "-lms", "100"],
                    stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            except (FileNotFoundError, OSError):
                return
            self.source = "nvidia-smi, 100 ms"
            self.thread = threading.Thread(target=self._run_smi, daemon=True)
        self.thread.start()

    def begin(self):
        self.timed = True

    def end(self):
        self.timed = False

    def _names(self, r) -> set:
        if isinstance(r, set):
            return r
        return {name for bit, name in self.REASONS.items() if r & bit}

    def stop(self) -> dict:
        self.stop_flag.set()
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
        if self.thread is not None:
            self.thread.join(timeout=5)
        if not self.samples:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no clock samples (NVML and nvidia-smi "
                                                                       "unavailable)"], "samples": 0}
        timed = [x for x in self.samples if x[0]]
        # the run's samples under load: power above the idle level of the run
        pmax = max(x[3] for x in self.samples)
        loaded = [x for x in self.samples if x[3] >= 0.5 * pmax]
        use = timed or loaded
        reasons = set()
        for x in use:
            reasons |= self._names(x[4])
        run_reasons = set()
        for x in loaded:
            run_reasons |= self._names(x[4])
        return {
            "sm_mhz": statistics.median(x[1] for x in use),
            "sm_max_mhz": max(x[2] for x in self.samples),
            "power_w_max": pmax,
            "samples": len(timed),
            "reasons": sorted(reasons),
            "window": "timed region" if timed else "whole run under load (no sample inside the timed region)",
            "source": self.source,
            "run": {"samples": len(self.samples), "samples_under_load": len(loaded),
                    "sm_mhz_median_under_load": statistics.median(x[1] for x in loaded) if loaded else None,
                    "reasons": sorted(run_reasons)},
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
    params = headline_params(exact=True)
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
        "config": headline_config(params),
        "runs": "the CPU restatement of the reference's arithmetic on all host cores (the reference's CUDA "
                "does not build on current toolkits)",
        "cpu_baseline": {"kind": res["kind"], "cores": res["cores"], "sample": res["sample"],
                         "value": res["value"], "unit": res["unit"]},
        "e2e": {"value": res["value"], "unit": "Gcell-updates/s", "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line))
    return 0


def rel_l2_fields(a, b) -> list:
    """Relative L2 distance of each field of state a from state b."""
    out = []
    for x, y in zip(a, b):
        x = np.asarray(x, np.float64)
        y = np.asarray(y, np.float64)
        den = float(np.sqrt(np.sum(y * y)))
        num = float(np.sqrt(np.sum((x - y) ** 2)))
        out.append(num / den if den > 0 else num)
    return out


def error_report(params, nsteps: int) -> dict:
    """FP32 GPU error of the headline workload after `nsteps` accepted steps
    from rest, against the FP32 oracle in both of its transcendental modes
    and against the FP64 oracle; the fast (FMA) variant against FP64."""
    from fivonagi_gb300 import Simulation
    from oracle import oracle

    oracle.set_threads(os.cpu_count() or 1)
    gpu = {}
    for name, exact in (("exact", 1), ("fast", 0)):
        sim = Simulation(params.replace(exact=exact))
        sim.init_state()
        sim.run(nsteps)
        gpu[name] = sim.get_state()
        sim.close()
    ref = {}
    for name, dtype, math in (("fvm32", np.float32, "fvm"), ("libm32", np.float32, "libm"),
                              ("libm64", np.float64, "libm")):
        o = oracle.OracleSim(params, dtype, math=math)
        o.init_state()
        o.run(nsteps)
        ref[name] = o.get_state()
        o.close()
    exact_bits = all(np.array_equal(g, r) for g, r in zip(gpu["exact"], ref["fvm32"]))
    return {
        "steps": nsteps,
        "fields": ["u1", "u2", "u3"],
        "metric": "relative L2 per field after the steps, from rest",
        "vs_fp32_oracle": rel_l2_fields(gpu["exact"], ref["fvm32"]),
        "bit_identical_to_fp32_oracle": bool(exact_bits),
        "vs_libm_oracle": rel_l2_fields(gpu["exact"], ref["libm32"]),
        "vs_fp64": rel_l2_fields(gpu["exact"], ref["libm64"]),
        "libm_fp32_oracle_vs_fp64": rel_l2_fields(ref["libm32"], ref["libm64"]),
        "fast_vs_fp64": rel_l2_fields(gpu["fast"], ref["libm64"]),
        "oracles": "fvm32: FP32 restatement with the hooks' sin from the library's correctly rounded "
                   "functions (what the GPU computes); libm32: FP32 with the host libm (the mode pinned "
                   "to the reference's own headers built on the host); libm64: FP64",
    }


def time_plain(params, launch, steps, warmup, stream=None, sampler=None):
    """Device time of `steps` back-to-back attempts of the headline workload
    (CUDA events on the handle's stream) with the launch `launch`."""
    from fivonagi_gb300 import Simulation, autotune

    sim = Simulation(params)
    autotune.set_launch(sim, launch)
    sim.init_state()
    if stream is not None:
        sim.set_stream(stream)
    if warmup:
        sim.run(warmup)
    if sampler is not None:
        sampler.begin()
    ms = sim.time_run(steps)
    if sampler is not None:
        sampler.end()
    st = sim.sync()
    return sim, ms, st


def fast_report(args, cells) -> dict:
    """The FMA-contracted variant at the headline size, autotuned."""
    from fivonagi_gb300 import autotune

    p = headline_params(exact=False)
    launch = autotune.tune(p)
    sim, ms, st = time_plain(p, launch, args.steps, args.warmup)
    sim.close()
    return {"value": cells * st["accepted"] / (ms * 1e-3) / 1e9, "unit": "Gcell-updates/s",
            "ms_per_step": ms / max(1, st["accepted"]), "steps": args.steps,
            "variant": "fast: FMA contraction (not bit-identical; held to FP32 accuracy, see error.fast_vs_fp64)"}


def batched_report(args) -> dict:
    """Config 3: 64 focused-beam simulations of uneven sizes and physics in
    the batched launch, against the same simulations one at a time with the
    plain path (autotuned per grid); `--steps` attempts each."""
    from fivonagi_gb300 import Batch, Simulation, autotune, configs

    plist = configs.batched(args.instances, seed=args.seed, exact=1)
    cells = [p.nx * p.ny for p in plist]
    blocks = autotune.tune_batch(plist)
    b = Batch(plist)
    b.set_launch(blocks)
    b.init_state()
    b.run(max(args.warmup, 3))
    ms_batch = b.time_run(args.steps)
    st = b.sync()
    acc = [x["accepted"] for x in st]
    b.close()
    batched = sum(c * a for c, a in zip(cells, acc)) / (ms_batch * 1e-3) / 1e9
    ms_seq, work_seq = 0.0, 0
    for p in plist:
        launch = autotune.tune(p, steps=20)
        sim = Simulation(p)
        autotune.set_launch(sim, launch)
        sim.init_state()
        sim.run(max(args.warmup, 3))
        ms_seq += sim.time_run(args.steps)
        work_seq += p.nx * p.ny * sim.sync()["accepted"]
        sim.close()
    sequential = work_seq / (ms_seq * 1e-3) / 1e9
    return {"value": batched, "unit": "Gcell-updates/s", "sequential": sequential,
            "ratio": batched / sequential, "ctas": blocks, "instances": len(plist), "cells_per_step": sum(cells),
            "steps": args.steps, "ms_per_attempt": ms_batch / args.steps,
            "workload": f"{len(plist)} focused-beam simulations, sides from {list(configs.SIDES)} drawn "
                        f"independently for x and y, random physics, seed {args.seed}"}


def adjoint_report(args) -> dict:
    """Config 4: the gradient of the windowed loss of the phased array
    (1024x1024, 4000 steps) with respect to its 256 element weights; cost
    of one gradient (recorded forward + backward) over a plain forward."""
    from fivonagi_gb300 import _abi

    p = _abi.default_params("phased-array")
    nsteps = args.adjoint_steps or 4000
    warm = min(200, nsteps)
    _time_design(p, *_adjoint_case(p, (700, 512), warm, args.seed), warm)  # first launches
    amp, ph, win = _adjoint_case(p, (700, 512), nsteps, args.seed)
    r = _time_design(p, amp, ph, win, nsteps)
    return {"forward_s": r["t_plain"], "recorded_forward_s": r["t_fwd"], "backward_s": r["t_bwd"],
            "gradient_over_forward": (r["t_fwd"] + r["t_bwd"]) / r["t_plain"],
            "backward_over_forward": r["t_bwd"] / r["t_plain"], "gradients_per_s": 1.0 / (r["t_fwd"] + r["t_bwd"]),
            "steps": nsteps, "adjoint_memory_gb": r["mem"] / 1e9,
            "workload": "phased array 1024x1024, 128 elements x (amplitude, phase), loss = mean u1^2 over a "
                        f"32x32 window at (700, 512) over the last 500 steps, checkpoint every ceil(sqrt(N)) "
                        f"steps, seed {args.seed}"}


def run_gpu(args):
    import ctypes as C

    import torch

    from fivonagi_gb300 import Simulation, _abi, autotune

    rank, world, local = dist_env()
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", init_method="env://")
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    exact = not args.fast
    params = headline_params(exact)
    cells = params.nx * params.ny
    try:
        uuid = str(torch.cuda.get_device_properties(local).uuid)
    except (AttributeError, RuntimeError):
        uuid = None
    sampler = ClockSampler(local, uuid)
    sampler.start()

    # ---- launch shape and division from the autotuner (cached; outside every
    # timed region), or as given (--blocks/--division: few launches before a
    # profiler's capture)
    DIVISIONS = {"default": _abi.FV_DIVISION_DEFAULT, "fma": _abi.FV_DIVISION_FMA, "exact": _abi.FV_DIVISION_EXACT}
    if args.blocks > 0:
        launch = autotune.Launch(args.blocks, DIVISIONS[args.division], max(args.shape, 0))
    else:
        launch = autotune.tune(params)
        if args.division != "default":
            launch = launch._replace(division=DIVISIONS[args.division])
        if args.shape >= 0:
            launch = launch._replace(shape=args.shape)

    # ---- device-timed throughput (state resident in HBM): K back-to-back
    # attempts between CUDA events on the solver's stream
    stream = torch.cuda.Stream(device=dev)
    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    sim, ms, st = time_plain(params, launch, args.steps, args.warmup, stream.cuda_stream, sampler)
    division_used = "exact" if sim.get_division() == _abi.FV_DIVISION_EXACT else "fma"
    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
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
        flushed.append(sim.time_run(1))
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
    autotune.set_launch(sim, launch)
    sim.set_stream(stream.cuda_stream)
    u0 = torch.zeros((3, params.ny, params.nx), dtype=torch.float32, pin_memory=True)
    u_out = torch.empty((3, params.ny, params.nx), dtype=torch.float32, pin_memory=True)
    lib = sim.lib
    stats = _abi.FvRunStats()
    e2e_steps = min(args.steps, args.e2e_steps)
    # warm-up outside the timed region: the handle's first pipelined
    # attempts allocate its pinned ring and capture its graphs (the timed
    # region then sets the state again)
    for st_ in sim.steps_pipelined(64):
        pass
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    # every attempt's stats come back to the host (fv_step_wait), with the
    # next block of attempts already enqueued (fv_steps_async), so the GPU
    # does not wait for the host's reads
    e2e_accepted = 0
    block = 32
    _abi.check(lib.fv_set_state(sim.h, u0[0].data_ptr(), u0[1].data_ptr(), u0[2].data_ptr(), 0), "set_state")
    queued = min(block, e2e_steps)
    _abi.check(lib.fv_steps_async(sim.h, queued), "fv_steps_async")
    for k in range(e2e_steps):
        if k % block == 0 and queued < e2e_steps:
            m = min(block, e2e_steps - queued)
            _abi.check(lib.fv_steps_async(sim.h, m), "fv_steps_async")
            queued += m
        _abi.check(lib.fv_step_wait(sim.h, C.byref(stats)), "fv_step_wait")
        e2e_accepted += stats.accepted
    _abi.check(lib.fv_get_state(sim.h, u_out[0].data_ptr(), u_out[1].data_ptr(), u_out[2].data_ptr(), 0),
               "get_state")
    t1 = time.perf_counter()
    sim.close()
    e2e_s = t1 - t0
    if world > 1:
        e2e_s = max_over_ranks(e2e_s, dev)
    state_bytes = 3 * cells * 4
    e2e = {
        "value": replica_throughput(cells, e2e_accepted, world, e2e_s * 1e3),
        "unit": "Gcell-updates/s",
        "steps": e2e_steps,
        "accepted": e2e_accepted,
        "h2d_bytes_per_step": state_bytes / e2e_steps,
        "d2h_bytes_per_step": state_bytes / e2e_steps + C.sizeof(_abi.FvRunStats),
        "calls": "fv_set_state(pinned host) + steps attempts through fv_steps_async (blocks of 32, the next "
                 "block enqueued before the current one is read) and fv_step_wait (every attempt's stats read "
                 "back) + fv_get_state(pinned host)",
    }

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
        "traffic_source": "ncu dram__bytes_read.sum + dram__bytes_write.sum of one step-kernel launch in CTA "
                          "shape 4x4 (profiles/step_kernel_focused_beam_4096x2048.md)",
        "kernel": "step_kernel (fused y/x sweeps, CFL, diffusion)",
        "launch": {"cta_shape": _abi.FV_CTA_SHAPES.get(launch.shape, str(launch.shape)), "ctas": launch.blocks,
                   "division": {_abi.FV_DIVISION_EXACT: "exact", _abi.FV_DIVISION_FMA: "fma"}.get(
                       launch.division, "library default (exact)")},
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
                  "thread_instructions_per_cell": prof.get("thread_instructions_per_cell"),
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
        "config": headline_config(params),
        "run": {
            "variant": "exact (no FMA contraction; bit-identical to the oracle)" if exact else "fast (FMA)",
            "accepted": accepted, "rejected": int(st["rejected"]), "T_end": st["T"],
            "parallelism": "replicas" if world > 1 else "single GPU",
            "ctas_per_launch": launch.blocks, "step_division": division_used,
            "cta_shape": _abi.FV_CTA_SHAPES[launch.shape] + " (warps per CTA x CTAs per SM)",
            "attempt_ms_l2_flushed": flushed_ms,
        },
        "roofline": roofline,
        "e2e": e2e,
        # per attempt: ghost-frame pre-pass, step, fix-up, finalize
        "gpu_launches": 4 * (accepted + int(st["rejected"])),
    }
    if rank == 0 and world == 1 and not args.headline_only:
        line["fast"] = fast_report(args, cells)
        line["batched"] = batched_report(args)
        line["adjoint"] = adjoint_report(args)
    line["clocks"] = sampler.stop()
    if rank == 0 and world == 1 and args.error_steps > 0:
        line["error"] = error_report(params, args.error_steps)
        if "fast" in line:
            line["fast"]["err_vs_fp64"] = line["error"]["fast_vs_fp64"]
    if rank == 0 and not args.no_cpu:
        line["cpu_baseline"] = cpu_sample(params, seconds=args.cpu_seconds, max_steps=200)
    if world > 1:
        torch.distributed.destroy_process_group()
    if rank == 0:
        print(json.dumps(line))
    return 0


def run_batched(args):
    """Config 3 alone: n focused-beam simulations of uneven sizes and
    physics, stepped by the batched launch, against the same simulations
    run one at a time with the plain path. Both legs are device-timed with
    CUDA events on their handle's stream."""
    import torch

    from fivonagi_gb300 import configs

    _, _, local = dist_env()
    torch.cuda.set_device(local)
    sampler = ClockSampler(local)
    sampler.start()
    r = batched_report(args)
    clocks = sampler.stop()
    line = {
        "metric": "Gcell-updates/s (batched, aggregate)",
        "value": r["value"],
        "unit": "Gcell-updates/s",
        "n_gpus": 1,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": r["ms_per_attempt"],
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f32",
        "data": "synthetic",
        "config": {"workload": r["workload"], "cells_per_step": r["cells_per_step"],
                   "sides": list(configs.SIDES), "variant": "exact", "ctas": r["ctas"]},
        "sequential_plain_path": {"value": r["sequential"], "unit": "Gcell-updates/s"},
        "batched_over_sequential": r["ratio"],
        "clocks": clocks,
        # per attempt: ghost-frame pre-pass, batch step, batch fix-up, batch finalize
        "gpu_launches": 4 * args.steps,
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


def designs_report(args, batch: int) -> dict:
    """Config 5: designs of the phased array on 2048x1024 (6000 steps),
    each with its own random weights and a focal target from an 8x8 grid in
    the right half (a seeded permutation), `batch` designs per
    fv_adjoint_batch (every forward attempt, replayed step and reverse step
    one launch sequence over the batch). Beside it: the plain forward of one
    design, the gradient cost per design over it, and the designs run one
    handle per design on `--concurrent` streams (the previous method), whose
    gradients must equal the batched ones bit for bit."""
    from concurrent.futures import ThreadPoolExecutor

    import numpy as np
    import torch

    from fivonagi_gb300 import Simulation, _abi
    from fivonagi_gb300.adjoint import Adjoint, AdjointBatch

    base = _abi.default_params("phased-array")
    p = base.replace(nx=2048, ny=1024, xmax=2047 / 24, ymax=1023 / 24, center=512.0)
    nsteps = args.adjoint_steps or 6000
    rng = np.random.default_rng(args.seed)
    targets = [(1024 + 128 * (k % 8) + 64, 128 * (k // 8) + 64) for k in rng.permutation(64)]
    cases = [_adjoint_case(p, targets[d], nsteps, args.seed + 1000 + d) for d in range(args.designs)]
    # plain forward of one design (the cost unit)
    sim = Simulation(p)
    sim.set_array_weights(cases[0][0], cases[0][1])
    sim.init_state()
    sim.run(min(200, nsteps))
    sim.init_state()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    sim.run(nsteps)
    t_plain = time.perf_counter() - t0
    sim.close()
    # batched: every design, `batch` at a time
    mem0 = _device_mem_used()
    t_fwd = t_bwd = 0.0
    grads = [None] * args.designs
    peak = 0
    for b0 in range(0, args.designs, batch):
        ds = list(range(b0, min(args.designs, b0 + batch)))
        ab = AdjointBatch(p, [cases[d][2] for d in ds], nsteps)
        peak = max(peak, _device_mem_used() - mem0)
        amp = np.stack([cases[d][0] for d in ds])
        ph = np.stack([cases[d][1] for d in ds])
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        ab.forward(amp, ph)
        t1 = time.perf_counter()
        ga, gp = ab.backward()
        t2 = time.perf_counter()
        t_fwd += t1 - t0
        t_bwd += t2 - t1
        for k, d in enumerate(ds):
            grads[d] = (ga[k], gp[k])
        ab.close()
    t_batched = t_fwd + t_bwd
    # optionally: smaller batches, several at once, each on its own stream
    # from a host thread (their launch sequences overlap as the single
    # handles' do)
    conc_batched = None
    if args.batch_streams > 1:
        from concurrent.futures import ThreadPoolExecutor as _TPE

        size = max(1, args.stream_batch)
        groups = [list(range(b0, min(args.designs, b0 + size))) for b0 in range(0, args.designs, size)]

        def run_group(ds):
            ab = AdjointBatch(p, [cases[d][2] for d in ds], nsteps)
            try:
                ab.forward(np.stack([cases[d][0] for d in ds]), np.stack([cases[d][1] for d in ds]))
                return ds, ab.backward()
            finally:
                ab.close()

        torch.cuda.synchronize()
        t0 = time.perf_counter()
        with _TPE(args.batch_streams) as ex:
            res = list(ex.map(run_group, groups))
        torch.cuda.synchronize()
        t_cb = time.perf_counter() - t0
        same_cb = all(np.array_equal(ga[k], grads[d][0]) and np.array_equal(gp[k], grads[d][1])
                      for ds, (ga, gp) in res for k, d in enumerate(ds))
        conc_batched = {"value": args.designs / t_cb, "designs_per_batch": size,
                        "concurrent_batches": args.batch_streams, "gradients_equal_batched": bool(same_cb),
                        "method": "fv_adjoint_batch handles of designs_per_batch designs, concurrent_batches at "
                                  "a time, each on its own stream from a host thread (creation included)"}
    # the previous method: one handle per design, `concurrent` streams
    conc = max(1, args.concurrent)
    n_conc = min(args.designs, args.conc_designs)

    def gradient(d):
        amp, ph, win = cases[d]
        adj = Adjoint(p, win, nsteps)
        try:
            adj.forward(amp, ph)
            return adj.backward()
        finally:
            adj.close()

    torch.cuda.synchronize()
    t0 = time.perf_counter()
    with ThreadPoolExecutor(conc) as ex:
        conc_grads = list(ex.map(gradient, range(n_conc)))
    torch.cuda.synchronize()
    t_conc = time.perf_counter() - t0
    same = all(np.array_equal(conc_grads[d][0], grads[d][0]) and np.array_equal(conc_grads[d][1], grads[d][1])
               for d in range(n_conc))
    best = conc_batched["value"] if conc_batched else args.designs / t_batched
    return {
        **_designs_fp64_check(grads, nsteps, args.seed),
        "value": max(best, args.designs / t_batched), "unit": "gradients/s",
        "batched_sequential": {"value": args.designs / t_batched, "designs_per_batch": batch,
                               "method": "fv_adjoint_batch handles of designs_per_batch designs, one after another"},
        "designs": args.designs, "designs_per_batch": batch, "steps": nsteps,
        "forward_plain_s": t_plain,
        "recorded_forward_s_per_design": t_fwd / args.designs,
        "backward_s_per_design": t_bwd / args.designs,
        "gradient_over_forward": t_batched / args.designs / t_plain,
        "adjoint_forward_ratio": t_bwd / args.designs / t_plain,
        "peak_adjoint_memory_gb": peak / 1e9,
        **({"batched_concurrent": conc_batched} if conc_batched else {}),
        "streams": {"value": n_conc / t_conc, "designs": n_conc, "concurrent": conc,
                    "method": "one fv_adjoint per design, each on its own stream from a host thread"},
        "batched_gradients_equal_alone": bool(same),
        "workload": f"phased array 2048x1024, {nsteps} steps, 128 elements x (amplitude, phase), 32x32 focal "
                    f"windows from an 8x8 grid in the right half, seed {args.seed}",
    }


def _designs_fp64_check(grads, nsteps, seed) -> dict:
    """Design 0's batched gradient against FP64 central differences of its
    loss on the same dt schedule (the committed fixture made on the host by
    tests/golden/gen_adjoint_config5.py), on the fixture's weights; only for
    the fixture's case (6000 steps, seed 0)."""
    import numpy as np

    path = os.path.join(os.path.dirname(os.path.abspath(__file__)), "tests", "golden", "adjoint_config5.json")
    if nsteps != 6000 or seed != 0 or grads[0] is None or not os.path.exists(path):
        return {}
    with open(path) as f:
        fx = json.load(f)
    if len(fx.get("fd64", [])) != len(fx.get("directions", [])) or None in fx["fd64"]:
        return {}
    g = np.concatenate(grads[0])[np.asarray(fx["directions"])]
    fd = np.asarray(fx["fd64"])
    rel = np.abs(g - fd) / np.abs(fd)
    return {"gradient_error_vs_fp64": {
        "design": 0, "weights": fx["direction_names"], "rel": [float(x) for x in rel], "max_rel": float(rel.max()),
        "reference": "FP64 central differences (h = 1e-4 relative) of the design's loss on its dt schedule, "
                     "computed on the host by the oracle"}}


def run_designs(args):
    """Config 5 alone (designs_report), as its own JSON line."""
    import torch

    _, _, local = dist_env()
    torch.cuda.set_device(local)
    sampler = ClockSampler(local)
    sampler.start()
    r = designs_report(args, args.designs_per_batch)
    clocks = sampler.stop()
    line = {
        "metric": "gradients/s",
        "value": r["value"],
        "unit": "gradients/s",
        "n_gpus": 1,
        "steps": r["steps"],
        "warmup": 0,
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f32",
        "data": "synthetic",
        "config": {"workload": r["workload"], "designs": r["designs"], "designs_per_batch": r["designs_per_batch"],
                   **({"concurrent_batches": args.batch_streams, "designs_per_concurrent_batch": args.stream_batch}
                      if args.batch_streams > 1 else {})},
        "designs": r,
        "clocks": clocks,
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
    ap.add_argument("--error-steps", type=int, default=500,
                    help="plain workload: steps from rest for the error object (0 leaves it out)")
    ap.add_argument("--headline-only", action="store_true",
                    help="plain workload: leave out the fast, batched and adjoint objects")
    ap.add_argument("--workload", choices=["plain", "batched", "adjoint", "designs"], default="plain",
                    help="plain: focused beam 4096x2048; batched: config-3 batch vs sequential; "
                         "adjoint: config-4 gradient; designs: config-5 gradients")
    ap.add_argument("--instances", type=int, default=64)
    ap.add_argument("--designs", type=int, default=32)
    ap.add_argument("--concurrent", type=int, default=4,
                    help="designs workload: designs run at a time, each on its own stream")
    ap.add_argument("--designs-per-batch", type=int, default=16,
                    help="designs workload: designs per fv_adjoint_batch (about 10 GB each at 2048x1024, 6000 steps)")
    ap.add_argument("--batch-streams", type=int, default=2,
                    help="designs workload: also run batches of --stream-batch designs this many at a time, "
                         "each on its own stream")
    ap.add_argument("--stream-batch", type=int, default=8,
                    help="designs workload: designs per batch for --batch-streams")
    ap.add_argument("--conc-designs", type=int, default=8,
                    help="designs workload: designs run one handle per design on streams, for comparison")
    ap.add_argument("--adjoint-steps", type=int, default=0,
                    help="adjoint and designs workloads: steps instead of the configuration's (a small "
                         "case for a profiler's launch list)")
    ap.add_argument("--blocks", type=int, default=0,
                    help="plain workload: CTAs per step launch instead of the autotuner's choice")
    ap.add_argument("--shape", type=int, default=-1, choices=[-1, *range(6)],
                    help="plain workload: the step kernel's CTA shape (fv_set_cta_shape) instead of the "
                         "autotuner's (or, with --blocks, shape 0)")
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
