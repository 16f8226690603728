"""Benchmark of the CHIMERA PIC step on GB300: particle*steps/s.

Workload (default --size cfg3, the largest configuration that fits one
GPU): the laser-wakefield set-up Nx = 4096 (dx = 0.04), Nr = 512 (dr = 0.4),
azimuthal modes m = 0..2, FixedCell (2, 2, 12) electrons at 0.002 n_c in the
x > 0 half of the box (~50.3M) over still ions (SpaceCharge +
StillAsBackground), Gaussian laser a0 = 3, w0 = 15, FWHM 10 lambda0/c
focused at the plasma entrance, moving window at c
(chimera_gb300/workloads.py; --size cfg2 is the 2048 x 256 x 2-mode set-up).
Inputs are synthetic (seeded numpy) of this shape.

  value  particle*steps/s of the split-precision form (SplitRun.make_step)
         with all state resident on the GPU (moving species only, as the
         metric counts them); --form fp64 makes the plain FP64 form the value
  fp64_gpu  the plain FP64 form (ChimeraRun.make_step) on the same workload
         in the same run, and split_over_fp64 the ratio of the two
  transform_errors  relative L2 of every split transform against the FP64
         kernels on the run's own fields after the timed steps
  e2e    the split form through the public API with the window's plasma
         injection (AddPlasma + AbsorbLayer + IonsOnTop, as in the
         reference's lpa-testrun.py): the generator's host data copied
         host->device every step, and the laser a0 read back every step
  roofline  the dominant stage's algorithmic bytes (or FLOPs) over its live
         CUDA-event time against MEASURED_PEAKS.json
  cpu_baseline  the oracle's C/OpenMP step on all host cores, a bounded
         sample of the e2e workload
  clocks  nvidia-smi SM clock and throttle reasons sampled through the run
  device_flags  the split form's device error flags after the run (a
         tensor-core CTA that gave up on a wait; deposit cells outside their
         block box); the run fails when either is set

--impl reference runs the oracle's CPU step driver (the reference's step
loop over the C restatement of its Fortran kernels, OpenMP on every host
core) on the e2e workload, from the same laser field.
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

from chimera_gb300 import workloads  # noqa: E402

METRIC = "particle*steps/s"
WORKLOAD_SIZE = "cfg3"


def build_run(device_kind, window, seed=1003):
    """ChimeraRun of the workload (GPU) or the oracle's CpuRun inputs."""
    if device_kind == "gpu":
        from chimera_gb300 import ChimeraRun
        comps = workloads.components(WORKLOAD_SIZE, window, seed)
        run = ChimeraRun(comps)
        return run, comps["Solvers"][0], comps["Particles"][0]
    from oracle.step import add_gauss_beam
    comps = workloads.components(WORKLOAD_SIZE, window, seed, device="cpu")
    solver = comps["Solvers"][0]
    add_gauss_beam(solver, workloads.config(WORKLOAD_SIZE)["laser"])
    return solver, comps["Particles"][0], comps["Particles"][1], comps["MovingFrames"][0]


class ClockSampler:
    """nvidia-smi clock / throttle samples (every 100 ms) from the warm-up
    through the timed region."""

    Q = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, index=0):
        self.index = index
        self.rows = []
        self.proc = None
        self.thread = None

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.Q}",
                 "--format=csv,noheader,nounits", "-lms", "100"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except OSError:
            self.proc = None
            return
        self.thread = threading.Thread(target=self._read, daemon=True)
        self.thread.start()

    def _read(self):
        for line in self.proc.stdout:
            parts = [p.strip() for p in line.split(",")]
            if len(parts) >= 7:
                self.rows.append(parts)

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        time.sleep(0.25)
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        if self.thread:
            self.thread.join(timeout=2)
        rows = self.rows
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"]}

        def num(v):
            try:
                return float(v)
            except ValueError:
                return None
        sm = [num(r[0]) for r in rows if num(r[0]) is not None]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in rows for i in range(4) if r[3 + i].lower() == "active"})
        return {"sm_mhz": float(np.median(sm)) if sm else None,
                "sm_max_mhz": num(rows[0][1]), "reasons": reasons, "samples": len(rows)}


def load_peaks():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(path):
        with open(path) as f:
            p = json.load(f)
        return p, "measured"
    return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0, "bf16_tflops_sustained": 1700.0}, "fallback"


# FP64 FMA throughput of this machine's GB300 (measured with a dependent-FMA
# probe: 1.20 TFLOP/s); the plain FP64 form's GEMMs are bound by it.
FP64_PEAK_TFLOPS = 1.20


def umma_tuned(lib):
    """The tensor-core products' tuned column-tile widths: one record
    [M, N, K, batch count, epilogue, width] per product shape."""
    import ctypes
    n = lib.chm_sp_umma_tuned(None, 0)
    buf = (ctypes.c_int32 * (6 * max(n, 1)))()
    lib.chm_sp_umma_tuned(buf, n)
    return [list(buf[6 * i: 6 * i + 6]) for i in range(n)]


def still_count(run, form):
    parts = run.fp.Particles if form == "split" else run.Particles
    return sum(p.num_particles for p in parts if "Still" in p.Args["Features"])


# algorithmic HBM bytes per particle of the particle stages
SPLIT_BYTES = {"push_electrons": 32 + 16,  # read ix,fx,y,z,p,w; write ix,fx,y,z
               "deposit_still": 20,       # read ix,fx,y,z,w
               "gather_push": 32 + 12}    # read ix,fx,y,z,p,w; write p
FP64_BYTES = {"push_velocs": 48 + 48 + 24, "push_coords": 24 + 24 + 24 + 24,
              "dep_curr": 24 + 24 + 8, "dep_dens": 24 + 8, "proj_fld": 24 + 8 + 48 + 48}
# DRAM bytes (read + write) per particle of the dominant split-form stage,
# by the number of stored modes, from one ncu capture of a quarter-radius
# case (traffic grows with the particle count): 2 modes from --size prof
# (4.13M particles per species: electrons (push + J + rho) 179.9 MB, still
# ions (rho) 87.3 MB); 3 modes from --size prof3 (12.49M per species:
# electrons 637.8 MB, still ions 273.1 MB)
SPLIT_TRAFFIC = {2: {"push_electrons": 179.90e6 / 4128768, "deposit_still": 87.29e6 / 4128768},
                 3: {"push_electrons": 637.78e6 / 12490704, "deposit_still": 273.07e6 / 12490704}}
GEMM_STAGES = ("chm_fb_graddiv", "chm_fb_rot", "chm_fb_grad", "chm_fb_div", "chm_fb_in",
               "chm_fb_out", "chm_fb_eb_out", "chm_sp_poisson", "chm_sp_poisson_psatd",
               "chm_sp_fb_in_acc",
               "chm_sp_fb_eb_out", "chm_sp_rot_b", "chm_sp_fb_grad")


def stage_roofline(form, prof, nprof, n_e, n_i, peaks, peak_kind):
    """Roofline of the dominant stage: algorithmic work over its live
    CUDA-event time, against the measured peak of its bound."""
    hbm = float(peaks.get("hbm_gbs", 6800.0))
    bf16 = float(peaks.get("bf16_tflops", 1900.0))
    rows = []
    for name, (calls, ms, flops) in prof.items():
        t = ms / nprof / 1e3  # seconds per step
        if t <= 0:
            continue
        if name in GEMM_STAGES and flops > 0:
            alg = flops / nprof / t / 1e12
            if form == "split":
                rows.append({"stage": name, "bound": "tensor", "achieved": alg, "unit": "TFLOP/s",
                             "peak": bf16, "frac": alg / bf16, "executed_tflops": 6 * alg,
                             "executed_frac": 6 * alg / bf16, "ms_per_step": t * 1e3})
            else:
                rows.append({"stage": name, "bound": "fp64", "achieved": alg, "unit": "TFLOP/s",
                             "peak": FP64_PEAK_TFLOPS, "frac": alg / FP64_PEAK_TFLOPS,
                             "ms_per_step": t * 1e3})
            continue
        nb = None
        bg_apart = "chm_sp_deposit_background" in prof  # (the still species' own pass)
        if name == "chm_sp_push_deposit":
            nb = n_e * SPLIT_BYTES["push_electrons"] + \
                (0 if bg_apart else n_i * SPLIT_BYTES["deposit_still"])
        elif name == "chm_sp_deposit_background":
            # a whole-cell window move: the int64 {re, im} grid read and
            # written once (the entering column's few ions aside)
            W = workloads.SIZES[WORKLOAD_SIZE]
            nb = 2 * 16 * W.nx * (W.nkr + 1) * W.modes
        elif name == "chm_sp_gather_push":
            nb = n_e * SPLIT_BYTES["gather_push"]
        elif name in ("chm_push_velocs", "chm_push_coords", "chm_proj_fld"):
            nb = n_e * FP64_BYTES[name[4:]]
        elif name == "chm_dep_curr_chnk":
            nb = n_e * FP64_BYTES["dep_curr"]
        elif name == "chm_dep_dens_chnk":
            nb = (2 * n_e + n_i) * FP64_BYTES["dep_dens"]
        if nb is not None:
            ach = nb / t / 1e9
            rows.append({"stage": name, "bound": "hbm", "achieved": ach, "unit": "GB/s",
                         "peak": hbm, "frac": ach / hbm, "ms_per_step": t * 1e3,
                         "algorithmic_bytes_per_step": nb})
    rows.sort(key=lambda r: -r["ms_per_step"])
    top = dict(rows[0]) if rows else {"stage": None}
    top["kernel"] = top.pop("stage")
    top["traffic"] = None
    tr = SPLIT_TRAFFIC.get(workloads.SIZES[WORKLOAD_SIZE].modes)
    if form == "split" and top.get("kernel") == "chm_sp_push_deposit" and tr:
        top["traffic"] = n_e * tr["push_electrons"] + \
            (0 if "chm_sp_deposit_background" in prof else n_i * tr["deposit_still"])
        top["traffic_source"] = ("ncu dram__bytes_read.sum + dram__bytes_write.sum of the "
                                 "quarter-radius case, scaled by particle count")
    top["peak_source"] = f"MEASURED_PEAKS.json ({peak_kind})" if top.get("bound") != "fp64" else \
        "FP64 FMA probe on this pool (1.20 TFLOP/s)"
    if top.get("bound") == "tensor":
        top["note"] = ("achieved counts the algorithmic 2 M N K flops of the FP32-accurate "
                       "products; the split-BF16 form executes 6 times that on the tensor "
                       "cores (executed_frac), and the stage includes its FP32 combines and "
                       "splits; the particle kernels' rows are in stages")
    top["stages"] = rows
    return top


def dist_setup(backend=None):
    """One process per GPU (torchrun env): replicas, so the process group
    only carries the barrier and the max-over-ranks timing (NCCL on GPUs,
    gloo without one)."""
    import torch
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if torch.cuda.is_available():
        torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group(backend or ("nccl" if torch.cuda.is_available() else "gloo"))
    return world, rank, local


def barrier(world):
    if world > 1:
        import torch.distributed as dist
        dist.barrier()


def max_over_ranks(world, v):
    if world == 1:
        return v
    import torch
    import torch.distributed as dist
    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([v], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def cpu_step_time(nsteps, warmup=0, window="none"):
    """Wall time per step and moving particles per step of the oracle's CPU
    step driver on this workload (from the same laser field as the GPU arm)."""
    from oracle.step import CpuRun, CpuSpecies
    solver, el, io, wind = build_run("cpu", window)
    run = CpuRun(solver, [CpuSpecies(el), CpuSpecies(io)], wind)
    for i in range(1, warmup + 1):
        run.make_step(i)
    psteps = 0
    t0 = time.perf_counter()
    for i in range(warmup + 1, warmup + nsteps + 1):
        run.make_step(i)
        psteps += run.Particles[0].n()
    dt = (time.perf_counter() - t0) / nsteps
    return dt, psteps / nsteps


def workload_name(window="none"):
    return workloads.SIZES[WORKLOAD_SIZE].name + ("_window_inject" if window == "inject" else "")


def run_reference(args):
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return 0
    cores = len(os.sched_getaffinity(0))
    os.environ.setdefault("OMP_NUM_THREADS", str(cores))
    # one warm-up step: the CPU step has no lazy initialisation after the first
    warm = min(args.warmup, 1)
    steps = args.steps
    clamp = None
    if args.ref_max_steps is not None and steps > args.ref_max_steps:
        steps = args.ref_max_steps
        clamp = f"steps clamped from {args.steps} to {steps} (--ref-max-steps)"
    t_step, n = cpu_step_time(steps, warm, window="inject")
    value = n / t_step
    W = workloads.SIZES[WORKLOAD_SIZE]
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": METRIC, "n_gpus": world,
        "steps": steps, "warmup": warm, "ms_per_step": 1e3 * t_step, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": workload_name("inject"), "particles": n, "cpu_threads": cores,
                   "nx": W.nx, "nr": W.nkr + 1, "modes": W.modes,
                   "window": "AbsorbLayer=64, AddPlasma, IonsOnTop, moving at c (the e2e "
                             "workload of the gb300 arm), from the same laser field",
                   "warmup_note": f"warm-up {warm} of {args.warmup}: the CPU step has no lazy "
                                  "initialisation after its first step",
                   "steps_note": clamp},
        "cpu_baseline": {"value": value, "unit": METRIC, "cores": cores, "kind": "port",
                         "sample": f"{steps} full steps of the workload (after {warm} warm-up) "
                                   "with the oracle's C/OpenMP restatement of the reference "
                                   "kernels and its step loop (oracle/step.py)"},
        "e2e": {"value": value, "unit": METRIC, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)
    return 0


def time_steps(run, first, count, nmov, stream, stepper=None):
    """CUDA-event time (ms) of `count` steps from step `first` (make_step, or
    `stepper`), and the moving particles summed over them."""
    import torch
    stepper = stepper or run.make_step
    ev0 = torch.cuda.Event(enable_timing=True)
    ev1 = torch.cuda.Event(enable_timing=True)
    ev0.record(stream)
    psteps = 0
    for i in range(first, first + count):
        stepper(i)
        psteps += nmov()
    ev1.record(stream)
    torch.cuda.synchronize()
    return ev0.elapsed_time(ev1), psteps


def run_gb300(args):
    import torch

    from chimera_gb300 import _lib, fimera
    from chimera_gb300.split import SplitRun, transform_errors

    world, rank, local = dist_setup()
    lib = _lib.load()
    W = workloads.SIZES[WORKLOAD_SIZE]
    stream = torch.cuda.current_stream()
    fp, solver, el = build_run("gpu", "none", seed=1003 + rank)
    # the clock sampler starts before the warm-up (its start-up stays out of
    # the timed region) and samples through warm-up and timed steps
    clocks = ClockSampler(local)
    clocks.start()
    step = 0
    # the plain FP64 form on the same workload: its own warm-up and steps
    fp64 = None
    if args.fp64_steps > 0 or args.form == "fp64":
        nsteps = args.steps if args.form == "fp64" else args.fp64_steps
        nwarm = args.warmup if args.form == "fp64" else 1
        for _ in range(nwarm):
            step += 1
            fp.make_step(step)
        torch.cuda.synchronize()
        barrier(world)
        ms64, ps64 = time_steps(fp, step + 1, nsteps, lambda: el.num_particles, stream)
        step += nsteps
        ms64 = max_over_ranks(world, ms64)
        fp64 = {"value": world * ps64 / (ms64 / 1e3), "unit": METRIC, "steps": nsteps,
                "warmup": nwarm, "ms_per_step": ms64 / nsteps, "dtype": "f64",
                "what": "ChimeraRun.make_step (the plain FP64 form: FP64 particles, complex128 "
                        "fields, FP64 products) on the same workload, device resident"}
    if args.form == "split":
        # the split form continues from the FP64 run's state; its re-sort by
        # deposit cell runs at the cadence the run-time tuner picks
        run = SplitRun(None, fp64_run=fp)
        nmov = lambda: run.num_moving  # noqa: E731
    else:
        run = fp
        nmov = lambda: el.num_particles  # noqa: E731
    n_moving = nmov()
    if args.form == "split":
        # each step's kernels replay from a CUDA graph (SplitRun.graph_step)
        stepper = run.graph_step
        for _ in range(args.warmup):
            step += 1
            stepper(step)
        torch.cuda.synchronize()
        # L2: the particle state (1.6 GB per species in the split form at
        # cfg3) is far larger than the 129 MB L2, so every step streams from HBM
        barrier(world)
        torch.cuda.synchronize()
        launches0 = lib.chm_launch_count()
        flops0 = lib.chm_gemm_flops()
        t0 = time.perf_counter()
        replays0 = getattr(run, "graph_replays", 0)
        ms, psteps = time_steps(run, step + 1, args.steps, nmov, stream, stepper)
        wall = time.perf_counter() - t0
        step += args.steps
        # kernels launched by the library, plus those replayed in graphs
        launches = lib.chm_launch_count() - launches0 + \
            (getattr(run, "graph_replays", 0) - replays0) * getattr(run, "graph_launches", 0)
        gemm_flops = lib.chm_gemm_flops() - flops0
        ms_max = max_over_ranks(world, ms)
        value = world * psteps / (ms_max / 1e3)
    else:
        ms_max = fp64["ms_per_step"] * fp64["steps"]
        value = fp64["value"]
        wall, launches, gemm_flops = None, None, 0.0
    barrier(world)
    clk = clocks.stop()

    # device error flags of the split form (must be clear)
    flags = {"umma_status": int(lib.chm_sp_umma_status()),
             "deposit_cells_dropped": int(lib.chm_sp_deposit_dropped())}
    # split transforms against the FP64 kernels on this run's own fields
    terr = None
    if args.form == "split" and not args.no_errors:
        terr = transform_errors(run)

    # stage profile of a few more steps (events around every C-ABI call)
    _lib.profile_begin()
    nprof = max(2, min(3, args.steps))
    for i in range(step + 1, step + nprof + 1):
        run.make_step(i)
    step += nprof
    prof = _lib.profile_end()
    tot = sum(v[1] for v in prof.values())
    stages = {k.replace("chm_", ""): {"calls": c / nprof, "ms_per_step": t / nprof,
                                      "share": t / tot if tot else None,
                                      "gemm_gflop_per_step": f / nprof / 1e9}
              for k, (c, t, f) in sorted(prof.items(), key=lambda kv: -kv[1][1])}
    # long-run decay: the same run continued to step decay_steps; the last
    # 20 steps timed against the first window (re-sorts included)
    decay = None
    if args.form == "split" and args.decay_steps > step + 20:
        run.sort_every = "auto"
        first = (args.warmup + 1 + (args.fp64_steps + 1 if args.fp64_steps > 0 else 0))
        while step < args.decay_steps - 20:
            step += 1
            run.make_step(step)
        torch.cuda.synchronize()
        ms_late, _ = time_steps(run, step + 1, 20, nmov, stream)
        step += 20
        decay = {"early_steps": [first, first + args.steps - 1],
                 "early_ms_per_step": ms_max / args.steps,
                 "late_steps": [step - 19, step], "late_ms_per_step": ms_late / 20,
                 "late_over_early": (ms_late / 20) / (ms_max / args.steps),
                 "sort": {"mode": "auto (SortCadence)",
                          "history": [{"step": h[0], "cadence": h[1], "sort_ms": h[2],
                                       "slope_ms_per_step": h[3]} for h in run.sorter.history]}}
        run.check_status()
    peaks, peak_kind = load_peaks()
    roofline = stage_roofline(args.form, prof, nprof, n_moving, still_count(run, args.form),
                              peaks, peak_kind)
    roofline["algorithmic_gemm_gflop_per_step"] = gemm_flops / max(1, args.steps) / 1e9
    del run, fp, solver, el
    torch.cuda.empty_cache()

    # end to end through the public API with per-step host I/O
    e2e = None
    if not args.no_e2e:
        run2, solver2, el2 = build_run("gpu", "inject", seed=2003 + rank)
        eb2 = lambda: solver2.Data["EB"]  # noqa: E731
        cnt2 = lambda: el2.num_particles  # noqa: E731
        if args.form == "split":
            run2 = SplitRun(None, fp64_run=run2)
            eb2 = lambda: run2.EB  # noqa: E731
            cnt2 = lambda: run2.num_moving  # noqa: E731
        # warm-up runs the same per-step work as the timed loop (the first
        # use of a kernel can load or compile its module)
        a0 = 0.0
        for i in range(1, args.warmup + 1):
            run2.make_step(i)
            cnt2()
            a0 = float(eb2()[:, 1, 0, 2].real.max().item())
        torch.cuda.synchronize()
        h0, d0 = fimera.io_bytes["h2d"], fimera.io_bytes["d2h"]
        live0 = run2.live_particle_steps() if args.form == "split" else 0
        barrier(world)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        ps2 = 0
        # the laser amplitude diagnostic of the demos (max Re Ey on axis) is
        # read back every step: reduced on the device, copied to pinned host
        # memory asynchronously and read by the host one step later, so the
        # host prepares the next step (plasma generation) while the GPU runs
        slots = [torch.empty((), dtype=torch.float32 if args.form == "split" else torch.float64,
                             pin_memory=True) for _ in range(2)]
        done = [torch.cuda.Event(), torch.cuda.Event()]
        a0s = []
        for n, i in enumerate(range(args.warmup + 1, args.warmup + args.steps + 1)):
            run2.make_step(i)
            ps2 += cnt2()
            slots[n % 2].copy_(eb2()[:, 1, 0, 2].real.max(), non_blocking=True)
            done[n % 2].record()
            if n >= 1:
                done[(n - 1) % 2].synchronize()
                a0s.append(float(slots[(n - 1) % 2]))
        done[(args.steps - 1) % 2].synchronize()
        a0s.append(float(slots[(args.steps - 1) % 2]))
        a0 = a0s[-1]
        if args.form == "split":
            # live particles after each step, summed on the device (absorbed
            # particles wait in place, weight zero, until a compaction)
            ps2 = run2.live_particle_steps() - live0
        torch.cuda.synchronize()
        t_e2e = max_over_ranks(world, time.perf_counter() - t0)
        h2d = (fimera.io_bytes["h2d"] - h0) / args.steps
        d2h = (fimera.io_bytes["d2h"] - d0) / args.steps + slots[0].element_size()
        if args.form == "split":
            d2h += 8 / args.steps  # the live-count read
            run2.check_status()
        e2e = {"value": world * ps2 / t_e2e, "unit": METRIC, "h2d_bytes_per_step": h2d,
               "d2h_bytes_per_step": d2h, "laser_a0_last": a0, "workload": workload_name("inject"),
               "what": "make_step with AddPlasma+AbsorbLayer window (the injected plasma's "
                       "host data copied H2D each step: random numbers and pattern tables in "
                       "the split form, the generated particles in the FP64 form) and a "
                       "laser-a0 read back each step (asynchronous copy to pinned memory, "
                       "consumed one step later)"}
        del run2, solver2, el2
        torch.cuda.empty_cache()

    fel = fel_leg(args, world) if (args.fel_steps > 0 and args.form == "split") else None

    cpu = None
    if rank == 0 and not args.no_cpu:
        cores = len(os.sched_getaffinity(0))
        os.environ.setdefault("OMP_NUM_THREADS", str(cores))
        t_cpu, n_cpu = cpu_step_time(args.cpu_steps, 0, window="inject")
        cpu = {"value": n_cpu / t_cpu, "unit": METRIC, "cores": cores, "kind": "port",
               "sample": f"{args.cpu_steps} full step(s) of the e2e workload (window with "
                         "injection and absorption, from the same laser field) with the "
                         "oracle's C/OpenMP restatement of the reference kernels and step loop"}

    split = args.form == "split"
    line = {
        "metric": METRIC, "value": value, "unit": METRIC, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms_max / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None,
        "dtype": "f32 (bf16x3 split tensor-core GEMMs)" if split else "f64",
        "data": "synthetic",
        "config": {"workload": workload_name(), "form": args.form, "particles_moving": n_moving,
                   "particles_still": n_moving, "nx": W.nx, "nr": W.nkr + 1, "modes": W.modes,
                   "ppc": list(W.ppc),
                   "parallelism": f"replicas{world}" if world > 1 else "single",
                   "l2": "inputs larger than L2 (particle state %.2f GB per species)"
                         % (n_moving * (32 if split else 80) / 1e9),
                   "step": "kernels replayed from a CUDA graph per step (SplitRun.graph_step)"
                           if split else "ChimeraRun.make_step"},
        "wall_s_timed": wall,
        "gpu_launches": launches,
        "fp64_gpu": fp64,
        "split_over_fp64": (value / fp64["value"]) if (split and fp64) else None,
        "max_transform_err": max(terr.values()) if terr else None,
        "transform_errors": terr,
        "device_flags": flags,
        "decay": decay,
        "tuning": {"umma_cols": umma_tuned(lib) if split else None,
                   "umma_cols_fields": "M, N, K, batch count, epilogue, column-tile width "
                                       "(timed on each shape's first launch)",
                   "sort": "every 64 steps in the timed steps; SortCadence picks it in the "
                           "decay run" if split else None},
        "roofline": roofline,
        "stages": stages,
        "clocks": clk,
        "e2e": e2e,
        "fel": fel,
        "cpu_baseline": cpu,
        "peaks": {"source": peak_kind, "hbm_gbs": peaks.get("hbm_gbs"),
                  "bf16_tflops": peaks.get("bf16_tflops")},
    }
    if rank == 0:
        print(json.dumps(line), flush=True)
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()
    if flags["umma_status"] or flags["deposit_cells_dropped"]:
        print(f"device error flags set: {flags}", file=sys.stderr)
        return 1
    return 0


def fel_leg(args, world=1):
    """The FEL workload (envelope solver, analytic undulator, Staged window;
    2048 x 128 x 3 envelope modes, 8.4M beam particles): the plain FP64 form
    and the split form (steps replayed from CUDA graphs) on the same run,
    particle*steps/s of each from CUDA events on the launch stream."""
    import torch

    from chimera_gb300 import ChimeraRun
    from chimera_gb300.split import SplitRun
    stream = torch.cuda.current_stream()
    fp = ChimeraRun(workloads.fel_components("fel4", seed=1004))
    beam = fp.Particles[0]
    step = 0
    for _ in range(1):
        step += 1
        fp.make_step(step)
    torch.cuda.synchronize()
    n64 = max(1, args.fel_fp64_steps)
    ms64, ps64 = time_steps(fp, step + 1, n64, lambda: beam.num_particles, stream)
    step += n64
    run = SplitRun(None, fp64_run=fp)
    for _ in range(3):
        step += 1
        run.graph_step(step)
    torch.cuda.synchronize()
    ms, ps = time_steps(run, step + 1, args.fel_steps, lambda: run.num_moving, stream,
                        run.graph_step)
    run.check_status()
    W = workloads.FEL["fel4"]
    out = {"workload": W.name, "particles": beam.num_particles, "nx": W.nx,
           "nr": int(run.nr), "nkr": int(run.nkr), "modes": int(run.nm),
           "split": {"value": world * ps / (ms / 1e3), "unit": METRIC, "steps": args.fel_steps,
                     "warmup": 3, "ms_per_step": ms / args.fel_steps},
           "fp64_gpu": {"value": world * ps64 / (ms64 / 1e3), "unit": METRIC, "steps": n64,
                        "warmup": 1, "ms_per_step": ms64 / n64},
           "accuracy": "radiated energy within 1 % of the FP64 form over 2400 steps "
                       "(tests/test_split_env_gpu.py, the 256 x 32 case)"}
    out["split_over_fp64"] = out["split"]["value"] / out["fp64_gpu"]["value"]
    del run, fp, beam
    torch.cuda.empty_cache()
    return out


def run_batched(args):
    """Batched workload: `args.batched` laser-wakefield instances of uneven
    size (chimera_gb300.batched.draw_instances, seed 1005) advanced together,
    one CUDA stream each, in the split form; against the same instances
    advanced one by one in the plain FP64 form."""
    import torch

    from chimera_gb300 import _lib
    from chimera_gb300.batched import BatchedRun, draw_instances, lwfa_instance
    from chimera_gb300.messages import msg
    msg.quiet = True
    lib = _lib.load()
    params = draw_instances(args.batched, 1005)
    batch = BatchedRun([lwfa_instance(**p) for p in params])
    for i in range(1, args.warmup + 1):
        batch.graph_step(i)
    batch.synchronize()
    torch.cuda.synchronize()
    launches0 = lib.chm_launch_count()
    captures0 = getattr(batch, "graph_captures", 0)
    t0 = time.perf_counter()
    psteps = 0
    for i in range(args.warmup + 1, args.warmup + args.steps + 1):
        batch.graph_step(i)
        psteps += batch.num_moving
    batch.synchronize()
    torch.cuda.synchronize()
    wall = time.perf_counter() - t0
    # kernels: those launched (captures), plus the replays' graph kernels
    launches = lib.chm_launch_count() - launches0 + args.steps * getattr(batch, "graph_launches", 0)
    value = psteps / wall
    # the same instances one by one in the plain FP64 form (their FP64 runs,
    # two steps each after one warm-up step)
    t_fp = 0.0
    n_fp = 0
    for run in batch.runs:
        fp = run.fp
        fp.make_step(args.warmup + args.steps + 1)
        torch.cuda.synchronize()
        t1 = time.perf_counter()
        for i in range(args.warmup + args.steps + 2, args.warmup + args.steps + 4):
            fp.make_step(i)
        torch.cuda.synchronize()
        t_fp += (time.perf_counter() - t1) / 2
        n_fp += sum(sp.num_particles for sp in fp.Particles if "Still" not in sp.Args["Features"])
    fp_value = n_fp / t_fp
    line = {
        "metric": METRIC, "value": value, "unit": METRIC, "n_gpus": 1, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": 1e3 * wall / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32 (bf16x3 split tensor-core GEMMs)",
        "data": "synthetic",
        "config": {"workload": f"batched_lwfa_{args.batched}", "instances": len(params),
                   "particles_moving": psteps // args.steps,
                   "nx": sorted({p["nx"] for p in params}), "nr": sorted({p["nr"] for p in params}),
                   "modes": sorted({p["max_mode"] + 1 for p in params}),
                   "streams": len(batch.streams), "timing": "host wall clock, all streams synced",
                   "step": "every instance's kernels in one CUDA graph per step (BatchedRun.graph_step)",
                   "graph_kernels_per_step": getattr(batch, "graph_launches", None),
                   "graph_captures_timed": getattr(batch, "graph_captures", 0) - captures0},
        "gpu_launches": launches,
        "fp64_one_by_one": {"value": fp_value, "unit": METRIC,
                            "what": "each instance's plain FP64 step alone, summed over instances"},
        "batched_over_fp64": value / fp_value,
        "tuning": {"umma_cols": umma_tuned(_lib.load()),
                   "umma_cols_fields": "M, N, K, batch count, epilogue, column-tile width"},
    }
    print(json.dumps(line), flush=True)
    return 0


def run_spectral(args):
    """The split form's spectral stages alone on the workload's grid (random
    complex64 fields, no particles), each timed with CUDA events: the case
    the tensor-core product kernel is profiled on.  --spectral-stages picks
    the stages (poisson, eb_out, fb_in, rot_b)."""
    import ctypes as C

    import torch

    from chimera_gb300 import _lib
    from chimera_gb300 import fimera as fm
    from chimera_gb300 import split
    from chimera_gb300.messages import msg
    from chimera_gb300.solvers import Solver
    msg.quiet = True
    S = Solver(dict(workloads.config(WORKLOAD_SIZE)["solver"]))
    A = S.Args
    nx, nr, nkr, nm = A["Nx"], A["Nr"], A["Nkr"], A["Mtot"]
    dev = torch.device("cuda")
    o = {k: split._prepare_ops(A[key], dev) for k, key in
         (("InCurr", "InCurr"), ("Out", "Out"), ("Dp", "DpS2S"), ("Dm", "DmS2S"))}
    ws = torch.empty(_lib.query("chm_sp_fb_ws_bytes", nx, nr, nkr, nm), dtype=torch.uint8,
                     device=dev)
    st = torch.cuda.current_stream().cuda_stream
    kx64 = S.dev["kx"]
    kx32 = kx64.to(torch.float32)
    pf32 = torch.from_numpy(np.asfortranarray(A["PoissFact"].astype(np.float32))).cuda()
    depf = torch.from_numpy(np.asfortranarray(A["DepFact"].astype(np.float32))).cuda()
    gen = torch.Generator(device=dev)
    gen.manual_seed(7)

    def rnd(shape):
        t = fm.fortran_zeros(shape, torch.complex64)
        t.real.normal_(generator=gen)
        t.imag.normal_(generator=gen)
        return t
    J, gp, gn = rnd((nx, nkr, nm, 3)), rnd((nx, nkr, nm, 3)), rnd((nx, nkr, nm, 3))
    EG, Bf = rnd((nx, nkr, nm, 6)), rnd((nx, nkr, nm, 3))
    G = EG[:, :, :, 3:]
    EB = fm.fortran_zeros((nx, nr, nm, 6), torch.complex64)
    acc = torch.randint(-2 ** 40, 2 ** 40, (nx * nr * nm * 3 * 2,), dtype=torch.int64, device=dev,
                        generator=gen)
    sc = torch.tensor([2.0 ** 40, 1.0], dtype=torch.float64, device=dev)
    lib = _lib.load()
    P = lambda name: C.addressof(o[name][0])  # noqa: E731
    stages = {
        "poisson": lambda: _lib.call("chm_sp_poisson", J.data_ptr(), gp.data_ptr(), gn.data_ptr(),
                                     pf32.data_ptr(), 10.0, P("Dp"), P("Dm"), kx32.data_ptr(), nx,
                                     nkr, nm, 3, 1, ws.data_ptr(), ws.numel(), st),
        "eb_out": lambda: _lib.call("chm_sp_fb_eb_out", EB.data_ptr(), EG.data_ptr(), Bf.data_ptr(),
                                    1.0, kx64.data_ptr(), P("Out"), nx, nr, nkr, nm, ws.data_ptr(),
                                    ws.numel(), st, None),
        "fb_in": lambda: _lib.call("chm_sp_fb_in_acc", J.data_ptr(), acc.data_ptr(), sc.data_ptr(),
                                   None, None, 1.0, kx64.data_ptr(), P("InCurr"), depf.data_ptr(), nx,
                                   nr, nkr, nm, 3, ws.data_ptr(), ws.numel(), st, None),
        "rot_b": lambda: _lib.call("chm_sp_rot_b", Bf.data_ptr(), G.data_ptr(), pf32.data_ptr(),
                                   P("Dp"), P("Dm"), kx32.data_ptr(), nx, nkr, nm, ws.data_ptr(),
                                   ws.numel(), st),
    }
    peaks, peak_kind = load_peaks()
    out = {}
    for name in args.spectral_stages.split(","):
        f = stages[name]
        f()
        torch.cuda.synchronize()
        f0 = lib.chm_gemm_flops()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        for _ in range(args.steps):
            f()
        e1.record()
        torch.cuda.synchronize()
        ms = e0.elapsed_time(e1) / args.steps
        fl = (lib.chm_gemm_flops() - f0) / args.steps
        out[name] = {"ms": ms, "algorithmic_tflops": fl / ms / 1e9,
                     "executed_tflops": 6 * fl / ms / 1e9,
                     "executed_frac": 6 * fl / ms / 1e9 / float(peaks.get("bf16_tflops", 1900.0))}
    print(json.dumps({"spectral_stages": out, "workload": workloads.SIZES[WORKLOAD_SIZE].name,
                      "umma_status": int(lib.chm_sp_umma_status()), "peaks": peak_kind}))
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--cpu-steps", type=int, default=1)
    ap.add_argument("--ref-max-steps", type=int, default=None,
                    help="reference arm: at most this many timed steps (recorded in the line)")
    ap.add_argument("--fp64-steps", type=int, default=2,
                    help="timed steps of the plain FP64 form in the same run (0: skip)")
    ap.add_argument("--decay-steps", type=int, default=500,
                    help="continue the timed split run to this step and time its last 20 steps")
    ap.add_argument("--fel-steps", type=int, default=20,
                    help="timed split steps of the FEL leg (0: skip)")
    ap.add_argument("--fel-fp64-steps", type=int, default=3,
                    help="timed FP64 steps of the FEL leg")
    ap.add_argument("--umma-cols", type=int, default=-1,
                    help="tensor-core product column-tile width: -1 tuned per shape (default), "
                         "0 the default width, > 0 forced (for profiler runs, whose serialised "
                         "launches would mislead the tuner)")
    ap.add_argument("--fel", action="store_true",
                    help="run the FEL leg alone (its own JSON line; profiling case)")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-errors", action="store_true")
    ap.add_argument("--form", default="split", choices=["fp64", "split"],
                    help="fp64 = plain FP64 form; split = split-precision form")
    ap.add_argument("--batched", type=int, default=0,
                    help="run the batched workload with this many instances instead")
    ap.add_argument("--spectral", action="store_true",
                    help="time the split form's spectral stages alone on the grid (profiling)")
    ap.add_argument("--spectral-stages", default="poisson,eb_out,fb_in,rot_b")
    ap.add_argument("--size", default="cfg3", choices=sorted(workloads.SIZES),
                    help="cfg3 = the benchmark workload; cfg2, cfg1 the smaller configurations; "
                         "prof3, prof, spec, small = reduced cases for profiling")
    args = ap.parse_args()
    if args.umma_cols != -1:
        from chimera_gb300 import _lib
        _lib.load().chm_sp_set_umma_cols(args.umma_cols)
    global WORKLOAD_SIZE
    WORKLOAD_SIZE = args.size
    if args.warmup < 3 and args.impl == "gb300":
        args.warmup = 3
    if args.impl == "reference":
        return run_reference(args)
    if args.batched:
        return run_batched(args)
    if args.spectral:
        return run_spectral(args)
    if args.fel:
        out = fel_leg(args)
        print(json.dumps({"metric": METRIC, "value": out["split"]["value"], "unit": METRIC,
                          "n_gpus": 1, "steps": args.fel_steps, "warmup": 3,
                          "ms_per_step": out["split"]["ms_per_step"], "higher_is_better": True,
                          "dtype": "f32 (bf16x3 split tensor-core GEMMs)", "data": "synthetic",
                          "config": {"workload": out["workload"]}, "fel": out}), flush=True)
        return 0
    return run_gb300(args)


if __name__ == "__main__":
    sys.exit(main())
