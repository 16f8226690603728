"""Batched form: many independent plasma instances of uneven size on one GPU.

Every instance is a ``SplitRun`` (split-precision form) with its own CUDA
stream.  ``BatchedRun.make_step(istep)`` issues each instance's step on its
stream, so the kernels of small instances, which fill only part of the GPU
alone, run concurrently; ``graph_step(istep)`` replays all the instances'
steps from one CUDA graph (one launch per step from the host).  Instances share nothing: each result is bitwise
the one the instance gives when advanced alone (the step is deterministic and
has no cross-instance state).

``lwfa_instances(count, seed)`` draws laser-wakefield instances with the
distributions of the batched workload: Nx in 256..2048 (multiples of 128), Nr
in 32..256 (multiples of 32), azimuthal modes 0..1 or 0..2, 2 x 2 x {4, 8}
particles per cell, density log-uniform in 1e-3..1e-2 n_c, a0 in 0.5..3 and
w0 in 8..15 (laser wavelengths); dx = 0.04, dr = 0.4, dt = dx, window moving
at c.  Plasma fills the box behind a 20 wavelength linear ramp.
"""
from __future__ import annotations

from copy import deepcopy

import numpy as np
import torch

from .split import SplitRun


class BatchedRun:
    """Advance several SplitRun instances together, one CUDA stream each."""

    def __init__(self, instances, form: str = "split"):
        if form not in ("split", "fp64"):
            raise ValueError("form is 'split' or 'fp64'")
        self.form = form
        self.runs = []
        for comps in instances:
            if form == "split":
                self.runs.append(SplitRun(comps))
            else:
                from .chimera_main import ChimeraRun
                self.runs.append(ChimeraRun(comps))
        self.streams = [torch.cuda.Stream() for _ in self.runs]
        # construction ran on the current stream; the instance streams start after it
        torch.cuda.current_stream().synchronize()

    def make_step(self, istep: int) -> None:
        for run, s in zip(self.runs, self.streams):
            with torch.cuda.stream(s):
                run.make_step(istep)

    def graph_step(self, istep: int) -> None:
        """make_step with every instance's step in one CUDA graph: the
        instances' device work is captured on their own streams (forked from
        the capture stream and joined back), so one replay per step runs them
        all, concurrently where they fit.  Captured on the second call (the
        first step runs eagerly) and again when an instance's particle arrays
        change; host-side window
        bookkeeping, re-sorts and error-flag reads run outside the graph.
        Falls back to make_step when a step is not capturable
        (SplitRun.graph_capturable)."""
        if self.form != "split" or not all(r.graph_capturable() for r in self.runs):
            return self.make_step(istep)
        if not getattr(self, "_eager_done", False):
            # the first step runs eagerly: the tensor-core products time their
            # column-tile widths on a shape's first launch, which a capture cannot
            self._eager_done = True
            return self.make_step(istep)
        cur = torch.cuda.current_stream()
        for r, s in zip(self.runs, self.streams):
            s.wait_stream(cur)
            with torch.cuda.stream(s):
                r._maybe_sort(istep)
                if not r._scales_valid:
                    r._refresh_scales()
            cur.wait_stream(s)
        key = tuple(r._layout_key(istep) for r in self.runs)
        graphs = getattr(self, "_graphs", None)
        layout = tuple(k[:-1] for k in key)
        if graphs is None or graphs[0] != layout:
            graphs = self._graphs = [layout, {}]  # per gradient-buffer assignment
        self._graph = graphs[1].get(tuple(k[-1] for k in key))
        if self._graph is None:
            from . import _lib
            lib = _lib.load()
            g = torch.cuda.CUDAGraph()
            n0 = lib.chm_launch_count()
            with torch.cuda.graph(g):
                cap = torch.cuda.current_stream()
                for r, s in zip(self.runs, self.streams):
                    s.wait_stream(cap)
                    with torch.cuda.stream(s):
                        r._step_body(istep)
                for s in self.streams:
                    cap.wait_stream(s)
            self.graph_launches = lib.chm_launch_count() - n0  # kernels per replay
            self._graph = graphs[1][tuple(k[-1] for k in key)] = g
            self.graph_captures = getattr(self, "graph_captures", 0) + 1
        else:
            for r in self.runs:
                r._host_effects(istep)
        self._graph.replay()
        for r in self.runs:
            r._after_step()

    def synchronize(self) -> None:
        for s in self.streams:
            s.synchronize()

    @property
    def num_moving(self) -> int:
        """Moving particles over all instances (the metric's particle count)."""
        if self.form == "split":
            return sum(r.num_moving for r in self.runs)
        return sum(sp.num_particles for r in self.runs for sp in r.Particles
                   if "Still" not in sp.Args["Features"])


def lwfa_instance(nx: int, nr: int, max_mode: int, ppc_theta: int, density: float, a0: float,
                  w0: float, seed: int) -> dict:
    """SimComps of one laser-wakefield instance (electrons over still ions)."""
    from .solvers import Solver
    from .species import Specie
    dx, dr = 0.04, 0.4
    xmin = -(nx * dx) + 1.92
    xmax = xmin + nx * dx
    grid = (xmin, xmax, nr * dr, dx, dr)
    ramp = 20.0

    def prof(x):
        return np.interp(x, [xmin, xmin + ramp, 1e9], [0.0, 1.0, 1.0])

    np.random.seed(seed)
    solver = Solver({"Grid": grid, "TimeStep": dx, "MaxAzimuthMode": max_mode,
                     "Features": ("SpaceCharge", "StillAsBackground")})
    fwhm = 10.0
    Lx = fwhm / (2 * np.sqrt(np.log(2) / 2))
    x_las = xmax - 0.25 * (xmax - xmin)
    solver.add_gauss_beam({"a0": a0, "k0": 1.0, "x0": x_las, "x_foc": x_las + 10.0, "Lx": Lx,
                           "LR": w0})
    el_in = {"Grid": grid, "TimeStep": dx, "Density": density, "FixedCell": (2, 2, ppc_theta),
             "Features": ("NoSorting",)}
    io_in = deepcopy(el_in)
    io_in["Charge"], io_in["Mass"], io_in["Features"] = 1.0, 1836.0, ("Still", "NoSorting")
    el, io = Specie(el_in), Specie(io_in)
    parts = el.gen_parts(Domain=(xmin + 1.5 * dx, xmax, 0.0, nr * dr), ProfileFunc=prof)
    el.add_particles(*[p.copy() for p in parts])
    parts[-1] = parts[-1] * -1
    io.add_particles(*parts)
    return {"Solvers": (solver,), "Particles": (el, io),
            "MovingFrames": ({"TimeStep": dx, "Steps": 1, "Velocity": 1.0},)}


def draw_instances(count: int, seed: int) -> list[dict]:
    """Parameters of `count` instances drawn from the batched workload."""
    rng = np.random.default_rng(seed)
    out = []
    for i in range(count):
        out.append({"nx": int(rng.integers(2, 17)) * 128, "nr": int(rng.integers(1, 9)) * 32,
                    "max_mode": int(rng.integers(1, 3)), "ppc_theta": int(rng.choice([4, 8])),
                    "density": float(10 ** rng.uniform(-3, -2)), "a0": float(rng.uniform(0.5, 3.0)),
                    "w0": float(rng.uniform(8.0, 15.0)), "seed": seed * 1000 + i})
    return out


def lwfa_instances(count: int, seed: int = 1005) -> list[dict]:
    """SimComps of `count` instances drawn from the batched workload."""
    return [lwfa_instance(**p) for p in draw_instances(count, seed)]
