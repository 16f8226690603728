"""Laser-wakefield workloads of the benchmark and the long-run tests.

Synthetic, seeded inputs of the configurations' shapes stand in for the
runs (the reference publishes no benchmark dataset).  Every workload is the
reference's plain LWFA set-up (doc/tests/lpa-testrun.py:30-58): one solver
with SpaceCharge + StillAsBackground, FixedCell electrons over still ions
with the same positions, a Gaussian laser added in spectral space
(solvers.py:555-610), dx = 0.04, dr = 0.4 (laser wavelengths), dt = dx and a
window moving at c.

  lwfa_4096x512_m3   Nx = 4096, Nr = 512, modes 0..2, ppc 2 x 2 x 12, density
                     0.002 n_c for x > 0 (half the box, ~50.3M electrons),
                     a0 = 3, w0 = 15, FWHM duration 10 / c, focused at the
                     plasma entrance x = 0
  lwfa_2048x256_m2   Nx = 2048, Nr = 256, modes 0..1, ppc 2 x 2 x 8, density
                     0.003 n_c behind a 20-wavelength linear up-ramp filling
                     the box (~16.8M electrons), a0 = 2, w0 = 12
  lwfa_512x64_m2     Nx = 512, Nr = 64, modes 0..1, ppc 2 x 2 x 4, density
                     0.002 n_c filling the box (~0.5M electrons), a0 = 1,
                     w0 = 10, focused at x = 0
Reduced cases for profiling: the 4096 x 512 set-up at a quarter of the
radius (Nr = 128, 12.6M electrons), the 2048 x 256 set-up at a quarter of
the radius, and its grid with one particle per cell.

``window="inject"`` adds the demos' plasma injection: AbsorbLayer = 64 cells
(AddPlasma with the workload's profile, IonsOnTop)."""
from __future__ import annotations

from copy import deepcopy
from dataclasses import dataclass, replace

import numpy as np


@dataclass(frozen=True)
class Workload:
    name: str
    nx: int
    nkr: int
    max_mode: int            # stored modes 0 .. max_mode
    ppc: tuple               # FixedCell (x, r, theta)
    density: float           # n_c
    a0: float
    w0: float                # laser waist (wavelengths)
    xmin: float              # left edge of the box
    plasma_x0: float         # plasma starts here (profile 0 before)
    ramp: float              # linear up-ramp length after plasma_x0
    laser_x0: float          # laser centre
    laser_xfoc: float        # focus
    fwhm: float = 10.0       # duration (wavelengths / c)
    dx: float = 0.04
    dr: float = 0.4

    @property
    def xmax(self):
        return self.xmin + self.nx * self.dx

    @property
    def modes(self):
        return self.max_mode + 1

    def profile(self, x):
        x = np.asarray(x, dtype=float)
        if self.ramp > 0:
            return np.interp(x, [self.plasma_x0, self.plasma_x0 + self.ramp, 1e9], [0.0, 1.0, 1.0])
        return (x >= self.plasma_x0).astype(float)


_CFG3 = Workload("lwfa_4096x512_m3", nx=4096, nkr=512, max_mode=2, ppc=(2, 2, 12), density=0.002,
                 a0=3.0, w0=15.0, xmin=-81.92, plasma_x0=0.0, ramp=0.0, laser_x0=-35.0,
                 laser_xfoc=0.0)
_CFG2 = Workload("lwfa_2048x256_m2", nx=2048, nkr=256, max_mode=1, ppc=(2, 2, 8), density=0.003,
                 a0=2.0, w0=12.0, xmin=-80.0, plasma_x0=-80.0, ramp=20.0, laser_x0=-30.0,
                 laser_xfoc=-10.0)
_CFG1 = Workload("lwfa_512x64_m2", nx=512, nkr=64, max_mode=1, ppc=(2, 2, 4), density=0.002,
                 a0=1.0, w0=10.0, xmin=-18.56, plasma_x0=-18.56, ramp=0.0, laser_x0=-8.0,
                 laser_xfoc=0.0)

SIZES = {
    "cfg3": _CFG3,
    "cfg2": _CFG2,
    "cfg1": _CFG1,
    # quarter radius of the 4096 x 512 set-up: 12.6M electrons (0.4 GB of
    # split-form particle state per species, above the 129 MB L2), a few GB
    # on the device, for ncu captures
    "prof3": replace(_CFG3, name="lwfa_4096x128_m3", nkr=128),
    "prof": replace(_CFG2, name="lwfa_2048x64_m2", nkr=64),
    # the 2048 x 256 grid with one particle per cell, for captures of the
    # spectral kernels at their full size
    "spec": replace(_CFG2, name="lwfa_2048x256_m2_ppc1", ppc=(1, 1, 1)),
    "small": replace(_CFG1, name="lwfa_512x64_m2_small"),
}


def config(size: str, nchunks: int = 16) -> dict:
    """Solver / laser / species dicts of a workload (the reference's keys)."""
    W = SIZES[size]
    grid = (W.xmin, W.xmax, W.nkr * W.dr, W.dx, W.dr)
    Lx = W.fwhm / (2 * np.sqrt(np.log(2) / 2))
    return dict(
        W=W,
        solver={"Grid": grid, "TimeStep": W.dx, "MaxAzimuthMode": W.max_mode,
                "Xchunked": (nchunks, 10), "Features": ("SpaceCharge", "StillAsBackground")},
        laser={"a0": W.a0, "k0": 1.0, "x0": W.laser_x0, "x_foc": W.laser_xfoc, "Lx": Lx,
               "LR": W.w0},
        electrons={"Grid": grid, "TimeStep": W.dx, "Density": W.density, "FixedCell": W.ppc,
                   "Xchunked": (nchunks, 10), "Features": ("NoSorting",)},
        # the generator's domain: the plasma part of the box (Xgrid starts at
        # xmin + dx)
        domain=(max(W.xmin + 1.5 * W.dx, W.plasma_x0), W.xmax, 0.0, W.nkr * W.dr),
        profile=W.profile)


def window(size: str, kind: str = "none") -> dict:
    W = SIZES[size]
    wind = {"TimeStep": W.dx, "Steps": 1, "Velocity": 1.0}
    if kind == "inject":
        wind.update({"AbsorbLayer": 64, "AddPlasma": W.profile, "Features": ("IonsOnTop",)})
    return wind


def components(size: str, kind: str = "none", seed: int = 1003, device=None) -> dict:
    """SimComps (Solvers, Particles, MovingFrames) of a workload: the solver
    with its laser and the electrons and still ions, built on `device`
    (torch CUDA by default)."""
    from .messages import msg
    from .solvers import Solver
    from .species import Specie
    msg.quiet = True
    cfg = config(size)
    np.random.seed(seed)
    kw = {} if device is None else {"device": device}
    solver = Solver(deepcopy(cfg["solver"]), **kw)
    if device in (None, "cuda"):
        solver.add_gauss_beam(cfg["laser"])
    el_in = deepcopy(cfg["electrons"])
    io_in = deepcopy(cfg["electrons"])
    io_in["Charge"], io_in["Mass"], io_in["Features"] = 1.0, 1836.0, ("Still", "NoSorting")
    el, io = Specie(el_in, **kw), Specie(io_in, **kw)
    parts = el.gen_parts(Domain=cfg["domain"], ProfileFunc=cfg["profile"])
    el.add_particles(*parts)
    parts[-1] = parts[-1] * -1
    io.add_particles(*parts)
    return {"Solvers": (solver,), "Particles": (el, io), "MovingFrames": (window(size, kind),)}


# ----------------------------------------------------------------------
# Free-electron-laser workloads: the reference's FEL set-up
# (doc/tests/fel-testrun.py): envelope solver (KxShift at the resonant
# wavenumber, CoPropagative at the beam velocity, NoPoissonCorrection), a
# relativistic beam in a planar analytic undulator (undul_analytic, the
# period as the length unit), a seed laser at the resonance and a Staged
# window moving with the beam.  Lengths follow fel-testrun.py (box 200 um,
# radius 1 mm cut at 0.7 mm, beam 80 um, undulator period 2.8 cm); the
# beam energy and undulator strength, grid and particle count are the
# workload's.
@dataclass(frozen=True)
class FelWorkload:
    name: str
    nx: int
    nr: int
    max_mode: int      # stored modes -max_mode .. max_mode
    rand_cell: int     # particles per cell (RandCell)
    gamma: float
    K0: float
    periods: float     # undulator length in periods
    dt: float = 1.0 / 30
    a0_seed: float = 0.15


FEL = {
    # 2048 x 128 grid, modes -1..1, ~8.4M beam particles
    "fel4": FelWorkload("fel_2048x128_m3", nx=2048, nr=128, max_mode=1, rand_cell=80,
                        gamma=200.0, K0=1.0, periods=80.0),
    # the same set-up on a 256 x 32 grid (the long-run test's case)
    "fel_small": FelWorkload("fel_256x32_m3", nx=256, nr=32, max_mode=1, rand_cell=16,
                             gamma=200.0, K0=1.0, periods=80.0),
}


def fel_components(size: str, seed: int = 1004, device=None) -> dict:
    """SimComps of an FEL workload (solver with its seed laser, the beam with
    its undulator, the Staged window)."""
    from . import fimera
    from .messages import msg
    from .solvers import Solver
    from .species import Specie
    msg.quiet = True
    W = FEL[size]
    lam0 = 2.8  # undulator period (cm), the length unit
    g0 = W.gamma
    gg = g0 / (1.0 + W.K0 ** 2 / 2) ** 0.5
    k_res = 2 * gg ** 2
    vb = (1.0 - gg ** -2) ** 0.5
    Lgx, Rg, Rcut = 200e-4 / lam0, 1000e-4 / lam0, 700e-4 / lam0
    lbx = lbr = 80e-4 / lam0
    dens = 20e-12 / 1.6022e-19 / (np.pi * 80e-4 ** 3) / (1.1e21 / 2.8e4 ** 2)
    np.random.seed(seed)
    kw = {} if device is None else {"device": device}
    solver = Solver({"Grid": (-0.5 * Lgx, 0.5 * Lgx, Rg, Lgx / W.nx, Rg / W.nr),
                     "TimeStep": W.dt, "MaxAzimuthMode": W.max_mode, "KxShift": k_res,
                     "Rcut": Rcut, "CoPropagative": vb,
                     "Features": {"NoPoissonCorrection": True}}, **kw)
    if device in (None, "cuda"):
        solver.add_gauss_beam({"a0": W.a0_seed, "k0": k_res, "x0": -30e-4 / lam0,
                               "x_foc": 70.0 / lam0, "Lx": 15e-4 / lam0, "LR": 180e-4 / lam0})
    beam = Specie({"Grid": (-0.5 * Lgx, 0.5 * Lgx, Rg, Lgx / W.nx, lbr / W.nr),
                   "TimeStep": W.dt, "Charge": -1.0, "Mass": 1.0, "Density": dens,
                   "RandCell": W.rand_cell, "MomentaMeans": (g0, 0.0, 0.0),
                   "MomentaSpreads": (1e-4 * g0, 2e-5 * g0, 2e-5 * g0),
                   "Devices": ([fimera.undul_analytic, np.array([W.K0, 1.0, 1.0, W.periods])],)},
                  **kw)
    beam.add_particles(*beam.gen_parts(Domain=(-0.5 * lbx, 0.5 * lbx, 0.0, lbr)))
    wind = {"TimeStep": W.dt, "Steps": 1, "Velocity": vb, "Features": ("Staged", "NoSorting")}
    return {"Solvers": (solver,), "Particles": (beam,), "MovingFrames": (wind,)}
