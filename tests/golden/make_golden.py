"""Generate the golden fixtures in tests/golden/ from the reference itself.

Run where a checkout of the reference is available, naming it:

    python tests/golden/make_golden.py <path-to-reference-checkout>

(or set CHIMERA_REFERENCE to that path).

The reference's own Python layer (moduls/solvers.py, species.py,
chimera_main.py) is imported unmodified as the package ``chimera``.  Its
Fortran extension cannot be built without gfortran/FFTW, so the oracle
(oracle/oracle.py, a C restatement of f90/*.f90) stands in for
``chimera.moduls.fimera``.  Three import shims make the Python 2/3-era code
load on Python 3.12 (they change no arithmetic): ``inspect.getargspec``
(species.py:21), ``np.int`` (solvers.py:678) and an empty ``h5py``
(chimera_main.py:21, used only by the checkpoint routines).

What the fixtures pin:
  - the FP64 operator build (DHT matrices, DpS2S/DmS2S, PSATD coefficients,
    DepFact, PoissFact, EnergyFact, damp profile): pure reference Python;
  - particle generation (gen_parts + genparts) with a seeded numpy RNG;
  - laser initialisation (add_gauss_beam) and short full PIC runs
    (ChimeraRun.make_step): the reference's step logic over oracle kernels.
"""
from __future__ import annotations

import inspect
import os
import sys
import tempfile
import types
from copy import deepcopy

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
REF = os.environ.get("CHIMERA_REFERENCE")
if len(sys.argv) > 1:
    REF = sys.argv[1]


def import_reference():
    sys.path.insert(0, ROOT)
    from oracle import oracle as orc  # noqa: E402

    if not hasattr(inspect, "getargspec"):
        inspect.getargspec = inspect.getfullargspec
    if not hasattr(np, "int"):
        np.int = int
    sys.modules.setdefault("h5py", types.ModuleType("h5py"))
    pkgroot = tempfile.mkdtemp(prefix="chimera_ref_")
    os.symlink(REF, os.path.join(pkgroot, "chimera"))
    sys.path.insert(0, pkgroot)
    import chimera  # noqa: F401
    import chimera.moduls  # noqa: F401
    sys.modules["chimera.moduls.fimera"] = orc
    chimera.moduls.fimera = orc
    from chimera.moduls.solvers import Solver
    from chimera.moduls.species import Specie
    from chimera.moduls.chimera_main import ChimeraRun
    return Solver, Specie, ChimeraRun, orc


OPERATOR_KEYS = ["Nx", "Nkr", "Nr", "Mtot", "leftX", "rightX", "lengthR", "dkx", "kx0",
                 "Xgrid", "Rgrid", "RgridFull", "kx", "kx_env", "kr", "kr_g", "kx_g", "w",
                 "In", "Out", "InCurr", "OutFull", "InFull", "DpS2S", "DmS2S", "PoissFact",
                 "DepFact", "VGrid", "EnergyFact", "idxM", "upperR", "lowerR"]


def solver_configs():
    return {
        "lpa_m2": {"Grid": (-6.0, 0.4, 4.0, 0.1, 0.25), "TimeStep": 0.1, "MaxAzimuthMode": 1,
                   "Features": ("SpaceCharge", "StillAsBackground")},
        "lpa_m3_chunked": {"Grid": (-5.0, 1.0, 3.0, 0.1, 0.3), "TimeStep": 0.1,
                           "MaxAzimuthMode": 2, "Xchunked": (4, 3),
                           "Features": ("SpaceCharge",)},
        "plain_m1_vacuum": {"Grid": (-3.0, 3.0, 3.0, 0.1, 0.2), "TimeStep": 0.1,
                            "MaxAzimuthMode": 0},
        "fel_env_k1": {"Grid": (-2.0, 2.0, 6.0, 4.0 / 64, 6.0 / 24), "TimeStep": 1.0 / 30,
                       "MaxAzimuthMode": 1, "KxShift": 20.0, "Rcut": 4.5,
                       "CoPropagative": 0.999, "Features": {"NoPoissonCorrection": True}},
    }


def dump_solver(prefix, s, out):
    for k in OPERATOR_KEYS:
        if k in s.Args:
            out[f"{prefix}/Args/{k}"] = np.asarray(s.Args[k])
    for k in ("PSATD_E", "PSATD_G"):
        out[f"{prefix}/Data/{k}"] = np.asarray(s.Data[k])


def lpa_run(Solver, Specie, ChimeraRun, nsteps, window):
    np.random.seed(1001)
    dx, dr = 0.1, 0.25
    solver_in = {"Grid": (-6.0, 0.4, 4.0, dx, dr), "TimeStep": dx, "MaxAzimuthMode": 1,
                 "Features": ("SpaceCharge", "StillAsBackground")}
    solver = Solver(solver_in)
    solver.add_gauss_beam({"a0": 1.0, "k0": 1.0, "x0": -2.5, "x_foc": 2.0, "Lx": 1.5, "LR": 2.5})
    EG0 = solver.Data["EG_fb"].copy()
    el_in = {"Grid": (-6.0, 0.4, 4.0, dx, dr), "TimeStep": dx, "Density": 0.02,
             "FixedCell": (2, 2, 2), "Features": ()}
    io_in = deepcopy(el_in)
    io_in["Charge"] = 1.0
    io_in["Mass"] = 1836.0
    io_in["Features"] = ("Still",)
    electrons, ions = Specie(el_in), Specie(io_in)
    prof = lambda x: np.interp(x, [-4.0, -3.0, 10.0], [0.0, 1.0, 1.0])  # noqa: E731
    parts = electrons.gen_parts(Domain=(-5.5, 0.3, 0.0, 3.5), ProfileFunc=prof)
    electrons.add_particles(*[p.copy() for p in parts])
    parts[-1] *= -1
    ions.add_particles(*parts)
    comps = {"Solvers": (solver,), "Particles": (electrons, ions)}
    if window:
        comps["MovingFrames"] = ({"TimeStep": dx, "Steps": 2, "AbsorbLayer": 8,
                                  "AddPlasma": prof, "Features": ("IonsOnTop",)},)
    else:
        # window moving at c, one cell per step, no absorption / injection
        comps["MovingFrames"] = ({"TimeStep": dx, "Steps": 1, "Velocity": 1.0},)
    init = {k: v.copy() for k, v in electrons.Data.items()}
    run = ChimeraRun(comps)
    for i in range(1, nsteps + 1):
        run.make_step(i)
    return solver, electrons, ions, EG0, init


def fel_run(Solver, Specie, ChimeraRun, orc, nsteps):
    np.random.seed(1004)
    K0, periods = 1.0, 4.0
    g0 = 20.0
    gg = g0 / (1. + K0 ** 2 / 2) ** .5
    k_res = 2 * gg ** 2
    vb = (1. - gg ** -2) ** 0.5
    Lgx, Rg, Nx, Nr = 0.6, 3.0, 64, 24
    dt = 1. / 30
    solver_in = {"Grid": (-0.5 * Lgx, 0.5 * Lgx, Rg, Lgx / Nx, Rg / Nr), "TimeStep": dt,
                 "MaxAzimuthMode": 1, "KxShift": k_res, "Rcut": 0.8 * Rg, "CoPropagative": vb,
                 "Features": {"NoPoissonCorrection": True}}
    solver = Solver(solver_in)
    solver.add_gauss_beam({"a0": 0.05, "k0": k_res, "x0": -0.05, "x_foc": 1.0, "Lx": 0.08,
                           "LR": 1.2})
    beam_in = {"Grid": (-0.5 * Lgx, 0.5 * Lgx, Rg, Lgx / Nx, 0.4 / Nr), "TimeStep": dt,
               "Charge": -1., "Mass": 1., "Density": 1e-4, "RandCell": 4,
               "MomentaMeans": (g0, 0., 0.), "MomentaSpreads": (1e-3 * g0, 1e-3, 1e-3),
               "Devices": ([orc.undul_analytic, np.array([K0, 1., 1., periods])],)}
    beam = Specie(beam_in)
    beam.add_particles(*beam.gen_parts(Domain=(-0.1, 0.1, 0.0, 0.4)))
    init = {k: v.copy() for k, v in beam.Data.items()}
    run = ChimeraRun({"Solvers": (solver,), "Particles": (beam,),
                      "MovingFrames": ({"TimeStep": dt, "Steps": 1, "Velocity": vb,
                                        "Features": ("Staged", "NoSorting")},)})
    for i in range(1, nsteps + 1):
        run.make_step(i)
    return solver, beam, init


def static_run(Solver, Specie, ChimeraRun, nsteps):
    """A beam-only space-charge run with the StaticKick solver, shaped as the
    reference's space-charge demo (Staged co-moving frame, Xchunked)."""
    np.random.seed(1006)
    size = 1.0
    xmin, xmax, lrg, nx, nr = -7.0 * size, 7.0 * size, 12.0 * size, 56, 24
    dx, dr, dt = (xmax - xmin) / nx, lrg / nr, 1.0
    solver = Solver({"Grid": (xmin, xmax, lrg, dx, dr), "TimeStep": dt, "MaxAzimuthMode": 1,
                     "Features": ("StaticKick",), "Xchunked": (4, 6)})
    beam = Specie({"Grid": (xmin, xmax, lrg, dx, dr), "TimeStep": dt, "Charge": -1., "Mass": 1.,
                   "Density": 1e-3, "FixedCell": (2, 2, 4), "MomentaMeans": (50.0, 0., 0.),
                   "Xchunked": (4, 6)})
    fu = lambda x, y, z: np.exp(-0.5 * (x ** 2 + y ** 2 + z ** 2) / size ** 2)  # noqa: E731
    beam.add_particles(*beam.gen_parts(Domain=(-3.5 * size, 3.5 * size, 0.0, 3.5 * size),
                                       ProfileFunc=fu))
    init = {k: v.copy() for k, v in beam.Data.items()}
    run = ChimeraRun({"Solvers": (solver,), "Particles": (beam,),
                      "MovingFrames": ({"TimeStep": dt, "Steps": 1,
                                        "Features": ("NoSorting", "Staged")},)})
    for i in range(nsteps):
        run.make_step(i)
    return solver, beam, init


def main():
    Solver, Specie, ChimeraRun, orc = import_reference()
    out = {}
    # 1) operator builds
    for name, cfg in solver_configs().items():
        s = Solver(deepcopy(cfg))
        dump_solver(f"op/{name}", s, out)
        if name == "lpa_m2":
            out["op/lpa_m2/damp_profile"] = s.get_damp_profile(12)
    # 2) particle generation
    np.random.seed(7)
    sp = Specie({"Grid": (-2.0, 1.0, 2.0, 0.1, 0.25), "TimeStep": 0.1, "Density": 0.01,
                 "FixedCell": (2, 2, 3), "MomentaSpreads": (0.1, 0.05, 0.05)})
    c, p, w = sp.gen_parts(Domain=(-1.5, 0.8, 0.0, 1.5),
                           ProfileFunc=lambda x, r: np.exp(-r ** 2) * (1 + 0.1 * x))
    out["gen/fixed/coords"], out["gen/fixed/momenta"], out["gen/fixed/weights"] = c, p, w
    c, p, w = sp.gen_parts(Xsteps=3)
    out["gen/xsteps/coords"], out["gen/xsteps/momenta"], out["gen/xsteps/weights"] = c, p, w
    # 3) LPA runs (laser + plasma, SpaceCharge, Still ions)
    for tag, nsteps, window in (("lpa", 6, False), ("lpa_window", 6, True)):
        solver, el, io, EG0, init = lpa_run(Solver, Specie, ChimeraRun, nsteps, window)
        out[f"{tag}/EG_fb_init"] = EG0
        for k in ("coords", "momenta", "weights"):
            out[f"{tag}/init/{k}"] = init[k]
        out[f"{tag}/nsteps"] = np.array(nsteps)
        for k in ("EG_fb", "J_fb", "Rho_fb", "EB", "BckGrndRho"):
            out[f"{tag}/solver/{k}"] = solver.Data[k]
        for k in ("coords", "coords_halfstep", "momenta", "weights", "EB"):
            out[f"{tag}/electrons/{k}"] = el.Data[k]
        out[f"{tag}/ions/coords"] = io.Data["coords"]
        out[f"{tag}/leftX"] = np.array(solver.Args["leftX"])
    # 4) FEL run (envelope solver, undulator device, staged co-moving frame)
    solver, beam, init = fel_run(Solver, Specie, ChimeraRun, orc, 5)
    for k in ("coords", "momenta", "weights"):
        out[f"fel/init/{k}"] = init[k]
    out["fel/EG_fb_init_skip"] = np.array(0)
    for k in ("EG_fb", "J_fb", "EB"):
        out[f"fel/solver/{k}"] = solver.Data[k]
    for k in ("coords", "momenta", "EB"):
        out[f"fel/beam/{k}"] = beam.Data[k]
    out["fel/leftX"] = np.array(solver.Args["leftX"])
    # 5) beam-only StaticKick run (space-charge demo shape)
    solver, beam, init = static_run(Solver, Specie, ChimeraRun, 4)
    for k in ("coords", "momenta", "weights"):
        out[f"static/init/{k}"] = init[k]
    for k in ("EG_fb", "J_fb", "EB"):
        out[f"static/solver/{k}"] = solver.Data[k]
    for k in ("coords", "coords_halfstep", "momenta"):
        out[f"static/beam/{k}"] = beam.Data[k]
    out["static/leftX"] = np.array(solver.Args["leftX"])
    path = os.path.join(HERE, "reference_golden.npz")
    np.savez_compressed(path, **out)
    print(f"wrote {path} ({os.path.getsize(path) / 1e6:.2f} MB, {len(out)} arrays)")


if __name__ == "__main__":
    if not REF or not os.path.isdir(REF):
        sys.exit("usage: make_golden.py <path-to-reference-checkout> (or set CHIMERA_REFERENCE)")
    main()
