"""GPU parity of whole PIC steps: the drop-in ChimeraRun on CUDA against runs
of the reference's own step loop (golden fixtures, tests/golden/).  FP64:
1e-10 relative L2 per quantity after several steps."""
from copy import deepcopy

import numpy as np
import pytest

from conftest import rel_l2

pytestmark = pytest.mark.gpu
TOL = 1e-10


def _run_lpa(window, nsteps):
    from chimera_gb300 import ChimeraRun, Solver, Specie
    from chimera_gb300.messages import msg
    msg.quiet = True
    np.random.seed(1001)
    dx, dr = 0.1, 0.25
    solver = Solver({"Grid": (-6.0, 0.4, 4.0, dx, dr), "TimeStep": dx, "MaxAzimuthMode": 1,
                     "Features": ("SpaceCharge", "StillAsBackground")})
    solver.add_gauss_beam({"a0": 1.0, "k0": 1.0, "x0": -2.5, "x_foc": 2.0, "Lx": 1.5, "LR": 2.5})
    EG0 = solver.Data["EG_fb"].cpu().numpy().copy()
    el_in = {"Grid": (-6.0, 0.4, 4.0, dx, dr), "TimeStep": dx, "Density": 0.02,
             "FixedCell": (2, 2, 2), "Features": ()}
    io_in = deepcopy(el_in)
    io_in["Charge"], io_in["Mass"], io_in["Features"] = 1.0, 1836.0, ("Still",)
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
        comps["MovingFrames"] = ({"TimeStep": dx, "Steps": 1, "Velocity": 1.0},)
    run = ChimeraRun(comps)
    for i in range(1, nsteps + 1):
        run.make_step(i)
    return solver, electrons, ions, EG0


@pytest.mark.parametrize("tag,window", [("lpa", False), ("lpa_window", True)])
def test_lpa_steps_match_reference(cuda, golden, tag, window):
    nsteps = int(golden[f"{tag}/nsteps"])
    solver, el, io, EG0 = _run_lpa(window, nsteps)
    assert rel_l2(EG0, golden[f"{tag}/EG_fb_init"]) < 1e-12  # laser init
    assert abs(solver.Args["leftX"] - float(golden[f"{tag}/leftX"])) < 1e-12
    for k in ("EG_fb", "J_fb", "Rho_fb", "EB", "BckGrndRho"):
        assert rel_l2(solver.Data[k].cpu().numpy(), golden[f"{tag}/solver/{k}"]) < TOL, k
    for k in ("coords", "coords_halfstep", "momenta", "weights", "EB"):
        ref = golden[f"{tag}/electrons/{k}"]
        got = el.Data[k].cpu().numpy()
        assert got.shape == ref.shape, k
        assert rel_l2(got, ref) < TOL, k
    assert io.Data["coords"].shape == golden[f"{tag}/ions/coords"].shape


def test_fel_steps_match_reference(cuda, golden):
    from chimera_gb300 import ChimeraRun, Solver, Specie, fimera
    from chimera_gb300.messages import msg
    msg.quiet = True
    np.random.seed(1004)
    K0, periods, g0 = 1.0, 4.0, 20.0
    gg = g0 / (1. + K0 ** 2 / 2) ** .5
    k_res = 2 * gg ** 2
    vb = (1. - gg ** -2) ** 0.5
    Lgx, Rg, Nx, Nr = 0.6, 3.0, 64, 24
    dt = 1. / 30
    solver = Solver({"Grid": (-0.5 * Lgx, 0.5 * Lgx, Rg, Lgx / Nx, Rg / Nr), "TimeStep": dt,
                     "MaxAzimuthMode": 1, "KxShift": k_res, "Rcut": 0.8 * Rg, "CoPropagative": vb,
                     "Features": {"NoPoissonCorrection": True}})
    solver.add_gauss_beam({"a0": 0.05, "k0": k_res, "x0": -0.05, "x_foc": 1.0, "Lx": 0.08,
                           "LR": 1.2})
    beam = Specie({"Grid": (-0.5 * Lgx, 0.5 * Lgx, Rg, Lgx / Nx, 0.4 / Nr), "TimeStep": dt,
                   "Charge": -1., "Mass": 1., "Density": 1e-4, "RandCell": 4,
                   "MomentaMeans": (g0, 0., 0.), "MomentaSpreads": (1e-3 * g0, 1e-3, 1e-3),
                   "Devices": ([fimera.undul_analytic, np.array([K0, 1., 1., periods])],)})
    beam.add_particles(*beam.gen_parts(Domain=(-0.1, 0.1, 0.0, 0.4)))
    for k in ("coords", "momenta", "weights"):
        assert rel_l2(beam.Data[k].cpu().numpy(), golden[f"fel/init/{k}"]) < 1e-15
    run = ChimeraRun({"Solvers": (solver,), "Particles": (beam,),
                      "MovingFrames": ({"TimeStep": dt, "Steps": 1, "Velocity": vb,
                                        "Features": ("Staged", "NoSorting")},)})
    for i in range(1, 6):
        run.make_step(i)
    for k in ("EG_fb", "EB"):
        assert rel_l2(solver.Data[k].cpu().numpy(), golden[f"fel/solver/{k}"]) < TOL, k
    for k in ("coords", "momenta", "EB"):
        assert rel_l2(beam.Data[k].cpu().numpy(), golden[f"fel/beam/{k}"]) < TOL, k


def test_static_kick_steps_match_reference(cuda, golden):
    """Beam-only StaticKick run (the space-charge demo's solver: Poisson
    correction, static field solve and field drift at the beam's mean
    momentum, Staged frame, Xchunked deposits) against the reference's step
    loop."""
    from chimera_gb300 import ChimeraRun, Solver, Specie
    from chimera_gb300.messages import msg
    msg.quiet = True
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
    for k in ("coords", "momenta", "weights"):
        assert rel_l2(beam.Data[k].cpu().numpy(), golden[f"static/init/{k}"]) < 1e-14, k
    run = ChimeraRun({"Solvers": (solver,), "Particles": (beam,),
                      "MovingFrames": ({"TimeStep": dt, "Steps": 1,
                                        "Features": ("NoSorting", "Staged")},)})
    for i in range(4):
        run.make_step(i)
    assert abs(solver.Args["leftX"] - float(golden["static/leftX"])) < 1e-12
    for k in ("EG_fb", "J_fb", "EB"):
        assert rel_l2(solver.Data[k].cpu().numpy(), golden[f"static/solver/{k}"]) < TOL, k
    # the x-chunk sort orders particles inside a chunk differently (the
    # reference's numpy quicksort vs a stable sort): compare particle sets,
    # each run's particles in the order of their positions
    got_c, ref_c = beam.Data["coords"].cpu().numpy(), golden["static/beam/coords"]
    assert got_c.shape == ref_c.shape
    key = lambda c: np.lexsort(np.round(c, 9)[::-1])  # noqa: E731  (round-off ties)
    og, orf = key(got_c), key(ref_c)
    for k in ("coords", "coords_halfstep", "momenta"):
        got = beam.Data[k].cpu().numpy()[:, og]
        ref = golden[f"static/beam/{k}"][:, orf]
        assert rel_l2(got, ref) < TOL, k
