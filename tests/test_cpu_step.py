"""The CPU step driver used as the benchmark's CPU baseline (oracle/step.py)
reproduces the golden runs of the reference's own step loop."""
from copy import deepcopy

import numpy as np
import pytest

from conftest import rel_l2


def _lpa(window):
    from chimera_gb300.messages import msg
    from chimera_gb300.solvers import Solver
    from chimera_gb300.species import Specie
    from oracle.step import CpuRun, CpuSpecies
    msg.quiet = True
    np.random.seed(1001)
    dx, dr = 0.1, 0.25
    solver = Solver({"Grid": (-6.0, 0.4, 4.0, dx, dr), "TimeStep": dx, "MaxAzimuthMode": 1,
                     "Features": ("SpaceCharge", "StillAsBackground")}, device="cpu")
    # the laser init runs kernels: take the reference's initial spectral field
    el_in = {"Grid": (-6.0, 0.4, 4.0, dx, dr), "TimeStep": dx, "Density": 0.02,
             "FixedCell": (2, 2, 2), "Features": ()}
    io_in = deepcopy(el_in)
    io_in["Charge"], io_in["Mass"], io_in["Features"] = 1.0, 1836.0, ("Still",)
    el, io = Specie(el_in, device="cpu"), Specie(io_in, device="cpu")
    prof = lambda x: np.interp(x, [-4.0, -3.0, 10.0], [0.0, 1.0, 1.0])  # noqa: E731
    parts = el.gen_parts(Domain=(-5.5, 0.3, 0.0, 3.5), ProfileFunc=prof)
    el.add_particles(*[p.copy() for p in parts])
    parts[-1] *= -1
    io.add_particles(*parts)
    if window:
        wind = {"TimeStep": dx, "Steps": 2, "AbsorbLayer": 8, "AddPlasma": prof,
                "Features": ("IonsOnTop",)}
    else:
        wind = {"TimeStep": dx, "Steps": 1, "Velocity": 1.0}
    return solver, CpuSpecies(el), CpuSpecies(io), wind, CpuRun


@pytest.mark.parametrize("tag,window", [("lpa", False), ("lpa_window", True)])
def test_cpu_step_driver_matches_reference_step_loop(golden, tag, window):
    import torch
    solver, el, io, wind, CpuRun = _lpa(window)
    solver.Data["EG_fb"] = torch.from_numpy(np.asfortranarray(golden[f"{tag}/EG_fb_init"]))
    run = CpuRun(solver, [el, io], wind)
    for i in range(1, int(golden[f"{tag}/nsteps"]) + 1):
        run.make_step(i)
    for k in ("EG_fb", "J_fb", "Rho_fb", "EB", "BckGrndRho"):
        assert rel_l2(run.D[k], golden[f"{tag}/solver/{k}"]) < 1e-13, k
    for k in ("coords", "momenta", "weights"):
        assert rel_l2(el.Data[k], golden[f"{tag}/electrons/{k}"]) < 1e-13, k


def test_cpu_laser_init_matches_reference(golden):
    """oracle.step.add_gauss_beam (the benchmark's CPU arm) reproduces the
    reference's spectral laser initialisation (solvers.py:555-610)."""
    import torch
    from oracle.step import add_gauss_beam
    solver, *_ = _lpa(False)
    solver.Data["EG_fb"] = torch.zeros(tuple(solver.Data["EG_fb"].shape), dtype=torch.complex128)
    add_gauss_beam(solver, {"a0": 1.0, "k0": 1.0, "x0": -2.5, "x_foc": 2.0, "Lx": 1.5, "LR": 2.5})
    assert rel_l2(solver.Data["EG_fb"].numpy(), golden["lpa/EG_fb_init"]) < 1e-12
