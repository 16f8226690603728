"""Checkpoints (chimera_main.py:325-410 drop_snap / read_snap as .npz): a run
restarted from a snapshot continues bitwise as the run that wrote it, in the
FP64 form and in the split form, with a moving window that absorbs and
injects plasma."""
from copy import deepcopy

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _comps():
    from chimera_gb300 import Solver, Specie
    from chimera_gb300.messages import msg
    msg.quiet = True
    np.random.seed(1001)
    dx, dr = 0.1, 0.25
    grid = (-6.0, 0.4, 4.0, dx, dr)
    solver = Solver({"Grid": grid, "TimeStep": dx, "MaxAzimuthMode": 1,
                     "Features": ("SpaceCharge", "StillAsBackground")})
    solver.add_gauss_beam({"a0": 1.0, "k0": 1.0, "x0": -2.5, "x_foc": 2.0, "Lx": 1.5, "LR": 2.5})
    el_in = {"Grid": grid, "TimeStep": dx, "Density": 0.02, "FixedCell": (2, 2, 2),
             "Features": ()}
    io_in = deepcopy(el_in)
    io_in["Charge"], io_in["Mass"], io_in["Features"] = 1.0, 1836.0, ("Still",)
    electrons, ions = Specie(el_in), Specie(io_in)
    prof = lambda x: np.interp(x, [-4.0, -3.0, 10.0], [0.0, 1.0, 1.0])  # noqa: E731
    parts = electrons.gen_parts(Domain=(-5.5, 0.3, 0.0, 3.5), ProfileFunc=prof)
    electrons.add_particles(*[p.copy() for p in parts])
    parts[-1] *= -1
    ions.add_particles(*parts)
    return {"Solvers": (solver,), "Particles": (electrons, ions),
            "MovingFrames": ({"TimeStep": dx, "Steps": 2, "AbsorbLayer": 8,
                              "AddPlasma": prof, "Features": ("IonsOnTop",)},)}


def _state(run):
    import torch
    s = run.Solvers[0]
    out = [s.Data["EG_fb"].clone(), s.Data["EB"].clone()]
    for sp in run.Particles:
        out += [sp.Data["coords"].clone(), sp.Data["momenta"].clone(), sp.Data["weights"].clone()]
    return out, torch


def test_fp64_restart_is_bitwise(cuda, tmp_path):
    from chimera_gb300 import ChimeraRun
    a = ChimeraRun(_comps())
    for i in range(1, 4):
        a.make_step(i)
    fname = a.drop_snap(str(tmp_path / "snap_"))
    assert fname.endswith(".npz")
    keys = set(np.load(fname).files)
    assert {"NumSolvers", "NumSpecies", "NumThreads", "solver0/Data/EG_fb", "solver0/Args/leftX",
            "specie0/Data/coords", "specie1/Args/Features"} - keys == {"specie1/Args/Features"}
    np.random.seed(77)
    for i in range(4, 8):
        a.make_step(i)
    b = ChimeraRun(_comps())
    b.read_snap(fname)
    np.random.seed(77)
    for i in range(4, 8):
        b.make_step(i)
    (sa, torch), (sb, _) = _state(a), _state(b)
    for x, y in zip(sa, sb):
        assert x.shape == y.shape and torch.equal(x, y)


def test_split_restart_is_bitwise(cuda, tmp_path):
    import torch
    from chimera_gb300.split import SplitRun
    a = SplitRun(_comps())
    for i in range(1, 4):
        a.make_step(i)
    fname = a.drop_snap(str(tmp_path / "snap_"))
    np.random.seed(77)
    for i in range(4, 8):
        a.make_step(i)
    b = SplitRun(_comps())
    b.read_snap(fname)
    np.random.seed(77)
    for i in range(4, 8):
        b.make_step(i)
    assert torch.equal(a.EG, b.EG)
    for Pa, Pb in zip(a.parts, b.parts):
        assert Pa.n == Pb.n
        # the slots of particles 0 .. n-1 in the tile layout (chm_sp_slot);
        # the unused slots of the last tile hold stale values
        i = torch.arange(Pa.n, device=a.EG.device)
        slot = (i & ~511) | ((i & 15) << 5) | ((i >> 4) & 31)
        for k in Pa.buf:
            assert torch.equal(Pa.buf[k][slot], Pb.buf[k][slot]), k
        assert torch.equal(Pa.dead[slot], Pb.dead[slot])
