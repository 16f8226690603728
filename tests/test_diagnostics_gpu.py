"""Device diagnostics (moduls/diagnostics.py, f90/utils.f90 intens_profO):
the GPU reductions against the oracle, and the Diagnostics class on a small
laser-plasma run (returned data and written files)."""
import os
from copy import deepcopy

import numpy as np
import pytest

from conftest import rel_l2

pytestmark = pytest.mark.gpu


def _cplx(rng, shape):
    return np.asfortranarray(rng.standard_normal(shape) + 1j * rng.standard_normal(shape))


@pytest.mark.parametrize("NO,shape", [(7, (17, 9, 3, 3)), (60, (40, 13, 5, 3)), (5, (8, 4, 1, 3))])
def test_intens_profo_matches_oracle(cuda, orc, NO, shape):
    import torch
    from chimera_gb300 import fimera
    rng = np.random.default_rng(NO)
    F = _cplx(rng, shape)
    ref = orc.intens_profo(F, NO)
    Fd = fimera.to_device(F, torch.complex128)
    got = fimera.intens_profo(Fd, NO)
    assert tuple(got.shape) == ref.shape == (NO, shape[1] - 1)
    assert rel_l2(got.cpu().numpy(), ref) < 1e-12
    # fixed summation order: bitwise reproducible
    again = fimera.intens_profo(Fd, NO)
    assert torch.equal(got, again)


def test_intens_profo_rejects_even_mode_count(cuda):
    import torch
    from chimera_gb300 import fimera
    from chimera_gb300._lib import ChimeraError
    F = fimera.fortran_zeros((8, 4, 2, 3), torch.complex128)
    with pytest.raises(ChimeraError):
        fimera.intens_profo(F, 10)


def test_energy_and_power_reductions_match_oracle(cuda, orc):
    import torch
    from chimera_gb300 import fimera
    rng = np.random.default_rng(3)
    EG = _cplx(rng, (32, 12, 2, 6))
    ef = np.asfortranarray(rng.uniform(0.0, 2.0, (32, 12, 2)))
    got = fimera.em_energy(fimera.to_device(EG, torch.complex128), ef)
    assert rel_l2(got.cpu().numpy(), orc.em_energy(EG, ef)) < 1e-13
    dat = _cplx(rng, (32, 9, 2, 3))
    rg = np.linspace(-0.1, 3.0, 9)
    got = fimera.power_profile(fimera.to_device(dat, torch.complex128), rg, 7.5)
    assert rel_l2(got.cpu().numpy(), orc.power_profile(dat, rg, 7.5)) < 1e-13


def _lpa_run(nsteps):
    from chimera_gb300 import ChimeraRun, Solver, Specie
    from chimera_gb300.messages import msg
    msg.quiet = True
    np.random.seed(1001)
    dx, dr = 0.1, 0.25
    grid = (-6.0, 0.4, 4.0, dx, dr)
    solver = Solver({"Grid": grid, "TimeStep": dx, "MaxAzimuthMode": 1,
                     "Features": ("SpaceCharge", "StillAsBackground")})
    solver.add_gauss_beam({"a0": 2.0, "k0": 1.0, "x0": -2.5, "x_foc": 2.0, "Lx": 1.5, "LR": 2.5})
    el_in = {"Grid": grid, "TimeStep": dx, "Density": 0.02, "FixedCell": (2, 2, 2),
             "Features": ()}
    io_in = deepcopy(el_in)
    io_in["Charge"], io_in["Mass"], io_in["Features"] = 1.0, 1836.0, ("Still",)
    electrons, ions = Specie(el_in), Specie(io_in)
    parts = electrons.gen_parts(Domain=(-5.5, 0.3, 0.0, 3.5))
    electrons.add_particles(*[p.copy() for p in parts])
    parts[-1] *= -1
    ions.add_particles(*parts)
    run = ChimeraRun({"Solvers": (solver,), "Particles": (electrons, ions),
                      "MovingFrames": ({"TimeStep": dx, "Steps": 1, "Velocity": 1.0},)})
    for i in range(1, nsteps + 1):
        run.make_step(i)
    return run, solver, electrons


def test_diagnostics_class_on_lpa_run(cuda, orc, tmp_path):
    from chimera_gb300 import fimera
    from chimera_gb300.diagnostics import Diagnostics, PwrFctr
    run, solver, electrons = _lpa_run(2)
    A = solver.Args
    ret = {"Return": True}
    diags = [{"Type": t, "Step": 2, "Features": dict(ret)}
             for t in ("EnergyEM", "Power", "Fields", "FieldsFB", "Density", "Particles")]
    D = Diagnostics(run, diags)
    # EnergyEM: the reference's numpy expression on host copies
    eg = solver.Data["EG_fb"].cpu().numpy()
    e_ref = orc.em_energy(eg, A["EnergyFact"])
    n = e_ref.shape[0]
    e_ref = np.r_[e_ref[n // 2 + 1:], e_ref[:n // 2 + 1]]
    (nrg,) = D.nrg_out(diags[0])
    assert rel_l2(nrg, e_ref) < 1e-12
    # Power: fb_vec_out of E, then the power profile
    dat = fimera.fb_vec_out(solver.Data["EG_fb"][:, :, :, :3], A["leftX"], *A["FBoutFull"])
    p_ref = orc.power_profile(dat.cpu().numpy(), A["RgridFull"], PwrFctr * 2 * A["dr"])
    (pwr,) = D.pwr_out(diags[1])
    assert rel_l2(pwr, p_ref) < 1e-12 and pwr.max() > 0
    # field dumps are copies of Data without the ghost row
    (ee,) = D.fld_out(diags[2])
    assert np.array_equal(ee.cpu().numpy(), solver.Data["EB"][:, 1:].cpu().numpy())
    (egr,) = D.fldfb_out(diags[3])
    assert np.array_equal(egr.cpu().numpy(), eg)
    (dens,) = D.dns_out(diags[4])
    assert dens.shape[1] == electrons.Args["Nr"] - 1  # the species grid, without its row 0
    (phs,) = D.phs_out(diags[5])
    assert phs.shape[0] == 7
    # 'Spot' needs an odd mode count (-nkO..nkO); the plain solver's 2 modes
    # are rejected, as f2py rejects them for intens_profO
    with pytest.raises(Exception):
        D.pwr_out({"Type": "Power", "Step": 1, "Features": {"Return": True, "Spot": True}})
    # file output: do_diags at a due step writes the reference's files
    out = str(tmp_path / "diags")
    F = Diagnostics(run, [{"Type": t, "Step": 2} for t in ("EnergyEM", "Power", "Fields")],
                    out_folder=out)
    F.do_diags(1)  # not due
    assert os.listdir(out) == []
    F.do_diags(2)
    names = sorted(os.listdir(out))
    assert names == ["ee_0_0000002.npy", "nrg_0.txt", "pwrX_0.txt"]
    assert rel_l2(np.loadtxt(os.path.join(out, "nrg_0.txt")), nrg) < 1e-15
    assert rel_l2(np.loadtxt(os.path.join(out, "pwrX_0.txt")), pwr) < 1e-15
    env = D.get_beam_envelops()
    assert env[0].shape == (3, 3) and np.all(np.isfinite(env[0]))
