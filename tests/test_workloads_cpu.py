"""The benchmark's and tests' workloads built on the host (no GPU): the
laser-wakefield sizes and the FEL set-up of the reference's fel-testrun.py
(envelope solver, analytic undulator, Staged window)."""
import numpy as np
import pytest


def test_lwfa_sizes():
    from chimera_gb300 import workloads
    W = workloads.SIZES["cfg3"]
    assert (W.nx, W.nkr, W.modes) == (4096, 512, 3)
    assert workloads.SIZES["cfg2"].modes == 2 and workloads.SIZES["cfg1"].nx == 512
    cfg = workloads.config("cfg1")
    assert cfg["solver"]["TimeStep"] == cfg["W"].dx  # dt = dx: one-cell window moves
    assert workloads.window("cfg1", "inject")["AbsorbLayer"] == 64


def test_fel_small_components_on_host():
    from chimera_gb300 import fimera, workloads
    comps = workloads.fel_components("fel_small", device="cpu")
    S, beam = comps["Solvers"][0], comps["Particles"][0]
    A = S.Args
    W = workloads.FEL["fel_small"]
    assert "KxShift" in A and "NoPoissonCorrection" in A["Features"]
    assert A["Mtot"] == 2 * W.max_mode + 1 and A["Nx"] == W.nx
    assert A["DpS2S"].shape[-1] == A["Mtot"] + 2  # the envelope's D operators: modes -K-1..K+1
    assert S.Data["PSATD_E"].is_complex()
    assert beam.Devices and beam.Devices[0][0] is fimera.undul_analytic
    # RandCell particles over the beam's cells: about (lbx / dx) x nr cells
    # (the generator takes every cell the domain touches)
    lbx, Lgx = 80e-4 / 2.8, 200e-4 / 2.8
    cells = lbx / (Lgx / W.nx) * W.nr
    assert beam.num_particles % W.rand_cell == 0
    assert abs(beam.num_particles / (cells * W.rand_cell) - 1) < 0.1
    wind = comps["MovingFrames"][0]
    assert "Staged" in wind["Features"] and 0.99 < wind["Velocity"] < 1.0
    x = beam.Data["coords"][0].cpu().numpy()
    assert np.all(np.abs(x) <= 0.5 * lbx + A["dx"])


@pytest.mark.parametrize("size", ["fel4", "fel_small"])
def test_fel_resonance(size):
    """k_res = 2 gamma_z^2 with gamma_z = gamma / sqrt(1 + K^2 / 2), the
    beam's speed below c by 1 / (2 gamma_z^2)."""
    from chimera_gb300 import workloads
    W = workloads.FEL[size]
    gz = W.gamma / np.sqrt(1 + W.K0 ** 2 / 2)
    vb = np.sqrt(1 - gz ** -2)
    assert abs((1 - vb) * 2 * gz ** 2 - 1) < 1e-3


def test_batched_draws_cover_the_ragged_configuration():
    """The batched workload's 64 instances (seed 1005): Nx 256-2048, Nr
    32-256, 2 or 3 stored modes, uneven particle counts; the draw is
    reproducible from its seed."""
    from chimera_gb300.batched import draw_instances
    P = draw_instances(64, 1005)
    assert P == draw_instances(64, 1005) and P != draw_instances(64, 1006)
    nx = {p["nx"] for p in P}
    nr = {p["nr"] for p in P}
    assert min(nx) >= 256 and max(nx) <= 2048 and len(nx) > 8
    assert min(nr) >= 32 and max(nr) <= 256 and len(nr) > 4
    assert {p["max_mode"] + 1 for p in P} == {2, 3}
    cells = [p["nx"] * p["nr"] * p["ppc_theta"] for p in P]
    assert max(cells) > 20 * min(cells)  # ragged: the particle counts differ widely
    assert len({p["seed"] for p in P}) == 64
