"""Host-side logic of the drop-in API against golden vectors produced by the
reference's own Python (tests/golden/make_golden.py): the FP64 operator build
and particle generation.  No kernel is called (tensors live on the CPU)."""
import os
from copy import deepcopy

import numpy as np
import pytest

from conftest import rel_l2

import sys, os  # noqa: E401
sys.path.insert(0, os.path.join(os.path.dirname(__file__), "golden"))


def _configs():
    from make_golden import solver_configs
    return solver_configs()


@pytest.mark.parametrize("name", ["lpa_m2", "lpa_m3_chunked", "plain_m1_vacuum", "fel_env_k1"])
def test_operator_build_matches_reference(golden, name):
    from chimera_gb300.solvers import Solver
    from chimera_gb300.messages import msg
    msg.quiet = True
    s = Solver(deepcopy(_configs()[name]), device="cpu")
    pre = f"op/{name}/Args/"
    keys = [k[len(pre):] for k in golden.files if k.startswith(pre)]
    assert keys
    for k in keys:
        ref = golden[pre + k]
        got = np.asarray(s.Args[k])
        assert got.shape == ref.shape, k
        if ref.dtype.kind in "fc":
            assert rel_l2(got, ref) <= 1e-15 or np.array_equal(got, ref), k
        else:
            assert np.array_equal(got, ref), k
    for k in ("PSATD_E", "PSATD_G"):
        ref = golden[f"op/{name}/Data/{k}"]
        got = s.Data[k].numpy()
        assert got.shape == ref.shape and rel_l2(got, ref) < 1e-15, k
    if name == "lpa_m2":
        assert np.array_equal(s.get_damp_profile(12), golden["op/lpa_m2/damp_profile"])


def test_gen_parts_matches_reference(golden):
    from chimera_gb300.species import Specie
    np.random.seed(7)
    sp = Specie({"Grid": (-2.0, 1.0, 2.0, 0.1, 0.25), "TimeStep": 0.1, "Density": 0.01,
                 "FixedCell": (2, 2, 3), "MomentaSpreads": (0.1, 0.05, 0.05)}, device="cpu")
    c, p, w = sp.gen_parts(Domain=(-1.5, 0.8, 0.0, 1.5),
                           ProfileFunc=lambda x, r: np.exp(-r ** 2) * (1 + 0.1 * x))
    assert c.shape == golden["gen/fixed/coords"].shape
    assert rel_l2(c, golden["gen/fixed/coords"]) < 1e-15
    assert np.array_equal(p, golden["gen/fixed/momenta"])
    assert rel_l2(w, golden["gen/fixed/weights"]) < 1e-15
    c, p, w = sp.gen_parts(Xsteps=3)
    assert rel_l2(c, golden["gen/xsteps/coords"]) < 1e-15
    assert np.array_equal(p, golden["gen/xsteps/momenta"])


def test_particle_store_append_and_permute_host():
    import torch
    from chimera_gb300.species import ParticleStore
    st = ParticleStore({"a": 3, "w": 1}, torch.device("cpu"), capacity=4)
    st.append({"a": np.arange(15.).reshape(3, 5), "w": np.arange(5.)})
    assert st.n == 5 and st.cap >= 5
    v = st.views()
    assert v["a"].shape == (3, 5) and v["w"].shape == (5,)
    assert v["a"].stride() == (st.cap, 1)


def test_moving_frame_defaults():
    from chimera_gb300.chimera_main import ChimeraRun
    run = ChimeraRun.__new__(ChimeraRun)
    run.MovingFrames = ({}, {"Features": ("Staged",), "Velocity": 0.5, "TimeStep": 0.1,
                             "Steps": 2})
    run.init_Moving_Frames()
    assert run.MovingFrames[0]["shiftX"] == 1.0
    assert abs(run.MovingFrames[1]["shiftX"] - 0.05) < 1e-15


def test_cell_order_patches_and_deposit_cells():
    """cell_order: a stable permutation; consecutive particles stay in one
    generation cell until it is exhausted, a cell's lower deposit cell
    (r < (j + 1/2) dr) comes before its upper one, the cells of a patch are
    contiguous, and consecutive cells/patches are neighbours."""
    torch = pytest.importorskip("torch")
    from chimera_gb300.split import cell_order
    rng = np.random.default_rng(7)
    dx, dr, X0 = 0.04, 0.4, -3.0
    nxc, nrc, ppc = 37, 21, 6
    gx = np.repeat(np.arange(nxc), nrc * ppc)
    gr = np.tile(np.repeat(np.arange(nrc), ppc), nxc)
    x = X0 + (gx + rng.uniform(0.01, 0.99, gx.size)) * dx
    r = (gr + rng.uniform(0.01, 0.99, gr.size)) * dr
    th = rng.uniform(0, 2 * np.pi, gx.size)
    coords = np.vstack([x, r * np.cos(th), r * np.sin(th)])
    perm = rng.permutation(gx.size)
    coords, gx, gr = coords[:, perm], gx[perm], gr[perm]
    P = 8
    o = cell_order(coords, X0, dx, dr, patch=P)
    assert sorted(o.tolist()) == list(range(gx.size))
    cx, cr = gx[o], gr[o]
    half = (np.sqrt(coords[1] ** 2 + coords[2] ** 2) / dr - gr >= 0.5)[o]
    cell = cx * 1000 + cr
    # each generation cell is one contiguous stretch, lower half first
    starts = np.flatnonzero(np.diff(cell)) + 1
    assert len(starts) == nxc * nrc - 1
    for a, b in zip(np.r_[0, starts], np.r_[starts, cell.size]):
        h = half[a:b]
        assert np.all(np.diff(h.astype(int)) >= 0)
        # stable: original order kept within a deposit cell
        for v in (False, True):
            idx = o[a:b][h == v]
            assert np.all(np.diff(idx) > 0)
    # consecutive cells are neighbours (serpentine) inside a patch, and
    # consecutive patches are neighbours
    seq_x, seq_r = cx[np.r_[0, starts]], cr[np.r_[0, starts]]
    pseq = (seq_x // P) * 1000 + seq_r // P
    pch = np.flatnonzero(np.diff(pseq)) + 1
    assert len(np.unique(pseq)) == len(pch) + 1  # every patch contiguous
    inner = np.setdiff1d(np.arange(1, seq_x.size), pch)
    assert np.all(np.abs(np.diff(seq_x))[inner - 1] + np.abs(np.diff(seq_r))[inner - 1] == 1)
    px, pr = seq_x[np.r_[0, pch]] // P, seq_r[np.r_[0, pch]] // P
    assert np.all(np.abs(np.diff(px)) + np.abs(np.diff(pr)) == 1)
    # the torch path gives the same permutation
    ot = cell_order(torch.from_numpy(coords), X0, dx, dr, patch=P)
    assert np.array_equal(ot.numpy(), o)


def test_snapshot_keys_and_restore_host(tmp_path):
    """drop_snap / read_snap key layout (chimera_main.py:325-410) on stand-in
    solver / species objects: containers and callables are skipped, arrays
    and scalars round-trip, species are resized to the stored count."""
    torch = pytest.importorskip("torch")
    from chimera_gb300 import snapshot

    class Store:
        def __init__(self):
            self.n = 3

        def resize(self, n):
            self.n = n

    class Sp:
        def __init__(self, n):
            self.store = Store()
            self.device = torch.device("cpu")
            self.chunks = torch.arange(4)
            self.w = torch.arange(8, dtype=torch.float64)
            self.store.n = n
            self.Data = {}
            self._sync()
            self.Args = {"dx": 0.1, "Features": ("Still",), "Xgrid": np.linspace(0, 1, 5),
                         "ProfileFunc": (lambda x: x), "Nx": 4, "name": "el"}

        def _sync(self):
            self.Data["weights"] = self.w[:self.store.n]

    class Sol:
        def __init__(self):
            self.Data = {"EB": torch.zeros((4, 3), dtype=torch.complex128), "nothing": None}
            self.Args = {"leftX": -1.5, "Grid": (0, 1), "kx": np.arange(6.0).reshape(2, 3)}

    sol, sp = Sol(), Sp(3)
    sol.Data["EB"] += 1 + 2j
    sp.w += 10
    arrays = snapshot.snap_arrays([sol], [sp])
    assert set(arrays) == {"solver0/Data/EB", "solver0/Args/leftX", "solver0/Args/kx",
                           "specie0/Data/weights", "specie0/Args/dx", "specie0/Args/Xgrid",
                           "specie0/Args/Nx", "specie0/Args/name", "specie0/chunks",
                           "NumSolvers", "NumSpecies", "NumThreads"}
    fname = snapshot.write(str(tmp_path / "s.npz"), arrays)
    sol2, sp2 = Sol(), Sp(5)
    sol2.Args["leftX"] = 0.0
    with np.load(fname) as f:
        snapshot.read_into(f, [sol2], [sp2])
    assert torch.equal(sol2.Data["EB"], sol.Data["EB"])
    assert sol2.Args["leftX"] == -1.5 and isinstance(sol2.Args["leftX"], float)
    assert np.array_equal(sol2.Args["kx"], sol.Args["kx"]) and sol2.Args["kx"].flags.f_contiguous
    assert sp2.store.n == 3 and torch.equal(sp2.Data["weights"], sp.Data["weights"])
    assert torch.equal(sp2.chunks, sp.chunks) and sp2.Args["name"] == "el"


def test_fixed_cell_tables_reproduce_the_host_generator():
    """The device generator's tables (species.fixed_cell_tables) and its
    index rule (particle (ir, ix, ip) at base[ir] + ix count[ir] +
    rank[ir, ip]), restated in numpy with the kernel's arithmetic, give the
    host generator's particles (fixed_cell_particles), including a grid
    whose first row drops pattern points (r <= 0)."""
    from chimera_gb300.species import fixed_cell_particles, fixed_cell_tables
    rng = np.random.default_rng(4)
    fc = (2, 3, 4)
    px, pr, po = np.mgrid[1:fc[0]:fc[0] * 1j, 1:fc[1]:fc[1] * 1j, 1:fc[2]:fc[2] * 1j]
    packx = (px.ravel() - 0.5) / fc[0]
    packr = (pr.ravel() - 0.5) / fc[1]
    packo = np.exp(2.j * np.pi * (po.ravel() - 1) / fc[2])
    for Rgrid in (0.3 * (np.arange(7) - 0.5), 0.3 * (np.arange(7) - 1.2)):
        Xgrid = -1.0 + 0.1 * np.arange(5)
        rand_o = np.asfortranarray(rng.random((5, 7)))
        ref = fixed_cell_particles(Xgrid, Rgrid, rand_o, packx, packr, packo)
        cx, cr, keep, count, rank, base = fixed_cell_tables(Xgrid, Rgrid, packx, packr)
        nxc, nrc, npc = cx.shape[0], cr.shape[0], packx.shape[0]
        num = int(count.sum()) * nxc
        assert num == ref.shape[1]
        out = np.zeros((4, num))
        for ir in range(nrc):
            for ix in range(nxc):
                for ip in range(npc):
                    if rank[ir, ip] < 0:
                        continue
                    o = base[ir] + ix * count[ir] + rank[ir, ip]
                    ang = 2.0 * np.pi * rand_o[ix, ir]
                    c, s = np.cos(ang), np.sin(ang)
                    ore = packo[ip].real * c - packo[ip].imag * s
                    oim = packo[ip].real * s + packo[ip].imag * c
                    out[:, o] = (cx[ix, ip], cr[ir, ip] * oim, cr[ir, ip] * ore, cr[ir, ip])
        assert np.array_equal(out[0], ref[0]) and np.array_equal(out[3], ref[3])
        assert np.abs(out[1:3] - ref[1:3]).max() <= 1e-15 * np.abs(ref[1:3]).max()


def test_diagnostics_dispatch_and_files_host(tmp_path, monkeypatch):
    """Diagnostics (diagnostics.py:27-149) host logic with stand-in solver /
    species objects and the device reductions replaced by the oracle's numpy
    restatements: Step selection, Return data, file names and contents."""
    torch = pytest.importorskip("torch")
    from oracle import oracle as orc
    from chimera_gb300 import diagnostics as dg

    monkeypatch.setattr(dg.chimera, "em_energy",
                        lambda eg, ef: torch.from_numpy(orc.em_energy(eg.numpy(), np.asarray(ef))))
    monkeypatch.setattr(dg.chimera, "power_profile",
                        lambda d, rg, fac: torch.from_numpy(orc.power_profile(d.numpy(), rg, fac)))
    monkeypatch.setattr(dg.chimera, "fb_vec_out", lambda v, leftX, kx, Out: v.clone())
    monkeypatch.setattr(dg.chimera, "to_device", lambda a, dtype, dev=None: torch.as_tensor(a))
    rng = np.random.default_rng(2)

    class Sol:
        Args = {"EnergyFact": rng.uniform(size=(8, 5, 2)), "RgridFull": np.linspace(-0.1, 1, 5),
                "dr": 0.25, "leftX": 0.0, "FBoutFull": (None, None), "MaxAzimuthMode": 1}
        Data = {"EG_fb": torch.from_numpy(rng.standard_normal((8, 5, 2, 6))
                                          + 1j * rng.standard_normal((8, 5, 2, 6))),
                "EB": torch.zeros((8, 6, 2, 6), dtype=torch.complex128)}

    class Run:
        Solvers = (Sol(),)
        Particles = ()

    sol = Run.Solvers[0]
    D = dg.Diagnostics(Run(), ({"Type": "EnergyEM", "Step": 3}, {"Type": "Power", "Step": 2},
                               {"Type": "Fields", "Step": 2}), out_folder=str(tmp_path / "d"))
    D.do_diags(1)
    assert sorted(os.listdir(tmp_path / "d")) == []
    D.do_diags(2)
    assert sorted(os.listdir(tmp_path / "d")) == ["ee_0_0000002.npy", "pwrX_0.txt"]
    D.do_diags(6)
    assert sorted(os.listdir(tmp_path / "d")) == ["ee_0_0000002.npy", "ee_0_0000006.npy",
                                                  "nrg_0.txt", "pwrX_0.txt"]
    e = orc.em_energy(sol.Data["EG_fb"].numpy(), sol.Args["EnergyFact"])
    e = np.r_[e[8 // 2 + 1:], e[:8 // 2 + 1]]
    assert np.allclose(np.loadtxt(tmp_path / "d" / "nrg_0.txt"), e, rtol=1e-14, atol=0)
    p = np.loadtxt(tmp_path / "d" / "pwrX_0.txt")
    assert p.shape == (2, 8)  # appended at steps 2 and 6
    (ret,) = D.nrg_out({"Type": "EnergyEM", "Step": 1, "Features": {"Return": True}})
    assert np.allclose(ret, e, rtol=1e-14, atol=0)


def test_window_cells_advance_exactly():
    """The split form's window position in cells: a move by a whole number
    of cells keeps the FP64 fraction exactly (the still species' background
    then moves with the window), fractional moves carry into the whole
    cells, and the position tracks the accumulated leftX to rounding."""
    from chimera_gb300.split import window_cells, window_cells_after
    X0, dx = -81.92 + 0.04, 0.04
    leftX = X0 + 0.37 * dx
    k, fd = window_cells(leftX, X0, dx)
    assert k == 0 and abs(fd - 0.37) < 1e-12
    k1, fd1 = window_cells_after(k, fd, dx, dx)  # one cell
    leftX += dx
    assert k1 == 1 and abs(fd1 - fd) < 1e-15  # (fd + 1 - 1 in FP64)
    f_first = fd1
    for _ in range(500):
        k1, fd1 = window_cells_after(k1, fd1, dx, dx)
        leftX += dx
    assert k1 == 501 and fd1 == f_first  # bitwise after the first move
    kl, fl = window_cells(leftX, X0, dx)
    assert abs((kl + fl) - (k1 + fd1)) < 1e-9  # the accumulated leftX agrees to rounding
    # a staged half move carries after two halves
    k2, f2 = window_cells_after(0, 0.75, 0.5 * 0.999 * dx, dx)
    assert k2 == 1 and abs(f2 - (0.75 + 0.4995 - 1.0)) < 1e-12


def test_background_shift_decision():
    """When the split form may move the still species' background with the
    window instead of re-depositing it (SplitRun._bg_shift): a whole-cell
    move of one unchanged still species without absorption or injection."""
    from types import SimpleNamespace

    from chimera_gb300.split import SplitRun
    dx = 0.04
    P = SimpleNamespace(n=1000, cap=2048, ptrs=lambda: [11, 12, 13, 14, 15, 16, 17, 18])
    run = SplitRun.__new__(SplitRun)
    run.nm, run.nx, run.dx = 3, 4096, dx
    run.have_bg = True
    run._wk, run._wfd = 10, 0.25
    run._bg_key = (P.n, P.cap, *P.ptrs())
    run._still = lambda: [(None, P)]
    assert run._bg_shift({"shiftX": dx}) == 1
    assert run._bg_shift({"shiftX": 3 * dx}) == 3
    assert run._bg_shift({"shiftX": 0.5 * dx}) == 0           # not a whole cell
    assert run._bg_shift({"shiftX": dx, "AbsorbLayer": 64}) == 0
    assert run._bg_shift({"shiftX": dx, "AddPlasma": None}) == 0
    run._bg_key = None                                         # particles changed
    assert run._bg_shift({"shiftX": dx}) == 0
    run._bg_key = (P.n, P.cap, *P.ptrs())
    run._still = lambda: [(None, P), (None, P)]               # two still species
    assert run._bg_shift({"shiftX": dx}) == 0
    run._still = lambda: [(None, P)]
    run.have_bg = False
    assert run._bg_shift({"shiftX": dx}) == 0


def test_sort_cadence_rule(monkeypatch):
    """SortCadence (the re-sort autotuner) on fake step and sort timings: the
    cadence is sqrt(2 S / g) with S the sort time and g the per-step time a
    sort recovered over the interval before it, clamped to [lo, hi]; a sort
    that recovers nothing sends it to hi."""
    import torch

    from chimera_gb300.split import SortCadence

    class Ev:
        def __init__(self, enable_timing=True):
            self.t = 0.0

        def query(self):
            return True

        def elapsed_time(self, other):
            return other.t - self.t

    monkeypatch.setattr(torch.cuda, "Event", Ev)
    sc = SortCadence(start=32, lo=8, hi=512)

    def interval(nsteps, base, slope, sort_ms):
        for s in range(nsteps):
            a, b = sc.step_events(s)
            b.t = base + slope * s
        a, b = sc.sort_events()
        b.t = sort_ms

    interval(32, 1.0, 0.01, 8.0)
    sc.update(32)
    assert sc.cadence == 32 and sc.history[-1] == (32, 32, 8.0, None)  # no earlier sort
    interval(32, 1.0, 0.01, 8.0)
    sc.update(64)
    g = 0.01 * (29.5 - 1.5) / 32  # last four minus first four steps, per step
    assert abs(sc.history[-1][3] - g) < 1e-12
    assert sc.cadence == int(np.sqrt(2 * 8.0 / g)) == 42
    interval(42, 1.0, 1.0, 8.0)      # slower after the sort than before it: hi
    sc.update(106)
    assert sc.history[-1][3] < 0 and sc.cadence == 512
    interval(8, 1.0, 0.0, 8.0)       # the sort recovered 39.5 ms over 42 steps: lo
    sc.update(114)
    assert abs(sc.history[-1][3] - 39.5 / 42) < 1e-12 and sc.cadence == 8
    interval(3, 1.0, 0.5, 8.0)       # too few steps to judge: unchanged
    sc.update(117)
    assert sc.history[-1][3] is None and sc.cadence == 8
    interval(8, 1.0, 0.0, 8.0)       # nothing recovered: hi
    sc.update(125)
    assert sc.history[-1][3] == 0 and sc.cadence == 512 and len(sc.history) == 6


def test_fused_undulator_parsing():
    """The devices the split push fuses (split.fused_undulator): the
    analytic and mapped undulators with their parameter counts, the map
    as FP32 column pairs; other devices, two devices and wrong parameter
    counts raise."""
    import torch

    from chimera_gb300 import fimera
    from chimera_gb300.split import fused_undulator
    cpu = torch.device("cpu")
    assert fused_undulator((), cpu) is None
    k, prm, amap = fused_undulator(([fimera.undul_analytic, np.array([2.0, 1.0, 1.0, 80.0])],), cpu)
    assert k == 1 and prm.tolist() == [2.0, 1.0, 1.0, 80.0] and amap is None
    k, _, _ = fused_undulator(([fimera.undul_analytic_taper, np.arange(5.0)],), cpu)
    assert k == 2
    a0 = np.asfortranarray(np.arange(14.0).reshape(2, 7))
    k, prm, amap = fused_undulator(([fimera.undul_mapped, a0, np.array([1.0, 0.3, 0.01])],), cpu)
    assert k == 3 and amap.dtype == torch.float32 and tuple(amap.shape) == (7, 2)
    assert amap.is_contiguous() and np.array_equal(amap.numpy(), a0.T)  # (a(0, c), a(1, c))
    k, _, amap = fused_undulator(([fimera.undul_mapped_tap, torch.from_numpy(a0),
                                   np.arange(5.0)],), cpu)
    assert k == 4 and np.array_equal(amap.numpy().ravel(), a0.T.ravel())
    with pytest.raises(NotImplementedError):
        fused_undulator(([fimera.planewave, np.zeros(7)],), cpu)
    with pytest.raises(NotImplementedError):
        fused_undulator(([fimera.undul_analytic, np.zeros(4)],) * 2, cpu)
    with pytest.raises(NotImplementedError):
        fused_undulator(([fimera.undul_mapped, np.zeros(3)],), cpu)  # no map
    with pytest.raises(ValueError):
        fused_undulator(([fimera.undul_analytic, np.zeros(3)],), cpu)
    with pytest.raises(ValueError):
        fused_undulator(([fimera.undul_mapped, np.zeros((3, 7)), np.zeros(3)],), cpu)
