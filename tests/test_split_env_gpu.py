"""Split-precision form of the envelope (KxShift) solver: the free-electron
laser set-up of the reference (doc/tests/fel-testrun.py, workloads "fel4" and
"fel_small" of chimera_gb300/workloads.py).

- every split transform of the envelope step (fb_in with the anti-echo
  DepFact, the envelope curl with PoissFact, fb_eb_out with the envelope
  eb_correction, the complex PSATD update) against the FP64 kernels at the
  2048 x 128 x 3-mode operator sizes, within TOL_T relative L2;
- the beam's carrier-phase current deposit and its gather + undulator +
  Boris push against the FP64 kernels (dep_curr_env, proj_fld_env,
  undul_analytic, push_velocs) on the same particles, and the gather with
  a mapped undulator (undul_mapped[_tap]) likewise;
- split steps against the FP64 form from the same state: fields, beam
  momenta and the radiated energy (Diagnostics.nrg_out summed,
  diagnostics.py:109-122) within 1 %, and graph replay bitwise equal to
  make_step."""
import ctypes as C

import numpy as np
import pytest

from conftest import rel_l2

pytestmark = pytest.mark.gpu
TOL_T = 1e-6


@pytest.fixture(scope="module")
def mods(cuda):
    import torch
    from chimera_gb300 import _lib, fimera, split
    from chimera_gb300.messages import msg
    msg.quiet = True
    return torch, _lib, fimera, split


def _st(torch):
    return torch.cuda.current_stream().cuda_stream


def _c(a, torch):
    return torch.from_numpy(np.asfortranarray(a)).cuda()


def _rand(shape, seed):
    rng = np.random.default_rng(seed)
    return np.asfortranarray(rng.standard_normal(shape) + 1j * rng.standard_normal(shape))


def _energy(torch, fm, S, EG):
    """sum over kx of diagnostics.py:112-114 (EnergyFact-weighted |E|^2)."""
    eg = fm.fortran_empty(tuple(EG.shape), torch.complex128, EG.device)
    eg.copy_(EG)
    return float(fm.em_energy(eg, S.Args["EnergyFact"]).sum())


def test_envelope_transforms_at_fel_sizes(mods):
    torch, _lib, fm, split = mods
    from chimera_gb300 import workloads
    from chimera_gb300 import Solver
    W = workloads.FEL["fel4"]
    lam0 = 2.8
    gg = W.gamma / (1.0 + W.K0 ** 2 / 2) ** 0.5
    Lgx, Rg = 200e-4 / lam0, 1000e-4 / lam0
    S = Solver({"Grid": (-0.5 * Lgx, 0.5 * Lgx, Rg, Lgx / W.nx, Rg / W.nr), "TimeStep": W.dt,
                "MaxAzimuthMode": W.max_mode, "KxShift": 2 * gg ** 2, "Rcut": 700e-4 / lam0,
                "CoPropagative": (1.0 - gg ** -2) ** 0.5,
                "Features": {"NoPoissonCorrection": True}})
    A = S.Args
    nx, nr, nkr, nm = A["Nx"], A["Nr"], A["Nkr"], A["Mtot"]
    dev = torch.device("cuda")
    o = {k: split._prepare_ops(A[key], dev) for k, key in
         (("InCurr", "InCurr"), ("Out", "Out"), ("Dp", "DpS2S"), ("Dm", "DmS2S"))}
    ws = torch.empty(_lib.query("chm_sp_fb_ws_bytes", nx, nr, nkr, nm), dtype=torch.uint8, device=dev)
    st = _st(torch)
    kxb = S.dev["kx_base"]
    kx32 = S.dev["kx"].to(torch.float32)
    pf32 = _c(A["PoissFact"].astype(np.float32), torch)
    errs = {}
    # fb_in of a current accumulator (J_z only, as the envelope deposit writes)
    rng = np.random.default_rng(4)
    scale = 2.0 ** 40
    acc = np.zeros((2, nx, nr, nm, 3), np.int64, order="F")
    acc[..., 2] = (rng.standard_normal(acc[..., 2].shape) * 2.0 ** 40).astype(np.int64)
    accd = torch.from_numpy(np.ravel(acc, order="F").copy()).cuda()
    scd = torch.tensor([scale, 1.0], dtype=torch.float64, device="cuda")
    depf = _c(A["DepFact"].astype(np.float32), torch)
    leftX = float(A["leftX"]) + 0.37 * A["dx"]
    Jfb = fm.fortran_zeros((nx, nkr, nm, 3), torch.complex64)
    _lib.call("chm_sp_fb_in_acc", Jfb.data_ptr(), accd.data_ptr(), scd.data_ptr(), None, None,
              leftX, kxb.data_ptr(), C.addressof(o["InCurr"][0]), depf.data_ptr(), nx, nr, nkr, nm,
              3, ws.data_ptr(), ws.numel(), st, None)
    Jsp = (acc[0] + 1j * acc[1]) / scale
    Jsp[:, 1] -= Jsp[:, 0]
    Jsp[:, 0] = 0
    ref = fm._fb_in(fm.fortran_zeros((nx, nkr, nm, 3)), _c(Jsp, torch), leftX, *A["FBCurrIn"], 3,
                    fact=S.dev["DepFact"])
    errs["fb_in"] = rel_l2(Jfb.cpu().numpy(), ref.cpu().numpy())
    # envelope curl with PoissFact
    G = _rand((nx, nkr, nm, 3), 5).astype(np.complex64)
    Bs = fm.fortran_zeros((nx, nkr, nm, 3), torch.complex64)
    _lib.call("chm_sp_rot_b_env", Bs.data_ptr(), _c(G, torch).data_ptr(), pf32.data_ptr(),
              C.addressof(o["Dp"][0]), C.addressof(o["Dm"][0]), kx32.data_ptr(), nx, nkr, nm,
              ws.data_ptr(), ws.numel(), st)
    Bd = fm.fb_rot_env(fm.fortran_zeros((nx, nkr, nm, 3)), _c(G.astype(np.complex128), torch),
                       A["DpS2S"], A["DmS2S"], A["kx"])
    Bd = fm.omp_mult_vec(Bd, A["PoissFact"])
    errs["rot_b_env"] = rel_l2(Bs.cpu().numpy(), Bd.cpu().numpy())
    # fb_eb_out with the envelope eb_correction
    E = _rand((nx, nkr, nm, 6), 6).astype(np.complex64)
    Bq = _rand((nx, nkr, nm, 3), 7).astype(np.complex64)
    EBs = fm.fortran_zeros((nx, nr, nm, 6), torch.complex64)
    _lib.call("chm_sp_fb_eb_out_env", EBs.data_ptr(), _c(E, torch).data_ptr(),
              _c(Bq, torch).data_ptr(), leftX, kxb.data_ptr(), C.addressof(o["Out"][0]), nx, nr,
              nkr, nm, ws.data_ptr(), ws.numel(), st, None)
    EBd = fm.fb_eb_out(fm.fortran_zeros((nx, nr, nm, 6)), _c(E.astype(np.complex128), torch),
                       _c(Bq.astype(np.complex128), torch), leftX, *A["FBout"], eb_mode=2)
    errs["fb_eb_out_env"] = rel_l2(EBs.cpu().numpy(), EBd.cpu().numpy())
    # complex PSATD without space charge
    EG = _rand((nx, nkr, nm, 6), 8).astype(np.complex64)
    Jr = _rand((nx, nkr, nm, 3), 9).astype(np.complex64)
    EGs = _c(EG, torch)
    c1 = fm.fortran_empty(tuple(S.Data["PSATD_E"].shape), torch.complex64, dev)
    c1.copy_(S.Data["PSATD_E"])
    c2 = fm.fortran_empty(tuple(S.Data["PSATD_G"].shape), torch.complex64, dev)
    c2.copy_(S.Data["PSATD_G"])
    _lib.call("chm_sp_psatd_c", EGs.data_ptr(), _c(Jr, torch).data_ptr(), c1.data_ptr(),
              c2.data_ptr(), nx * nkr * nm, st)
    EGd = fm.maxwell_push_wo_spchrg(_c(EG.astype(np.complex128), torch),
                                    _c(Jr.astype(np.complex128), torch), S.Data["PSATD_E"],
                                    S.Data["PSATD_G"])
    errs["psatd_c"] = rel_l2(EGs.cpu().numpy(), EGd.cpu().numpy())
    print("envelope transforms at 2048 x 128 x 3 modes: "
          + " ".join(f"{k} {v:.2e}" for k, v in errs.items()))
    assert max(errs.values()) < TOL_T, errs
    assert _lib.load().chm_sp_umma_status() == 0


def test_envelope_particle_kernels_match_fp64(mods):
    """On the small FEL beam after two steps (fields present), from the same
    particles and fields: the split gather + undulator + Boris against
    proj_fld_env + undul_analytic + push_velocs (the end-of-step window), then
    the split push + J_z deposit with the carrier against push_coords +
    dep_curr_env (the window moved by the first half of the Staged step, as
    make_step deposits)."""
    torch, _lib, fm, split = mods
    from chimera_gb300 import ChimeraRun, workloads
    run = ChimeraRun(workloads.fel_components("fel_small", seed=1004))
    for i in range(1, 3):
        run.make_step(i)
    S, spc = run.Solvers[0], run.Particles[0]
    A, d = S.Args, spc.Data
    nx, nr, nm = A["Nx"], A["Nr"], A["Mtot"]
    dev = torch.device("cuda")
    n = spc.num_particles
    dx = float(A["dx"])
    X0 = float(A["Xgrid"][0]) - 7 * dx  # (any origin of the cell index)
    st = _st(torch)
    kdx = float(A["kx0"] * dx)
    tab = torch.zeros(nx + 4, dtype=torch.complex64, device=dev)
    x64 = fm.fortran_zeros((3, n), torch.float64)
    p64 = fm.fortran_zeros((3, n), torch.float64)
    w64 = torch.zeros(n, dtype=torch.float64, device=dev)

    def window(leftX):
        s = (leftX - X0) / dx
        k = int(np.floor(s))
        _lib.call("chm_sp_carrier", tab.data_ptr(), tab.numel(), float(A["kx0"]), X0, dx, k, st,
                  None)
        return k, s - k

    def split_parts():
        P = split._SpParticles(dev, n)
        P.append_f64(d["coords"], d["momenta"], d["weights"], X0, dx)
        return P

    def to_f64(P):
        _lib.call("chm_sp_to_f64", *P.ptrs(), P.n, x64.data_ptr(), x64.stride(0), x64.stride(1),
                  p64.data_ptr(), p64.stride(0), p64.stride(1), w64.data_ptr(), w64.stride(0), X0,
                  dx, st)

    # gather + undulator + Boris at the end-of-step window and fields
    P = split_parts()
    k, f = window(float(A["leftX"]))
    EB32 = fm.fortran_empty(tuple(S.Data["EB"].shape), torch.complex64, dev)
    EB32.copy_(S.Data["EB"])
    p0 = d["momenta"].clone()
    und = np.array(spc.Devices[0][1], dtype=np.float64)
    prm = np.zeros(5)
    prm[:und.size] = und
    dtq = spc.Args["push_fact"] * spc.Args["TimeStep"]
    _lib.call("chm_sp_gather_push_env", *P.ptrs(), P.n, k, f, float(A["dr_inv"]),
              EB32.data_ptr(), nx, nr, nm, float(dtq), tab.data_ptr(), tab.numel(), kdx, 1,
              prm.ctypes.data, None, 0, X0, dx, st, None)
    spc.make_field()
    d["EB"] = fm.proj_fld_env(d["coords"], d["weights"], S.Data["EB"], d["EB"], A["leftX"],
                              *A["DepProj"])
    gathered = float(d["EB"].abs().max())
    spc.make_device(3)
    spc.push_velocs()
    to_f64(P)
    # transverse kicks (p_x ~ gamma: its FP32 rounding would swamp its kick),
    # against the FP32-rounded initial momenta the split kernel started from
    # The kick of a co-propagating wave on the beam is E + v x B ~ (1 - v) E:
    # its error is measured against the uncancelled kick |E| dt q/m
    p0_32 = p0.to(torch.float32).to(torch.float64)
    dp_sp = (p64 - p0_32)[1:].cpu().numpy()
    dp_64 = (d["momenta"] - p0)[1:].cpu().numpy()
    err_dp = float(np.abs(dp_sp - dp_64).max()) / (gathered * abs(dtq))
    # push + J_z deposit, the window moved by the Staged frame's first half
    P = split_parts()
    leftX_d = float(A["leftX"]) + float(run.MovingFrames[0]["shiftX"])
    k, f = window(leftX_d)
    wsum = float(d["weights"].abs().sum())
    e = 61.0 - np.ceil(np.log2(wsum))
    scale = torch.tensor([2.0 ** e, wsum], dtype=torch.float64, device=dev)
    acc = torch.zeros(nx * nr * nm * 3 * 2, dtype=torch.int64, device=dev)
    _lib.call("chm_sp_push_deposit_env", *P.ptrs(), P.n, k, f, 1.0 / dx, float(A["dr_inv"]),
              float(spc.Args["TimeStep"]), dx, nx, nr, nm, acc.data_ptr(), scale.data_ptr(),
              tab.data_ptr(), tab.numel(), kdx, st, None)
    spc.push_coords()
    J = fm.fortran_zeros((nx, nr, nm, 3))
    J = fm.dep_curr_env(d["coords_halfstep"], d["momenta"], d["weights"], J, leftX_d,
                        *A["DepProj"])
    a = acc.view(3, nm, nr, nx, 2).permute(3, 2, 1, 0, 4).cpu().numpy().astype(np.float64)
    Jsp = (a[..., 0] + 1j * a[..., 1]) / 2.0 ** e
    Jsp[:, 1] -= Jsp[:, 0]  # the ghost-row fold the FP64 deposit applies (fb_in's, split)
    Jsp[:, 0] = 0
    err_j = rel_l2(Jsp, J.cpu().numpy())
    to_f64(P)
    err_x = float((x64[0] - d["coords"][0]).abs().max()) / dx  # in x cells
    err_r = float((x64[1:] - d["coords"][1:]).abs().max()) * float(A["dr_inv"])  # in r cells
    print(f"envelope particle kernels: J {err_j:.2e}  x {err_x:.2e} cells  y, z {err_r:.2e} cells "
          f" kick {err_dp:.2e} of |E| dt (|EB| gathered {gathered:.3g})")
    assert np.abs(J.cpu().numpy()).max() > 0 and gathered > 0 and np.abs(dp_64).max() > 0
    assert err_j < 1e-5 and err_x < 1e-6 and err_r < 1e-6 and err_dp < 1e-6


@pytest.mark.parametrize("tap", [False, True])
def test_envelope_gather_mapped_undulator_matches_fp64(mods, tap):
    """The split gather + mapped undulator + Boris (und_kind 3, 4) against
    proj_fld_env + undul_mapped[_tap] + push_velocs on the small FEL beam
    after two steps: a map of step 0.35 periods (not a multiple of the grid's
    cell) over the beam, with a 10 % taper for undul_mapped_tap."""
    torch, _lib, fm, split = mods
    from chimera_gb300 import ChimeraRun, workloads
    run = ChimeraRun(workloads.fel_components("fel_small", seed=1004))
    for i in range(1, 3):
        run.make_step(i)
    S, spc = run.Solvers[0], run.Particles[0]
    A, d = S.Args, spc.Data
    nx, nr, nm = A["Nx"], A["Nr"], A["Mtot"]
    dev = torch.device("cuda")
    n = spc.num_particles
    dx = float(A["dx"])
    X0 = float(A["Xgrid"][0]) - 3 * dx
    st = _st(torch)
    tab = torch.zeros(nx + 4, dtype=torch.complex64, device=dev)
    s = (float(A["leftX"]) - X0) / dx
    k = int(np.floor(s))
    _lib.call("chm_sp_carrier", tab.data_ptr(), tab.numel(), float(A["kx0"]), X0, dx, k, st, None)
    # the map: a wiggler field of 1-period wavelength sampled every 0.35
    # periods, from 4 steps before the beam's head to 4 after its tail (the
    # particles near both ends fall in the map's skipped edge columns)
    xs = d["coords"][0]
    mdx = 0.35
    xleft = float(xs.min()) - 4 * mdx
    nmap = int(np.ceil((float(xs.max()) - xleft) / mdx)) + 4
    xc = xleft + mdx * np.arange(nmap)
    K0 = workloads.FEL["fel_small"].K0
    a0 = np.asfortranarray(np.stack([K0 * np.sin(2 * np.pi * xc), 0.7 * K0 * np.cos(2 * np.pi * xc)]))
    prm = np.zeros(5)
    if tap:
        prm[:5] = (1.0, xleft, mdx, 0.8 * nmap * mdx, 0.1)
    else:
        prm[:3] = (1.0, xleft, mdx)
    P = split._SpParticles(dev, n)
    P.append_f64(d["coords"], d["momenta"], d["weights"], X0, dx)
    EB32 = fm.fortran_empty(tuple(S.Data["EB"].shape), torch.complex64, dev)
    EB32.copy_(S.Data["EB"])
    p0 = d["momenta"].clone()
    amap = torch.from_numpy(np.ascontiguousarray(a0.T)).to(dev, torch.float32)
    dtq = spc.Args["push_fact"] * spc.Args["TimeStep"]
    _lib.call("chm_sp_gather_push_env", *P.ptrs(), P.n, k, s - k, float(A["dr_inv"]),
              EB32.data_ptr(), nx, nr, nm, float(dtq), tab.data_ptr(), tab.numel(),
              float(A["kx0"] * dx), 4 if tap else 3, prm.ctypes.data, amap.data_ptr(), nmap,
              X0, dx, st, None)
    spc.make_field()
    d["EB"] = fm.proj_fld_env(d["coords"], d["weights"], S.Data["EB"], d["EB"], A["leftX"],
                              *A["DepProj"])
    spc.Devices = ((fm.undul_mapped_tap if tap else fm.undul_mapped, a0, prm[:5 if tap else 3]),)
    spc.make_device(3)
    field = float(d["EB"].abs().max())
    spc.push_velocs()
    x64 = fm.fortran_zeros((3, n), torch.float64)
    p64 = fm.fortran_zeros((3, n), torch.float64)
    w64 = torch.zeros(n, dtype=torch.float64, device=dev)
    _lib.call("chm_sp_to_f64", *P.ptrs(), P.n, x64.data_ptr(), x64.stride(0), x64.stride(1),
              p64.data_ptr(), p64.stride(0), p64.stride(1), w64.data_ptr(), w64.stride(0), X0,
              dx, st)
    p0_32 = p0.to(torch.float32).to(torch.float64)
    dp_sp = (p64 - p0_32)[1:].cpu().numpy()
    dp_64 = (d["momenta"] - p0)[1:].cpu().numpy()
    err_dp = float(np.abs(dp_sp - dp_64).max()) / (field * abs(dtq))
    print(f"mapped undulator{' (tapered)' if tap else ''}: kick {err_dp:.2e} of |F| dt "
          f"(|F| {field:.3g}, {nmap} map columns)")
    assert field > 0 and np.abs(dp_64).max() > 0
    assert err_dp < 1e-6


def test_fel_split_steps_track_fp64(mods):
    """10 steps of the small FEL set-up in both forms from the same state:
    fields, beam momenta and positions, radiated energy."""
    torch, _lib, fm, split = mods
    from chimera_gb300 import ChimeraRun, workloads
    ref = ChimeraRun(workloads.fel_components("fel_small", seed=1004))
    run = split.SplitRun(workloads.fel_components("fel_small", seed=1004))
    assert run.env and run.undulators[0] is not None
    for i in range(1, 11):
        ref.make_step(i)
        run.make_step(i)
    e64 = _energy(torch, fm, ref.Solvers[0], ref.Solvers[0].Data["EG_fb"])
    e32 = _energy(torch, fm, run.solver, run.EG)
    run.to_fp64()
    s_ref, s_sp = ref.Solvers[0], run.solver
    err_eg = rel_l2(s_sp.Data["EG_fb"].cpu().numpy(), s_ref.Data["EG_fb"].cpu().numpy())
    err_eb = rel_l2(s_sp.Data["EB"].cpu().numpy(), s_ref.Data["EB"].cpu().numpy())
    o = run.order0[0].cpu().numpy()
    p_ref = ref.Particles[0].Data["momenta"].cpu().numpy()[:, o]
    p_sp = run.fp.Particles[0].Data["momenta"].cpu().numpy()
    p0 = ref.Particles[0].Data["momenta"].cpu().numpy()[:, o]
    err_p = rel_l2(p_sp, p_ref)
    # the transverse momenta (the undulator's wiggle), on their own
    err_pt = rel_l2(p_sp[1:], p_ref[1:])
    x_ref = ref.Particles[0].Data["coords"].cpu().numpy()[:, o]
    x_sp = run.fp.Particles[0].Data["coords"].cpu().numpy()
    print(f"FEL split vs fp64 after 10 steps: EG {err_eg:.2e} EB {err_eb:.2e} p {err_p:.2e} "
          f"p_perp {err_pt:.2e} x {np.abs(x_sp - x_ref).max():.2e} energy {e32:.6g} / {e64:.6g}")
    assert np.abs(p0[1:]).max() > 0
    assert err_eg < 1e-4 and err_eb < 1e-4 and err_p < 1e-6 and err_pt < 1e-4
    assert abs(e32 - e64) < 0.01 * abs(e64)
    assert _lib.load().chm_sp_umma_status() == 0


def test_fel_graph_step_equals_make_step(mods):
    torch, _lib, fm, split = mods
    from chimera_gb300 import workloads
    a = split.SplitRun(workloads.fel_components("fel_small", seed=1004))
    b = split.SplitRun(workloads.fel_components("fel_small", seed=1004))
    for i in range(1, 6):
        a.make_step(i)
        b.graph_step(i)
    torch.cuda.synchronize()
    assert b.graph_replays == 4
    assert a.solver.Args["leftX"] == b.solver.Args["leftX"]
    assert torch.equal(a.EG, b.EG) and torch.equal(a.EB, b.EB)
    for Pa, Pb in zip(a.parts, b.parts):
        for k in Pa.NAMES:
            assert torch.equal(Pa.buf[k][: Pa.n], Pb.buf[k][: Pb.n]), k


def test_fel_2400_steps_radiated_energy_within_1pct(mods):
    """The small FEL set-up through its 80-period undulator (2400 steps) in
    both forms: the radiated energy (EnergyFact-weighted |E|^2 summed, the
    quantity of Diagnostics.nrg_out, diagnostics.py:109-122) grows more than
    tenfold over the seed and the split form stays within 1 % of the FP64
    form along the run; the split steps replay from CUDA graphs."""
    torch, _lib, fm, split = mods
    from chimera_gb300 import ChimeraRun, workloads
    ref = ChimeraRun(workloads.fel_components("fel_small", seed=1004))
    run = split.SplitRun(workloads.fel_components("fel_small", seed=1004))
    S = ref.Solvers[0]
    e0 = _energy(torch, fm, S, S.Data["EG_fb"])
    worst, rows = 0.0, []
    for i in range(1, 2401):
        ref.make_step(i)
        run.graph_step(i)
        if i % 300 == 0:
            a, b = _energy(torch, fm, S, S.Data["EG_fb"]), _energy(torch, fm, run.solver, run.EG)
            worst = max(worst, abs(b - a) / abs(a))
            rows.append((i, a, b))
    for r in rows:
        print("step %d: radiated energy %.6e (fp64) %.6e (split)" % r)
    print(f"gain {rows[-1][1] / e0:.2f}, worst relative deviation {worst:.2e}")
    assert rows[-1][1] > 10 * e0
    assert worst < 0.01
    run.check_status()
