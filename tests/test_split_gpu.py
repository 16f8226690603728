"""Split-precision form on the GPU: the tcgen05 split-BF16 GEMM, every split
transform against the FP64 kernels on the same inputs (target: <= 1e-6
relative L2 per transform, stated as TOL_T), and whole steps against the FP64
form (fields within 1e-4 relative L2 after 6 steps, laser a0 / wake within
1 %)."""
import ctypes as C
from copy import deepcopy

import numpy as np
import pytest

from conftest import rel_l2

pytestmark = pytest.mark.gpu
TOL_T = 1e-6   # per transform, FP32 data and split-BF16 products


@pytest.fixture(scope="module")
def mods(cuda):
    import torch
    from chimera_gb300 import _lib, fimera, split
    return torch, _lib, fimera, split


def _st(torch):
    return torch.cuda.current_stream().cuda_stream


@pytest.mark.parametrize("M,K,N", [(128, 32, 16), (256, 64, 64), (512, 256, 256), (200, 70, 40)])
def test_tensor_core_gemm_matches_fp64(mods, M, K, N):
    torch, _lib, fimera, split = mods
    rng = np.random.default_rng(M + K + N)
    B = np.asfortranarray(rng.standard_normal((K, N, 1)))
    A = np.asfortranarray(rng.standard_normal((M, K)).astype(np.float32))
    ops, buf, d = split._prepare_ops(B, torch.device("cuda"))
    At = torch.from_numpy(A).cuda() if A.flags.c_contiguous else torch.from_numpy(np.ascontiguousarray(A.T)).cuda().t()
    ref = A.astype(np.float64) @ B[:, :, 0]
    ws = torch.empty(_lib.query("chm_sp_gemm_ws_bytes", M, K, 1), dtype=torch.uint8, device="cuda")
    for engine in (1, 0):
        Ct = torch.zeros((N, M), dtype=torch.float32, device="cuda").t()  # (M, N) column-major
        _lib.call("chm_sp_gemm", Ct.data_ptr(), At.data_ptr(), C.addressof(ops), 0, M, engine,
                  ws.data_ptr(), ws.numel(), _st(torch))
        torch.cuda.synchronize()
        err = rel_l2(Ct.cpu().numpy(), ref)
        assert err < 1e-6, (engine, err)
    assert _lib.load().chm_sp_umma_status() == 0
    assert _lib.load().chm_sp_deposit_dropped() == 0  # every deposit cell inside its box


def _ops(golden, name):
    return {k.split("/")[-1]: golden[k] for k in golden.files if k.startswith(f"op/{name}/Args/")}


def _c(a, torch):
    return torch.from_numpy(np.asfortranarray(a)).cuda()


def _rand(shape, seed):
    rng = np.random.default_rng(seed)
    return np.asfortranarray(rng.standard_normal(shape) + 1j * rng.standard_normal(shape))


@pytest.fixture(scope="module")
def lpa(mods, golden):
    """The plain LPA operators (Nx=64, Nkr=16, 2 modes) prepared for the split form."""
    torch, _lib, fimera, split = mods
    g = _ops(golden, "lpa_m2")
    dev = torch.device("cuda")
    o = {k: split._prepare_ops(g[key], dev) for k, key in
         (("InCurr", "InCurr"), ("Out", "Out"), ("Dp", "DpS2S"), ("Dm", "DmS2S"))}
    nx, nr, nkr, nm = int(g["Nx"]), int(g["Nr"]), int(g["Nkr"]), int(g["Mtot"])
    ws = torch.empty(_lib.query("chm_sp_fb_ws_bytes", nx, nr, nkr, nm), dtype=torch.uint8,
                     device=dev)
    return g, o, ws, (nx, nr, nkr, nm)


def test_split_spectral_operators_match_fp64(mods, lpa):
    torch, _lib, fm, split = mods
    g, o, ws, (nx, nr, nkr, nm) = lpa
    st = _st(torch)
    kx64 = _c(g["kx"], torch)
    kx32 = kx64.to(torch.float32)
    pf = g["PoissFact"]
    pf32 = _c(pf.astype(np.float32), torch)
    # fb_grad
    # (every device input is bound to a name: a temporary's memory could be
    # handed to the next allocation before the asynchronous kernel reads it)
    s = _rand((nx, nkr, nm), 1).astype(np.complex64)
    sd = _c(s, torch)
    out = fm.fortran_zeros((nx, nkr, nm, 3), torch.complex64)
    _lib.call("chm_sp_fb_grad", out.data_ptr(), sd.data_ptr(), C.addressof(o["Dp"][0]),
              C.addressof(o["Dm"][0]), kx32.data_ptr(), nx, nkr, nm, ws.data_ptr(), ws.numel(), st)
    ref = fm.fb_grad(fm.fortran_zeros((nx, nkr, nm, 3)), _c(s.astype(np.complex128), torch),
                     g["DpS2S"], g["DmS2S"], g["kx"])
    assert rel_l2(out.cpu().numpy(), ref.cpu().numpy()) < TOL_T
    # Poisson correction (3 x graddiv + poiss_corr)
    J = _rand((nx, nkr, nm, 3), 2).astype(np.complex64)
    gp = (0.1 * _rand((nx, nkr, nm, 3), 3)).astype(np.complex64)
    gn = (0.1 * _rand((nx, nkr, nm, 3), 4)).astype(np.complex64)
    Js = _c(J, torch)
    gpd, gnd = _c(gp, torch), _c(gn, torch)
    _lib.call("chm_sp_poisson", Js.data_ptr(), gpd.data_ptr(), gnd.data_ptr(),
              pf32.data_ptr(), 10.0, C.addressof(o["Dp"][0]), C.addressof(o["Dm"][0]),
              kx32.data_ptr(), nx, nkr, nm, 3, 1, ws.data_ptr(), ws.numel(), st)
    Jd = _c(J.astype(np.complex128), torch)
    for _ in range(3):
        v = Jd.clone(memory_format=torch.preserve_format)
        v = fm.fb_graddiv(v, g["DpS2S"], g["DmS2S"], g["kx"])
        Jd = fm.poiss_corr(Jd, v, _c(gp.astype(np.complex128), torch),
                           _c(gn.astype(np.complex128), torch), 10.0, pf)
    assert rel_l2(Js.cpu().numpy(), Jd.cpu().numpy()) < TOL_T
    # B = rot(G) PoissFact
    G = _rand((nx, nkr, nm, 3), 5).astype(np.complex64)
    Bs = fm.fortran_zeros((nx, nkr, nm, 3), torch.complex64)
    Gd = _c(G, torch)
    _lib.call("chm_sp_rot_b", Bs.data_ptr(), Gd.data_ptr(), pf32.data_ptr(),
              C.addressof(o["Dp"][0]), C.addressof(o["Dm"][0]), kx32.data_ptr(), nx, nkr, nm,
              ws.data_ptr(), ws.numel(), st)
    Bd = fm.fb_rot(fm.fortran_zeros((nx, nkr, nm, 3)), _c(G.astype(np.complex128), torch),
                   g["DpS2S"], g["DmS2S"], g["kx"])
    Bd = fm.omp_mult_vec(Bd, pf)
    assert rel_l2(Bs.cpu().numpy(), Bd.cpu().numpy()) < TOL_T
    # EB out with eb_correction
    E = _rand((nx, nkr, nm, 6), 6).astype(np.complex64)
    Bq = _rand((nx, nkr, nm, 3), 7).astype(np.complex64)
    EBs = fm.fortran_zeros((nx, nr, nm, 6), torch.complex64)
    leftX = float(g["leftX"]) + 3.3
    Ed, Bqd = _c(E, torch), _c(Bq, torch)
    _lib.call("chm_sp_fb_eb_out", EBs.data_ptr(), Ed.data_ptr(), Bqd.data_ptr(),
              leftX, kx64.data_ptr(), C.addressof(o["Out"][0]), nx, nr, nkr, nm, ws.data_ptr(),
              ws.numel(), st, None)
    EBd = fm.fb_eb_out(fm.fortran_zeros((nx, nr, nm, 6)), _c(E.astype(np.complex128), torch),
                       _c(Bq.astype(np.complex128), torch), leftX, g["kx"], g["Out"], eb_mode=1)
    assert rel_l2(EBs.cpu().numpy(), EBd.cpu().numpy()) < TOL_T


@pytest.mark.parametrize("space_charge", [1, 0])
def test_poisson_with_fused_psatd_equals_two_calls(mods, lpa, space_charge):
    """chm_sp_poisson_psatd (PSATD fused into the correction's last J
    update) gives bitwise the J and E/G of chm_sp_poisson + chm_sp_psatd."""
    torch, _lib, fm, split = mods
    g, o, ws, (nx, nr, nkr, nm) = lpa
    st = _st(torch)
    kx32 = _c(g["kx"], torch).to(torch.float32)
    pf32 = _c(g["PoissFact"].astype(np.float32), torch)
    nterm = 5 if space_charge else 3
    rng = np.random.default_rng(8)
    c1 = _c(rng.standard_normal((nx, nkr, nm, nterm)).astype(np.float32), torch)
    c2 = _c(rng.standard_normal((nx, nkr, nm, nterm)).astype(np.float32), torch)
    J0 = _c(_rand((nx, nkr, nm, 3), 2).astype(np.complex64), torch)
    EG0 = _c(_rand((nx, nkr, nm, 6), 3).astype(np.complex64), torch)
    gp = _c((0.1 * _rand((nx, nkr, nm, 3), 4)).astype(np.complex64), torch)
    gn = _c((0.1 * _rand((nx, nkr, nm, 3), 5)).astype(np.complex64), torch)
    sc_args = (gp.data_ptr(), gn.data_ptr()) if space_charge else (None, None)
    Ja, EGa = J0.clone(memory_format=torch.preserve_format), EG0.clone(memory_format=torch.preserve_format)
    _lib.call("chm_sp_poisson", Ja.data_ptr(), *sc_args, pf32.data_ptr(), 10.0,
              C.addressof(o["Dp"][0]), C.addressof(o["Dm"][0]), kx32.data_ptr(), nx, nkr, nm, 3,
              space_charge, ws.data_ptr(), ws.numel(), st)
    _lib.call("chm_sp_psatd", EGa.data_ptr(), Ja.data_ptr(), *sc_args, c1.data_ptr(),
              c2.data_ptr(), nterm, nx * nkr * nm, st)
    Jb, EGb = J0.clone(memory_format=torch.preserve_format), EG0.clone(memory_format=torch.preserve_format)
    _lib.call("chm_sp_poisson_psatd", Jb.data_ptr(), *sc_args, pf32.data_ptr(), 10.0,
              C.addressof(o["Dp"][0]), C.addressof(o["Dm"][0]), kx32.data_ptr(), nx, nkr, nm, 3,
              space_charge, EGb.data_ptr(), c1.data_ptr(), c2.data_ptr(), nterm, ws.data_ptr(),
              ws.numel(), st)
    torch.cuda.synchronize()
    assert torch.equal(Ja, Jb) and torch.equal(EGa, EGb)
    assert not torch.equal(EGa, EG0)


def _lpa_comps(seed, xchunked=False, max_mode=1):
    from chimera_gb300 import Solver, Specie
    from chimera_gb300.messages import msg
    msg.quiet = True
    np.random.seed(seed)
    dx, dr = 0.1, 0.25
    solver = Solver({"Grid": (-6.0, 0.4, 4.0, dx, dr), "TimeStep": dx, "MaxAzimuthMode": max_mode,
                     "Features": ("SpaceCharge", "StillAsBackground")})
    solver.add_gauss_beam({"a0": 1.0, "k0": 1.0, "x0": -2.5, "x_foc": 2.0, "Lx": 1.5, "LR": 2.5})
    el_in = {"Grid": (-6.0, 0.4, 4.0, dx, dr), "TimeStep": dx, "Density": 0.02,
             "FixedCell": (2, 2, 2), "Features": ()}
    io_in = deepcopy(el_in)
    io_in["Charge"], io_in["Mass"], io_in["Features"] = 1.0, 1836.0, ("Still",)
    el, io = Specie(el_in), Specie(io_in)
    prof = lambda x: np.interp(x, [-4.0, -3.0, 10.0], [0.0, 1.0, 1.0])  # noqa: E731
    parts = el.gen_parts(Domain=(-5.5, 0.3, 0.0, 3.5), ProfileFunc=prof)
    el.add_particles(*[p.copy() for p in parts])
    parts[-1] *= -1
    io.add_particles(*parts)
    return {"Solvers": (solver,), "Particles": (el, io),
            "MovingFrames": ({"TimeStep": dx, "Steps": 1, "Velocity": 1.0},)}


@pytest.mark.parametrize("nsteps,max_mode", [(1, 1), (6, 1), (6, 2)])
def test_split_steps_track_fp64_form(mods, nsteps, max_mode):
    """max_mode 2: three stored modes (the cell-run kernels' NM = 3 forms)."""
    torch, _lib, fm, split = mods
    from chimera_gb300 import ChimeraRun
    ref = ChimeraRun(_lpa_comps(1001, max_mode=max_mode))
    run = split.SplitRun(_lpa_comps(1001, max_mode=max_mode))
    for i in range(1, nsteps + 1):
        ref.make_step(i)
        run.make_step(i)
    run.to_fp64()
    s_ref, s_sp = ref.Solvers[0], run.solver
    err_eg = rel_l2(s_sp.Data["EG_fb"].cpu().numpy(), s_ref.Data["EG_fb"].cpu().numpy())
    err_eb = rel_l2(s_sp.Data["EB"].cpu().numpy(), s_ref.Data["EB"].cpu().numpy())
    # the split form stores each generation cell's particles in deposit-cell
    # order; compare in that order
    o = run.order0[0].cpu().numpy()
    p_ref = ref.Particles[0].Data["momenta"].cpu().numpy()[:, o]
    p_sp = run.fp.Particles[0].Data["momenta"].cpu().numpy()
    err_p = rel_l2(p_sp, p_ref)
    x_ref = ref.Particles[0].Data["coords"].cpu().numpy()[:, o]
    x_sp = run.fp.Particles[0].Data["coords"].cpu().numpy()
    print(f"split vs fp64 after {nsteps} steps: EG {err_eg:.2e} EB {err_eb:.2e} "
          f"p {err_p:.2e} x {np.abs(x_sp - x_ref).max():.2e}")
    assert err_eg < 1e-4 and err_eb < 1e-4 and err_p < 1e-4
    a0_ref = s_ref.Data["EB"][:, 1, 0, 2].real.max().item()
    a0_sp = s_sp.Data["EB"][:, 1, 0, 2].real.max().item()
    assert abs(a0_sp - a0_ref) < 0.01 * abs(a0_ref)
    assert _lib.load().chm_sp_umma_status() == 0
    assert _lib.load().chm_sp_deposit_dropped() == 0  # every deposit cell inside its box


def _sp_particles(torch, n, nx, nr, dr, seed, runs=True):
    """Split-layout particles: runs of 8 in one cell (as generated cell by
    cell) or fully random positions; thermal momenta; a few zero weights."""
    rng = np.random.default_rng(seed)
    if runs:
        ncell = (n + 7) // 8
        cx = rng.integers(-2, nx + 1, ncell).repeat(8)[:n]
        cr = rng.integers(0, nr - 1, ncell).repeat(8)[:n]
        fx = (rng.integers(0, 4, n) + 0.5) / 4.0
        r = (cr + (rng.integers(0, 2, n) + 0.25) / 2.0) * dr
    else:
        cx = rng.integers(-2, nx + 1, n)
        fx = rng.random(n)
        r = rng.random(n) * (nr - 1) * dr
    th = rng.random(n) * 2 * np.pi
    cols = {"ix": cx.astype(np.int32) + 100, "fx": fx.astype(np.float32),
            "y": (r * np.cos(th)).astype(np.float32), "z": (r * np.sin(th)).astype(np.float32),
            "px": (0.05 * rng.standard_normal(n)).astype(np.float32),
            "py": (0.05 * rng.standard_normal(n)).astype(np.float32),
            "pz": (0.05 * rng.standard_normal(n)).astype(np.float32),
            "w": (1e-3 * (0.5 + rng.random(n))).astype(np.float32)}
    cols["w"][rng.random(n) < 0.01] = 0.0
    # tile layout: particle i at slot chm_sp_slot(i) of arrays of whole tiles
    cap = (n + 511) // 512 * 512
    slot = _slots(n)
    out = {}
    for k, v in cols.items():
        a = np.zeros(cap, dtype=v.dtype)
        a[slot] = v
        out[k] = torch.from_numpy(a).cuda()
    return out


def _slots(n):
    """chm_sp_slot(i) for i < n (the tile layout of the split form)."""
    i = np.arange(n, dtype=np.int64)
    return (i & ~511) | ((i & 15) << 5) | ((i >> 4) & 31)


def _gather(a, n):
    """particle-order values 0 .. n-1 of a tile-layout array"""
    return a[_slots(n)]


@pytest.mark.parametrize("nm,runs,push", [(2, True, 1), (2, False, 1), (1, True, 1), (2, True, 0),
                                          (3, True, 1), (3, False, 1), (3, True, 0)])
def test_cell_run_deposit_equals_generic_kernel(mods, nm, runs, push):
    """The cell-run push/deposit kernel (nm 1..3) and the per-particle kernel
    agree (accumulators within 1e-6 relative L2, same pushed positions)."""
    torch, _lib, fm, split = mods
    nx, nr, dr, n = 64, 32, 0.5, 40000 + 37
    P0 = _sp_particles(torch, n, nx, nr, dr, 7 + nm, runs)
    names = ("ix", "fx", "y", "z", "px", "py", "pz", "w")
    st = _st(torch)
    sws = torch.empty(_lib.query("chm_sp_scale_ws_bytes"), dtype=torch.uint8, device="cuda")
    scale = torch.zeros(2, dtype=torch.float64, device="cuda")
    _lib.call("chm_sp_weight_scale", scale.data_ptr(), P0["w"].data_ptr(), n, sws.data_ptr(),
              sws.numel(), st)
    out = {}
    for variant in ("run", "generic"):
        entry = "chm_sp_push_deposit" + ("_generic" if variant == "generic" else "")
        P = {k: v.clone() for k, v in P0.items()}
        accJ = torch.zeros(nx * nr * nm * 3 * 2, dtype=torch.int64, device="cuda")
        accR = torch.zeros(nx * nr * nm * 2, dtype=torch.int64, device="cuda")
        _lib.call(entry, *[P[k].data_ptr() for k in names], n, 100, 0.25,
                  1 / 0.1, 1 / dr, 0.1, nx, nr, nm, push,
                  accJ.data_ptr() if push else None, scale.data_ptr() if push else None,
                  accR.data_ptr(), scale.data_ptr(), st, None)
        torch.cuda.synchronize()
        out[variant] = (accJ.cpu().numpy(), accR.cpu().numpy(),
                        {k: P[k].cpu().numpy() for k in names})
    a, b = out["run"], out["generic"]
    # the run kernel sums a run's values in FP32 before rounding them to the
    # block's 32-bit quantum (2^-30 of a bound of the block's summed |values|);
    # the generic kernel rounds every particle.  With random momenta (little
    # current per node against the bound) the two differ by ~1e-6.
    for u, v, tol in ((a[0], b[0], 1e-5), (a[1], b[1], 1e-6)):
        assert rel_l2(u.astype(np.float64), v.astype(np.float64)) < tol
    assert np.abs(a[1]).sum() > 0 and (not push or np.abs(a[0]).sum() > 0)
    xa = a[2]["ix"] + a[2]["fx"].astype(np.float64)
    xb = b[2]["ix"] + b[2]["fx"].astype(np.float64)
    assert np.abs(xa - xb).max() < 1e-5
    for k in ("y", "z", "px", "py", "pz", "w"):
        assert np.allclose(a[2][k], b[2][k], rtol=1e-6, atol=1e-7), k


def test_absorb_and_compact(mods):
    """chm_sp_absorb marks exactly the particles outside the box and returns
    the scale of the survivors; compaction keeps the live ones in order."""
    torch, _lib, fm, split = mods
    n, nx, nr, dr = 30011, 64, 32, 0.5
    P = _sp_particles(torch, n, nx, nr, dr, 3, runs=False)
    names = ("ix", "fx", "y", "z", "px", "py", "pz", "w")
    ref = {k: _gather(v.cpu().numpy(), n) for k, v in P.items()}
    cap = P["w"].numel()
    dead = torch.zeros(cap, dtype=torch.uint8, device="cuda")
    dead[torch.from_numpy(_slots(50)).cuda()] = 1  # already dead: stay dead, not counted again
    cnt = torch.zeros(2, dtype=torch.int64, device="cuda")
    st = _st(torch)
    k, f, xmin, xmax, r2 = 100, 0.25, 8.0, 60.0, (12.0 * dr) ** 2
    scale = torch.zeros(2, dtype=torch.float64, device="cuda")
    sws = torch.empty(_lib.query("chm_sp_scale_ws_bytes"), dtype=torch.uint8, device="cuda")
    _lib.call("chm_sp_absorb", P["ix"].data_ptr(), P["fx"].data_ptr(), P["y"].data_ptr(),
              P["z"].data_ptr(), P["w"].data_ptr(), dead.data_ptr(), n, k, f, xmin, xmax, r2,
              cnt.data_ptr(), scale.data_ptr(), sws.data_ptr(), sws.numel(), st)
    _lib.call("chm_sp_count_live", cnt.data_ptr(), n, st)
    xc = (ref["ix"] - k).astype(np.float32) + (ref["fx"] - np.float32(f))
    r2p = ref["y"] * ref["y"] + ref["z"] * ref["z"]
    out_box = ~((xc >= xmin) & (xc <= xmax) & (r2p <= np.float32(r2)))
    dead_ref = out_box.copy()
    dead_ref[:50] = True
    newly = out_box.copy()
    newly[:50] = False
    torch.cuda.synchronize()
    assert np.array_equal(_gather(dead.cpu().numpy(), n).astype(bool), dead_ref)
    assert int(cnt[0]) == int(newly.sum())
    assert int(cnt[1]) == n - int(newly.sum())
    w = _gather(P["w"].cpu().numpy(), n)
    assert np.all(w[newly] == 0) and np.array_equal(w[~dead_ref], ref["w"][~dead_ref])
    # the same pass gives the deposit scale of the surviving weights
    B = float(np.abs(w.astype(np.float64)).sum())
    sc = scale.cpu().numpy()
    assert abs(sc[1] - B) <= 1e-6 * B
    assert sc[0] == 2.0 ** (61 - int(np.ceil(np.log2(sc[1]))))
    Q = {k: torch.empty_like(v) for k, v in P.items()}
    ws = torch.empty(_lib.query("chm_sp_compact_ws_bytes", n), dtype=torch.uint8, device="cuda")
    n_out = torch.zeros(1, dtype=torch.int64, device="cuda")
    _lib.call("chm_sp_compact", *[P[k].data_ptr() for k in names], dead.data_ptr(), n,
              *[Q[k].data_ptr() for k in names], n_out.data_ptr(), ws.data_ptr(), ws.numel(), st)
    torch.cuda.synchronize()
    m = int(n_out.item())
    assert m == int((~dead_ref).sum())
    for key in names:
        exp = (ref[key] if key != "w" else w)[~dead_ref]
        assert np.array_equal(_gather(Q[key].cpu().numpy(), m), exp), key


def _logical(q):
    q = np.asarray(q, dtype=np.int64)
    return (q & ~511) | ((q & 31) << 4) | ((q >> 5) & 15)


def test_sort_by_cell_matches_host(mods):
    """chm_sp_sort_cells: the stable order of the documented deposit-cell key
    (host restatement with the same FP32 arithmetic), dead particles dropped,
    the live count returned, every particle moved whole."""
    torch, _lib, fm, split = mods
    n, nx, nr, dr = 70000 + 123, 96, 40, 0.5
    P = _sp_particles(torch, n, nx, nr, dr, 21, runs=False)
    names = ("ix", "fx", "y", "z", "px", "py", "pz", "w")
    cap = P["w"].numel()
    rng = np.random.default_rng(4)
    dead_h = np.zeros(cap, np.uint8)
    dead_h[_slots(n)[rng.random(n) < 0.05]] = 1
    dead = torch.from_numpy(dead_h).cuda()
    win_k, win_f = 100, np.float32(0.375)
    st = _st(torch)
    Q = {k: torch.full_like(v, 7) for k, v in P.items()}
    ws = torch.empty(_lib.query("chm_sp_sort_ws_bytes", n), dtype=torch.uint8, device="cuda")
    n_out = torch.zeros(1, dtype=torch.int64, device="cuda")
    _lib.call("chm_sp_sort_cells", *[P[k].data_ptr() for k in names], dead.data_ptr(), n, win_k,
              float(win_f), nx, nr, np.float32(1 / dr), *[Q[k].data_ptr() for k in names],
              n_out.data_ptr(),
              ws.data_ptr(), ws.numel(), st)
    torch.cuda.synchronize()
    h = {k: v.cpu().numpy() for k, v in P.items()}
    q = np.arange(cap)
    live = (_logical(q) < n) & (dead_h == 0)
    f32 = np.float32
    y, z = h["y"], h["z"]
    sv = np.sqrt(y * y + z * z).astype(f32) * f32(1 / dr)
    grf = np.floor(sv)
    fr = (sv - grf).astype(f32)
    half = (fr >= f32(0.5)).astype(np.uint64)
    dxf = (h["fx"] - win_f).astype(f32)
    sx = (dxf - np.floor(dxf)).astype(f32)
    sr = np.where(half == 1, fr - f32(0.5), fr + f32(0.5)).astype(f32)
    qx = np.minimum(3, np.floor(sx * f32(4)).astype(np.int64)).astype(np.uint64)
    qr = np.minimum(3, np.floor(sr * f32(4)).astype(np.int64)).astype(np.uint64)
    gr = np.minimum(np.maximum(grf.astype(np.int64), 0), nr + 4).astype(np.uint64)
    gx = np.minimum(np.maximum(h["ix"].astype(np.int64) - win_k + 8, 0), nx + 24).astype(np.uint64)
    npx = np.uint64((nx + 24) // 4 + 1)
    px, lx, pr, lr = gx >> 2, gx & 3, gr >> 2, gr & 3
    pxs = np.where(pr & 1, npx - 1 - px, px)
    lxs = np.where(lr & 1, 3 - lx, lx)
    key = ((((((pr * npx + pxs) * 4 + lr) * 4 + lxs) * 2 + half) << 4) | (qx << 2) | qr)
    key = np.where(live, key, 0xffffffff).astype(np.uint64)
    order = np.argsort(key, kind="stable")
    nlive = int(live.sum())
    assert int(n_out.item()) == nlive
    src = order[:nlive]  # source slots in sorted order
    for k in names:
        got = _gather(Q[k].cpu().numpy(), nlive)
        assert np.array_equal(got, h[k][src]), k
    assert np.all(np.diff(key[src].astype(np.int64)) >= 0)


def test_tile_slot_map(mods):
    """chm_sp_slot / chm_sp_capacity follow the documented tile layout."""
    torch, _lib, fm, split = mods
    lib = _lib.load()
    for i in (0, 1, 15, 16, 31, 511, 512, 513, 10**6 + 7):
        assert lib.chm_sp_slot(i) == int(_slots(i + 1)[-1])
    assert lib.chm_sp_capacity(1) == 512 and lib.chm_sp_capacity(513) == 1024
    assert sorted(_slots(1024)) == list(range(1024))


def _window_comps(seed):
    comps = _lpa_comps(seed)
    dx = 0.1
    prof = lambda x: np.interp(x, [-4.0, -3.0, 10.0], [0.0, 1.0, 1.0])  # noqa: E731
    comps["MovingFrames"] = ({"TimeStep": dx, "Steps": 1, "Velocity": 1.0, "AbsorbLayer": 6,
                              "AddPlasma": prof, "Features": ("IonsOnTop",)},)
    return comps


@pytest.mark.parametrize("sort_every", [64, 2])
def test_split_window_with_injection_tracks_fp64_form(mods, sort_every):
    """Moving window with absorption and plasma injection (the demos'
    AbsorbLayer + AddPlasma + IonsOnTop): same particle counts as the FP64
    form and fields within 1e-4 after 8 steps, with compactions in between
    (and re-sorts by deposit cell every 2 steps)."""
    torch, _lib, fm, split = mods
    from chimera_gb300 import ChimeraRun
    ref = ChimeraRun(_window_comps(2024))
    run = split.SplitRun(_window_comps(2024))
    run.compact_every = 3
    run.sort_every = sort_every
    live = 0
    for i in range(1, 9):
        np.random.seed(500 + i)  # the same injected plasma in both runs
        ref.make_step(i)
        np.random.seed(500 + i)
        run.make_step(i)
        live += ref.Particles[0].num_particles
    assert run.live_particle_steps() == live
    run.to_fp64()
    for s_ref, s_sp in ((ref.Particles[0], run.fp.Particles[0]), (ref.Particles[1], run.fp.Particles[1])):
        assert s_sp.num_particles == s_ref.num_particles
    err = rel_l2(run.solver.Data["EG_fb"].cpu().numpy(), ref.Solvers[0].Data["EG_fb"].cpu().numpy())
    assert err < 1e-4, err
    assert _lib.load().chm_sp_umma_status() == 0
    assert _lib.load().chm_sp_deposit_dropped() == 0  # every deposit cell inside its box


@pytest.mark.parametrize("nm,runs", [(2, True), (2, False), (1, True), (3, True), (3, False)])
def test_cell_run_gather_matches_generic_kernel(mods, nm, runs):
    """Cell-run gather + Boris (nm 1..3) against the per-particle kernel."""
    torch, _lib, fm, split = mods
    nx, nr, dr, n = 64, 32, 0.5, 40000 + 37
    P0 = _sp_particles(torch, n, nx, nr, dr, 11 + nm, runs)
    names = ("ix", "fx", "y", "z", "px", "py", "pz", "w")
    rng = np.random.default_rng(5)
    eb = np.asfortranarray((rng.standard_normal((nx, nr, nm, 6)) +
                            1j * rng.standard_normal((nx, nr, nm, 6))).astype(np.complex64))
    ebd = torch.from_numpy(eb).cuda()
    out = {}
    for variant in ("run", "generic"):
        entry = "chm_sp_gather_push" + ("_generic" if variant == "generic" else "")
        P = {k: v.clone() for k, v in P0.items()}
        _lib.call(entry, *[P[k].data_ptr() for k in names], n, 100, 0.25, 1 / dr,
                  ebd.data_ptr(), nx, nr, nm, 0.05, _st(torch), None)
        torch.cuda.synchronize()
        out[variant] = np.stack([P[k].cpu().numpy() for k in ("px", "py", "pz")])
    p0 = np.stack([P0[k].cpu().numpy() for k in ("px", "py", "pz")])
    assert np.abs(out["run"] - p0).max() > 1e-3  # the fields did push
    assert np.abs(out["run"] - out["generic"]).max() <= 1e-6 * np.abs(out["generic"]).max()


def test_batched_instances_match_single_runs(mods):
    """Instances advanced together on separate streams give bitwise the
    fields and particles they give when advanced alone."""
    torch, _lib, fm, split = mods
    from chimera_gb300.batched import BatchedRun, draw_instances, lwfa_instance
    from chimera_gb300.messages import msg
    msg.quiet = True
    params = [dict(p, nx=min(p["nx"], 256), nr=min(p["nr"], 32)) for p in draw_instances(3, 7)]
    batch = BatchedRun([lwfa_instance(**p) for p in params])
    for i in range(1, 4):
        batch.make_step(i)
    batch.synchronize()
    for p, run in zip(params, batch.runs):
        alone = split.SplitRun(lwfa_instance(**p))
        for i in range(1, 4):
            alone.make_step(i)
        torch.cuda.synchronize()
        assert torch.equal(alone.EG, run.EG) and torch.equal(alone.EB, run.EB)
        for Pa, Pb in zip(alone.parts, run.parts):
            assert Pa.n == Pb.n
            for k in Pa.NAMES:
                assert torch.equal(Pa.buf[k][: Pa.n], Pb.buf[k][: Pb.n]), k
    assert batch.num_moving == sum(r.num_moving for r in batch.runs) > 0
    assert _lib.load().chm_sp_umma_status() == 0
    assert _lib.load().chm_sp_deposit_dropped() == 0  # every deposit cell inside its box


def test_graph_step_equals_make_step(mods):
    """SplitRun.graph_step (the step's kernels replayed from a CUDA graph,
    re-captured after each re-sort) gives bitwise the fields and particles of
    make_step."""
    torch, _lib, fm, split = mods
    runs = [split.SplitRun(_lpa_comps(1001)), split.SplitRun(_lpa_comps(1001))]
    for r in runs:
        r.sort_every = 3
    for i in range(1, 8):
        runs[0].make_step(i)
        runs[1].graph_step(i)
    torch.cuda.synchronize()
    a, b = runs
    # (the first step runs eagerly; the others replay graphs)
    assert b.graph_captures >= 2 and b.graph_replays == 6 and b.graph_launches > 10
    assert a.solver.Args["leftX"] == b.solver.Args["leftX"]
    assert torch.equal(a.EG, b.EG) and torch.equal(a.EB, b.EB)
    for Pa, Pb in zip(a.parts, b.parts):
        assert Pa.n == Pb.n
        for k in Pa.NAMES:
            assert torch.equal(Pa.buf[k][: Pa.n], Pb.buf[k][: Pb.n]), k
    b.check_status()


def test_batched_graph_step_matches_single_runs(mods):
    """BatchedRun.graph_step (every instance's step in one CUDA graph) gives
    bitwise what each instance gives alone."""
    torch, _lib, fm, split = mods
    from chimera_gb300.batched import BatchedRun, draw_instances, lwfa_instance
    from chimera_gb300.messages import msg
    msg.quiet = True
    params = [dict(p, nx=min(p["nx"], 256), nr=min(p["nr"], 32)) for p in draw_instances(3, 9)]
    batch = BatchedRun([lwfa_instance(**p) for p in params])
    for i in range(1, 5):
        batch.graph_step(i)
    batch.synchronize()
    assert batch.graph_captures == 2  # even and odd steps (the gradient buffers swap)
    for p, run in zip(params, batch.runs):
        alone = split.SplitRun(lwfa_instance(**p))
        for i in range(1, 5):
            alone.make_step(i)
        torch.cuda.synchronize()
        assert torch.equal(alone.EG, run.EG) and torch.equal(alone.EB, run.EB)
        for Pa, Pb in zip(alone.parts, run.parts):
            for k in Pa.NAMES:
                assert torch.equal(Pa.buf[k][: Pa.n], Pb.buf[k][: Pb.n]), k


@pytest.mark.parametrize("spreads,with_profile", [((0.0, 0.0, 0.0), True), ((0.1, 0.05, 0.05), False)])
def test_device_plasma_generation_matches_host(mods, spreads, with_profile):
    """Specie.gen_parts_device (chm_gen_fixed_cell) against the host
    generator gen_parts (particle_tools.f90:84-128, species.py:132-215) from
    the same RNG state: the same random numbers consumed, x, weights and
    momenta bitwise, y and z to the device's FP64 cos/sin."""
    torch, _lib, fm, split = mods
    from chimera_gb300 import Specie
    from chimera_gb300.messages import msg
    msg.quiet = True
    prof = (lambda x: np.interp(x, [-3.0, -1.0, 9.0], [0.0, 1.0, 1.0])) if with_profile else None
    sp = Specie({"Grid": (-3.0, 1.0, 2.0, 0.1, 0.25), "TimeStep": 0.1, "Density": 0.01,
                 "FixedCell": (2, 2, 3), "MomentaSpreads": spreads})
    np.random.seed(11)
    hc, hp, hw = sp.gen_parts(Xsteps=3, ProfileFunc=prof)
    st_h = np.random.get_state()
    np.random.seed(11)
    dc, dp, dw = (t.cpu().numpy() for t in sp.gen_parts_device(Xsteps=3, ProfileFunc=prof))
    st_d = np.random.get_state()
    assert np.array_equal(st_h[1], st_d[1]) and st_h[2] == st_d[2]  # same RNG stream
    assert dc.shape == hc.shape and dc.shape[1] > 0
    assert np.array_equal(dc[0], hc[0])
    assert np.abs(dc[1:] - hc[1:]).max() <= 1e-14 * np.abs(hc[1:]).max()
    assert np.array_equal(dw, hw)
    assert np.array_equal(dp, hp)


def test_background_moves_with_whole_cell_windows(mods):
    """With a window moving one cell per step (dt = dx at c) the still
    ions' background density is moved with the window and only the entering
    column deposited (chm_sp_deposit_background shift mode): bitwise the full
    re-deposit of every move, through re-sorts (a full deposit after each)
    and graph replay."""
    torch, _lib, fm, split = mods
    from chimera_gb300 import workloads
    runs = [split.SplitRun(workloads.components("cfg1", "none", seed=1001)) for _ in range(2)]
    runs[1].bg_shift = False
    for r in runs:
        r.sort_every = 5
    shifted = 0
    for i in range(1, 13):
        runs[0].graph_step(i)
        runs[1].graph_step(i)
        torch.cuda.synchronize()
        shifted += runs[0]._bg_plan(i + 1) > 0
        assert torch.equal(runs[0].accBG, runs[1].accBG), i
    assert shifted >= 6
    assert torch.equal(runs[0].EG, runs[1].EG) and torch.equal(runs[0].EB, runs[1].EB)
    for r in runs:
        r.check_status()
