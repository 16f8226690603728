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
TOL_T = 2e-6   # per transform, FP32 data and FP32-accumulated split products


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
        assert err < 2e-6, (engine, err)
    assert _lib.load().chm_sp_umma_status() == 0


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
              ws.numel(), st)
    EBd = fm.fb_eb_out(fm.fortran_zeros((nx, nr, nm, 6)), _c(E.astype(np.complex128), torch),
                       _c(Bq.astype(np.complex128), torch), leftX, g["kx"], g["Out"], eb_mode=1)
    assert rel_l2(EBs.cpu().numpy(), EBd.cpu().numpy()) < TOL_T


def _lpa_comps(seed, xchunked=False):
    from chimera_gb300 import Solver, Specie
    from chimera_gb300.messages import msg
    msg.quiet = True
    np.random.seed(seed)
    dx, dr = 0.1, 0.25
    solver = Solver({"Grid": (-6.0, 0.4, 4.0, dx, dr), "TimeStep": dx, "MaxAzimuthMode": 1,
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


@pytest.mark.parametrize("nsteps", [1, 6])
def test_split_steps_track_fp64_form(mods, nsteps):
    torch, _lib, fm, split = mods
    from chimera_gb300 import ChimeraRun
    ref = ChimeraRun(_lpa_comps(1001))
    run = split.SplitRun(_lpa_comps(1001))
    for i in range(1, nsteps + 1):
        ref.make_step(i)
        run.make_step(i)
    run.to_fp64()
    s_ref, s_sp = ref.Solvers[0], run.solver
    err_eg = rel_l2(s_sp.Data["EG_fb"].cpu().numpy(), s_ref.Data["EG_fb"].cpu().numpy())
    err_eb = rel_l2(s_sp.Data["EB"].cpu().numpy(), s_ref.Data["EB"].cpu().numpy())
    p_ref = ref.Particles[0].Data["momenta"].cpu().numpy()
    p_sp = run.fp.Particles[0].Data["momenta"].cpu().numpy()
    err_p = rel_l2(p_sp, p_ref)
    x_ref = ref.Particles[0].Data["coords"].cpu().numpy()
    x_sp = run.fp.Particles[0].Data["coords"].cpu().numpy()
    print(f"split vs fp64 after {nsteps} steps: EG {err_eg:.2e} EB {err_eb:.2e} "
          f"p {err_p:.2e} x {np.abs(x_sp - x_ref).max():.2e}")
    assert err_eg < 1e-4 and err_eb < 1e-4 and err_p < 1e-4
    a0_ref = s_ref.Data["EB"][:, 1, 0, 2].real.max().item()
    a0_sp = s_sp.Data["EB"][:, 1, 0, 2].real.max().item()
    assert abs(a0_sp - a0_ref) < 0.01 * abs(a0_ref)
    assert _lib.load().chm_sp_umma_status() == 0
