"""Accuracy of the split-precision form at the configurations' operator sizes.

Every split transform (tcgen05 split-BF16 products, FP32 FFT and epilogues)
against the FP64 kernels on the same complex64 inputs, on the operator sets
the solver builds (solvers.py:717-759) for the three laser-wakefield grids:
Nx=512 / Nkr=64 / 2 modes, Nx=2048 / Nkr=256 / 2 modes and Nx=4096 / Nkr=512
/ 3 modes.  The gate is TOL_T relative L2 per transform.  Also: the bare
tensor-core product against an FP64 product up to K = N = 512, and the
tensor-core kernel's bounded waits (a wait that runs out is reported and the
kernel frees its tensor memory)."""
import ctypes as C

import numpy as np
import pytest

from conftest import rel_l2

pytestmark = pytest.mark.gpu
TOL_T = 1e-6      # per transform (FP32 data, split-BF16 products)
TOL_GEMM = 4e-7   # the bare product, random data

GRIDS = {  # name: (nx, nkr, MaxAzimuthMode, dx, dr)
    "lwfa_512x64_m2": (512, 64, 1, 0.04, 0.4),
    "lwfa_2048x256_m2": (2048, 256, 1, 0.04, 0.4),
    "lwfa_4096x512_m3": (4096, 512, 2, 0.04, 0.4),
}


@pytest.fixture(scope="module")
def mods(cuda):
    import torch
    from chimera_gb300 import _lib, fimera, split
    return torch, _lib, fimera, split


def _st(torch):
    return torch.cuda.current_stream().cuda_stream


def _gemm(torch, _lib, ops, mode, A, engine=1):
    M, K = A.shape
    At = torch.from_numpy(np.ascontiguousarray(A.T)).cuda().t()
    Ct = torch.zeros((ops.N, M), dtype=torch.float32, device="cuda").t()  # (M, N) column-major
    ws = torch.empty(_lib.query("chm_sp_gemm_ws_bytes", M, K, 1), dtype=torch.uint8, device="cuda")
    _lib.call("chm_sp_gemm", Ct.data_ptr(), At.data_ptr(), C.addressof(ops), mode, M, engine,
              ws.data_ptr(), ws.numel(), _st(torch))
    torch.cuda.synchronize()
    return Ct.cpu().numpy()


@pytest.mark.parametrize("K,N", [(64, 64), (256, 256), (512, 512), (513, 200), (96, 40)])
def test_tensor_core_gemm_accuracy(mods, K, N):
    torch, _lib, fm, split = mods
    rng = np.random.default_rng(K * 7 + N)
    B = np.asfortranarray(rng.standard_normal((K, N, 1)))
    A = rng.standard_normal((1024, K)).astype(np.float32)
    ops, buf, d = split._prepare_ops(B, torch.device("cuda"))
    got = _gemm(torch, _lib, ops, 0, A)
    err = rel_l2(got, A.astype(np.float64) @ B[:, :, 0])
    print(f"tensor-core product K={K} N={N}: rel L2 {err:.2e}")
    assert err < TOL_GEMM
    assert _lib.load().chm_sp_umma_status() == 0


def test_tensor_core_wait_limit_reports_and_recovers(mods):
    """With a pipeline wait limit of 0 every wait gives up at once: the
    kernel reports it (chm_sp_umma_status), writes nothing and frees its
    tensor memory, so the next launch at the default limit runs normally."""
    torch, _lib, fm, split = mods
    lib = _lib.load()
    rng = np.random.default_rng(3)
    B = np.asfortranarray(rng.standard_normal((256, 128, 1)))
    A = rng.standard_normal((512, 256)).astype(np.float32)
    ops, buf, d = split._prepare_ops(B, torch.device("cuda"))
    assert lib.chm_sp_umma_status() == 0
    prev = lib.chm_sp_set_umma_spin_limit(0)
    try:
        got = _gemm(torch, _lib, ops, 0, A)
    finally:
        lib.chm_sp_set_umma_spin_limit(prev)
    assert lib.chm_sp_umma_status() != 0
    assert not np.any(got)  # the CTAs that gave up wrote nothing
    assert lib.chm_sp_umma_status() == 0  # read and reset
    got = _gemm(torch, _lib, ops, 0, A)
    assert rel_l2(got, A.astype(np.float64) @ B[:, :, 0]) < TOL_GEMM
    assert lib.chm_sp_umma_status() == 0


def _c(a, torch):
    return torch.from_numpy(np.asfortranarray(a)).cuda()


def _rand(shape, seed):
    rng = np.random.default_rng(seed)
    return np.asfortranarray(rng.standard_normal(shape) + 1j * rng.standard_normal(shape))


@pytest.fixture(scope="module", params=list(GRIDS))
def grid(request, mods):
    torch, _lib, fm, split = mods
    from chimera_gb300 import Solver
    from chimera_gb300.messages import msg
    msg.quiet = True
    nx, nkr, mx, dx, dr = GRIDS[request.param]
    S = Solver({"Grid": (0.0, nx * dx, nkr * dr, dx, dr), "TimeStep": dx, "MaxAzimuthMode": mx,
                "Features": ("SpaceCharge",)})
    A = S.Args
    dev = torch.device("cuda")
    ops = {k: split._prepare_ops(A[key], dev) for k, key in
           (("InCurr", "InCurr"), ("Out", "Out"), ("Dp", "DpS2S"), ("Dm", "DmS2S"))}
    nr, nm = A["Nr"], A["Mtot"]
    ws = torch.empty(_lib.query("chm_sp_fb_ws_bytes", nx, nr, nkr, nm), dtype=torch.uint8,
                     device=dev)
    yield request.param, S, ops, ws, (nx, nr, nkr, nm)
    del ops, ws
    torch.cuda.empty_cache()


def test_split_transforms_at_config_sizes(mods, grid):
    """fb_in (from the deposit accumulators, with DepFact), fb_grad, the
    3-iteration Poisson correction, curl + PoissFact and fb_eb_out with
    eb_correction, each within TOL_T of the FP64 kernels."""
    torch, _lib, fm, split = mods
    name, S, o, ws, (nx, nr, nkr, nm) = grid
    A = S.Args
    st = _st(torch)
    kx64 = _c(A["kx"], torch)
    kx32 = kx64.to(torch.float32)
    pf = A["PoissFact"]
    pf32 = _c(pf.astype(np.float32), torch)
    errs = {}
    # fb_in of a 64-bit fixed-point deposit accumulator (scale 2^40)
    rng = np.random.default_rng(9)
    scale = 2.0 ** 40
    acc = np.zeros((2, nx, nr, nm, 3), np.int64, order="F")
    acc[...] = (rng.standard_normal(acc.shape) * 2.0 ** 40).astype(np.int64)
    accd = torch.from_numpy(np.ravel(acc, order="F").copy()).cuda()
    scd = torch.tensor([scale, 1.0], dtype=torch.float64, device="cuda")
    depf = _c(A["DepFact"].astype(np.float32), torch)
    leftX = float(A["leftX"]) + 3.3
    Jfb = fm.fortran_zeros((nx, nkr, nm, 3), torch.complex64)
    _lib.call("chm_sp_fb_in_acc", Jfb.data_ptr(), accd.data_ptr(), scd.data_ptr(), None, None,
              leftX, kx64.data_ptr(), C.addressof(o["InCurr"][0]), depf.data_ptr(), nx, nr, nkr, nm,
              3, ws.data_ptr(), ws.numel(), st, None)
    Jsp = (acc[0] + 1j * acc[1]) / scale
    Jsp[:, 1] -= Jsp[:, 0]  # the ghost-row fold of the deposit
    Jsp[:, 0] = 0
    ref = fm._fb_in(fm.fortran_zeros((nx, nkr, nm, 3)), _c(Jsp, torch), leftX,
                    *A["FBCurrIn"], 3, fact=S.dev["DepFact"])
    errs["fb_in"] = rel_l2(Jfb.cpu().numpy(), ref.cpu().numpy())
    del accd, Jfb, ref
    # fb_grad
    s = _rand((nx, nkr, nm), 1).astype(np.complex64)
    sd = _c(s, torch)
    out = fm.fortran_zeros((nx, nkr, nm, 3), torch.complex64)
    _lib.call("chm_sp_fb_grad", out.data_ptr(), sd.data_ptr(), C.addressof(o["Dp"][0]),
              C.addressof(o["Dm"][0]), kx32.data_ptr(), nx, nkr, nm, ws.data_ptr(), ws.numel(), st)
    ref = fm.fb_grad(fm.fortran_zeros((nx, nkr, nm, 3)), _c(s.astype(np.complex128), torch),
                     A["DpS2S"], A["DmS2S"], A["kx"])
    errs["fb_grad"] = rel_l2(out.cpu().numpy(), ref.cpu().numpy())
    del sd, out, ref
    # Poisson correction (3 x graddiv + poiss_corr)
    J = _rand((nx, nkr, nm, 3), 2).astype(np.complex64)
    gp = (0.1 * _rand((nx, nkr, nm, 3), 3)).astype(np.complex64)
    gn = (0.1 * _rand((nx, nkr, nm, 3), 4)).astype(np.complex64)
    Js, gpd, gnd = _c(J, torch), _c(gp, torch), _c(gn, torch)
    _lib.call("chm_sp_poisson", Js.data_ptr(), gpd.data_ptr(), gnd.data_ptr(), pf32.data_ptr(),
              10.0, C.addressof(o["Dp"][0]), C.addressof(o["Dm"][0]), kx32.data_ptr(), nx, nkr, nm,
              3, 1, ws.data_ptr(), ws.numel(), st)
    Jd = _c(J.astype(np.complex128), torch)
    gp64, gn64 = _c(gp.astype(np.complex128), torch), _c(gn.astype(np.complex128), torch)
    for _ in range(3):
        v = Jd.clone(memory_format=torch.preserve_format)
        v = fm.fb_graddiv(v, A["DpS2S"], A["DmS2S"], A["kx"])
        Jd = fm.poiss_corr(Jd, v, gp64, gn64, 10.0, pf)
    errs["poisson"] = rel_l2(Js.cpu().numpy(), Jd.cpu().numpy())
    del Js, gpd, gnd, Jd, gp64, gn64, v
    # B = rot(G) * PoissFact
    G = _rand((nx, nkr, nm, 3), 5).astype(np.complex64)
    Gd = _c(G, torch)
    Bs = fm.fortran_zeros((nx, nkr, nm, 3), torch.complex64)
    _lib.call("chm_sp_rot_b", Bs.data_ptr(), Gd.data_ptr(), pf32.data_ptr(),
              C.addressof(o["Dp"][0]), C.addressof(o["Dm"][0]), kx32.data_ptr(), nx, nkr, nm,
              ws.data_ptr(), ws.numel(), st)
    Bd = fm.fb_rot(fm.fortran_zeros((nx, nkr, nm, 3)), _c(G.astype(np.complex128), torch),
                   A["DpS2S"], A["DmS2S"], A["kx"])
    Bd = fm.omp_mult_vec(Bd, pf)
    errs["rot_b"] = rel_l2(Bs.cpu().numpy(), Bd.cpu().numpy())
    del Gd, Bs, Bd
    # fb_eb_out with eb_correction
    E = _rand((nx, nkr, nm, 6), 6).astype(np.complex64)
    Bq = _rand((nx, nkr, nm, 3), 7).astype(np.complex64)
    Ed, Bqd = _c(E, torch), _c(Bq, torch)
    EBs = fm.fortran_zeros((nx, nr, nm, 6), torch.complex64)
    _lib.call("chm_sp_fb_eb_out", EBs.data_ptr(), Ed.data_ptr(), Bqd.data_ptr(), leftX,
              kx64.data_ptr(), C.addressof(o["Out"][0]), nx, nr, nkr, nm, ws.data_ptr(), ws.numel(),
              st, None)
    EBd = fm.fb_eb_out(fm.fortran_zeros((nx, nr, nm, 6)), _c(E.astype(np.complex128), torch),
                       _c(Bq.astype(np.complex128), torch), leftX, A["kx"], A["Out"], eb_mode=1)
    errs["fb_eb_out"] = rel_l2(EBs.cpu().numpy(), EBd.cpu().numpy())
    print(f"{name}: " + " ".join(f"{k} {v:.2e}" for k, v in errs.items()))
    assert max(errs.values()) < TOL_T, errs
    assert _lib.load().chm_sp_umma_status() == 0


def _split_outputs(torch, _lib, fm, S, o, ws, dims):
    """fb_in (factor epilogue), the Poisson correction (shift epilogue) and
    fb_eb_out (stored products) of fixed random inputs."""
    nx, nr, nkr, nm = dims
    A = S.Args
    st = _st(torch)
    kx64 = _c(A["kx"], torch)
    kx32 = kx64.to(torch.float32)
    pf32 = _c(A["PoissFact"].astype(np.float32), torch)
    rng = np.random.default_rng(19)
    acc = (rng.standard_normal(2 * nx * nr * nm * 3) * 2.0 ** 40).astype(np.int64)
    accd = torch.from_numpy(acc).cuda()
    scd = torch.tensor([2.0 ** 40, 1.0], dtype=torch.float64, device="cuda")
    depf = _c(A["DepFact"].astype(np.float32), torch)
    Jfb = fm.fortran_zeros((nx, nkr, nm, 3), torch.complex64)
    _lib.call("chm_sp_fb_in_acc", Jfb.data_ptr(), accd.data_ptr(), scd.data_ptr(), None, None,
              float(A["leftX"]) + 1.7, kx64.data_ptr(), C.addressof(o["InCurr"][0]),
              depf.data_ptr(), nx, nr, nkr, nm, 3, ws.data_ptr(), ws.numel(), st, None)
    Js = _c(_rand((nx, nkr, nm, 3), 12).astype(np.complex64), torch)
    gp = _c((0.1 * _rand((nx, nkr, nm, 3), 13)).astype(np.complex64), torch)
    gn = _c((0.1 * _rand((nx, nkr, nm, 3), 14)).astype(np.complex64), torch)
    _lib.call("chm_sp_poisson", Js.data_ptr(), gp.data_ptr(), gn.data_ptr(), pf32.data_ptr(),
              10.0, C.addressof(o["Dp"][0]), C.addressof(o["Dm"][0]), kx32.data_ptr(), nx, nkr, nm,
              3, 1, ws.data_ptr(), ws.numel(), st)
    E = _c(_rand((nx, nkr, nm, 6), 15).astype(np.complex64), torch)
    Bq = _c(_rand((nx, nkr, nm, 3), 16).astype(np.complex64), torch)
    EB = fm.fortran_zeros((nx, nr, nm, 6), torch.complex64)
    _lib.call("chm_sp_fb_eb_out", EB.data_ptr(), E.data_ptr(), Bq.data_ptr(), float(A["leftX"]),
              kx64.data_ptr(), C.addressof(o["Out"][0]), nx, nr, nkr, nm, ws.data_ptr(), ws.numel(),
              st, None)
    torch.cuda.synchronize()
    return [Jfb.cpu(), Js.cpu(), EB.cpu()]


def test_column_tile_widths_change_no_bit(mods, grid):
    """The tensor-core products give the same bits at every column-tile
    width, so the tuner's choice changes only the speed: the default width,
    64 and 32 columns forced, and the tuned widths, on the three epilogues at
    the configurations' operator sizes.  The tuner records one width per
    shape, a candidate (a multiple of 16, 32 and up)."""
    torch, _lib, fm, split = mods
    name, S, o, ws, dims = grid
    lib = _lib.load()
    prev = lib.chm_sp_set_umma_cols(0)
    try:
        ref = _split_outputs(torch, _lib, fm, S, o, ws, dims)
        for mode in (64, 32, -1):
            lib.chm_sp_set_umma_cols(mode)
            if mode < 0:
                lib.chm_sp_umma_tune_reset()
            got = _split_outputs(torch, _lib, fm, S, o, ws, dims)
            for r, g in zip(ref, got):
                assert torch.equal(r, g), (name, mode)
        n = lib.chm_sp_umma_tuned(None, 0)
        buf = (C.c_int32 * (6 * max(n, 1)))()
        assert lib.chm_sp_umma_tuned(buf, n) == n > 0
        recs = np.array(buf[: 6 * n]).reshape(n, 6)
        print(f"{name}: tuned (M, N, K, count, epilogue, width):", recs.tolist())
        assert np.all(recs[:, 5] % 16 == 0) and np.all(recs[:, 5] >= 16)
        assert np.all(recs[:, 5] <= 128)
    finally:
        lib.chm_sp_set_umma_cols(prev)
    assert lib.chm_sp_umma_status() == 0
