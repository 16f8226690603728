"""Drop-in ``Solver`` (the reference's moduls/solvers.py:26-779) on GB300.

The FP64 operator build (Bessel-zero DHT matrices, mode-coupling matrices,
PSATD coefficients, filters) runs once on the host in numpy, as in the
reference; every field array of ``Data`` is a torch CUDA tensor in Fortran
order and every per-step operation calls the CUDA kernels through
``chimera_gb300.fimera``.

``Args`` keeps the reference's numpy arrays under the reference's names.  The
argument packs the kernels are called with (``FBDiff``, ``DepProj``,
``FBCurrIn``, ``FBIn``, ``FBout``, ``FBoutFull``) hold device copies, so
``fimera.fb_vec_in(J_fb, J, leftX, *Args['FBCurrIn'])`` reads no host memory.

This module restates the reference's GPLv3-licensed Python layer
(hightower8083/chimera) statement by statement to keep its API as a
drop-in; it is a derivative of that code and is distributed under the GNU
General Public License, version 3 or later, as the reference is.
"""
from __future__ import annotations

import numpy as np
import torch
from numpy.linalg import inv
from scipy.constants import c, e, epsilon_0, m_e
from scipy.special import j1, jn, jn_zeros

from . import fimera as chimera
from .fimera import fortran_zeros
from .messages import msg

_DEV_KEYS = ("kx", "kx_env", "In", "InCurr", "Out", "OutFull", "DpS2S", "DmS2S", "Rgrid",
             "DepFact", "PoissFact")


def _dev_tensor(a, dtype=torch.float64, device=None):
    arr = np.asfortranarray(np.asarray(a), dtype={torch.float64: np.float64,
                                                  torch.complex128: np.complex128}[dtype])
    return torch.from_numpy(arr).to(device or "cuda")


def spectral_operators(args: dict, ext: int = 0):
    """Spectral r-grid and the DHT / coupling operators (solvers.py:717-759).

    Returns In, Out, DpS2S, DmS2S, w, kr, kr_g, kx_g, idxM with the mode axis
    last; envelope (KxShift) solvers store modes -M..M (plus `ext` extra on
    each side) in the order -M..-1, 0..M."""
    Nx, Nkr, Nko, lengthR = args["Nx"], args["Nkr"], args["Nko"], args["lengthR"]
    kx, RgridFull = args["kx"], args["RgridFull"]
    env = "KxShift" in args
    if env:
        mmin, mmax = -Nko - ext, Nko + ext
        mtot = 2 * Nko + 1 + 2 * ext
        mmin_x, mmax_x, mtot_x = mmin - 1, mmax + 1, mtot + 2
    else:
        mmin, mmax = 0, Nko + ext
        mtot = Nko + 1 + ext
        mmin_x, mmax_x, mtot_x = 0, mmax + 1, mtot + 1
    kr = np.zeros((Nkr, mtot_x))
    kr_g = np.zeros((Nx, Nkr, mtot))
    w = np.zeros((Nx, Nkr, mtot))
    Out = np.zeros((Nkr, Nkr, mtot))
    In = np.zeros((Nkr, Nkr, mtot))
    Dp = np.zeros((Nkr, Nkr, mtot))
    Dm = np.zeros((Nkr, Nkr, mtot))
    # negative mode indices wrap to the end of the arrays, as numpy indexing
    # does in the reference
    for m in range(mmin_x, mmax_x + 1):
        kr[:, m] = jn_zeros(m, Nkr) / lengthR
    r = RgridFull[1:, None]
    kx_g = None
    for m in range(mmin, mmax + 1):
        kr_g[:, :, m], kx_g = np.meshgrid(kr[:, m], kx)
        w[:, :, m] = np.sqrt(kx_g ** 2 + kr_g[:, :, m] ** 2)
        Out[:, :, m] = jn(m, r * kr[:, m][None, :])
        In[:, :, m] = inv(Out[:, :, m])
        Dp[:, :, m] = In[:, :, m].dot(0.5 * kr[:, m + 1][None, :] * jn(m, r * kr[:, m + 1][None, :]))
        Dm[:, :, m] = In[:, :, m].dot(0.5 * kr[:, abs(m - 1)][None, :]
                                      * jn(m, r * kr[:, abs(m - 1)][None, :]))
    if env and Nko > 0:
        def order(a):
            return np.concatenate((a[..., mmin:], a[..., :mmax + 1]), axis=-1)
        Out, In, Dp, Dm, w, kr_g, kr = (order(a) for a in (Out, In, Dp, Dm, w, kr_g, kr))
    idxM = np.arange(mmin, mmax + 1)
    return In, Out, Dp, Dm, w, kr, kr_g, kx_g, idxM


class Solver:
    """Quasi-cylindrical Fourier-Bessel PSATD field solver (solvers.py:26)."""

    def __init__(self, solver_in, msg=msg, device=None):
        self.device = torch.device(device or "cuda")
        A = self.Args = solver_in
        if "Features" not in A:
            A["Features"] = ()
        if "TimeActive" not in A:
            A["TimeInterval"] = (0.0, np.inf)
        A["Nko"] = A["MaxAzimuthMode"]
        A["leftX"], A["rightX"], A["lengthR"], A["dx"], A["dr"] = A["Grid"]
        A["dt"] = A["TimeStep"]
        A["dx_inv"], A["dr_inv"], A["dt_inv"] = 1.0 / A["dx"], 1.0 / A["dr"], 1.0 / A["dt"]

        # x-grid: an even node count (divisible by the chunk count)
        if "Xchunked" in A:
            A["nthrds"] = A["Xchunked"][0]
            A["Nxchunk"] = 2 * int(np.round(0.5 / A["nthrds"] / A["dx"] * (A["rightX"] - A["leftX"])))
            A["Nx"] = A["Nxchunk"] * A["nthrds"]
        else:
            A["Nx"] = int(2 * np.round(0.5 / A["dx"] * (A["rightX"] - A["leftX"])))
        A["Xgrid"] = A["rightX"] - A["dx"] * np.arange(A["Nx"])[::-1]
        A["leftX"] = A["Xgrid"][0]

        # spectral x-grid
        A["kx0"] = 2 * np.pi * A["KxShift"] if "KxShift" in A else 0.0
        A["kx_env"] = 2 * np.pi * np.fft.fftfreq(A["Nx"], A["dx"])
        A["kx"] = A["kx0"] + A["kx_env"]
        A["dkx"] = (A["kx"][1] - A["kx"][0]) / (2. * np.pi)

        # r-grid with the dr/2 offset (row 0 is the ghost at -dr/2)
        A["Nkr"] = int(np.round(A["lengthR"] / A["dr"]))
        A["Nr"] = A["Nkr"] + 1
        A["RgridFull"] = A["dr"] * (np.arange(A["Nr"]) - 0.5)
        A["lengthR"] = A["RgridFull"][-1] + A["dr"]

        _, _, A["DpS2S"], A["DmS2S"], _, _, _, _, _ = spectral_operators(A, ext=1)
        (A["InFull"], A["OutFull"], _, _, A["w"], A["kr"], A["kr_g"], A["kx_g"],
         A["idxM"]) = spectral_operators(A, ext=0)

        A["Mtot"] = A["InFull"].shape[-1]
        A["PoissFact"] = 1. / A["w"] ** 2
        VGrid = 2 * np.pi * A["dx"] * A["dr"] * A["RgridFull"]
        A["VGrid"] = (A["RgridFull"] > 0.0) / VGrid
        A["InCurr"] = A["InFull"] * A["VGrid"][None, 1:, None]

        msg.print_("sol/bounds", [A[k] for k in ("leftX", "rightX", "lengthR")])
        msg.print_("sol/resols", [A[k] for k in ("dx", "dr", "dt")])
        msg.print_("sol/actv", A["TimeInterval"])
        msg.print_("sol/grdsz", [A[k] for k in ("Nx", "Nkr", "Mtot")])
        if "KxShift" in A:
            msg.print_("sol/shift")

        if "Rcut" in A:
            ncut = int((A["RgridFull"] < A["Rcut"]).sum())
            A["Rgrid"] = A["RgridFull"][:ncut]
            A["In"] = A["InFull"][:, :ncut - 1]
            A["InCurr"] = A["InCurr"][:, :ncut - 1]
            A["Out"] = A["OutFull"][:ncut - 1]
            A["Rcut"] = A["Rgrid"].max()
            msg.print_("sol/rcut", (A["Rcut"], ncut))
        else:
            A["In"], A["Out"], A["Rgrid"] = A["InFull"], A["OutFull"], A["RgridFull"]
        A["Nr"] = A["Rgrid"].shape[0]
        A["lowerR"] = (A["Rgrid"] * (A["Rgrid"] >= 0)).min()
        A["upperR"] = A["Rgrid"].max()

        # energy integration factor (solvers.py:143-149)
        mabs = (np.abs(A["idxM"]) + 1)[None, None, :]
        A["EnergyFact"] = (0.5e-2 * (m_e * c ** 2 / e) ** 2 * (4 * np.pi * epsilon_0)
                           * A["lengthR"] ** 2 / A["dkx"] * jn(mabs, A["kr_g"] * A["lengthR"]) ** 2)
        if "KxShift" not in A:
            A["EnergyFact"] *= 0.5

        for k in ("DpS2S", "DmS2S", "InCurr", "In", "Out"):
            A[k] = np.swapaxes(A[k], 0, 1)
        for k in list(A.keys()):
            if isinstance(A[k], np.ndarray):
                A[k] = np.asfortranarray(A[k])

        # low-pass / anti-echo filter folded into DepFact (solvers.py:164-176)
        if "KxShift" in A:
            filt_x = self.antialias()
            kx_base = A["kx_env"]
        else:
            filt_x = np.cos(0.5 * A["dx"] * A["kx_g"])[:, :, None] ** 2
            kx_base = A["kx"]
        A["DepFact"] = np.asfortranarray((2 * np.pi) ** 2 / A["Nx"] * filt_x
                                         * np.cos(0.5 * A["dr"] * A["kr_g"]) ** 2)

        # device copies and the argument packs of the kernel calls
        dv = self.dev = {k: _dev_tensor(A[k], device=self.device) for k in _DEV_KEYS if k in A}
        dv["kx_base"] = _dev_tensor(kx_base, device=self.device)
        A["FBDiff"] = [dv["DpS2S"], dv["DmS2S"], dv["kx"]]
        A["DepProj"] = [dv["Rgrid"], A["dx_inv"], A["dr_inv"]]
        if "KxShift" in A:
            A["DepProj"] += (A["kx0"],)
        A["FBCurrIn"] = (dv["kx_base"], dv["InCurr"])
        A["FBIn"] = (dv["kx_base"], dv["In"])
        A["FBout"] = (dv["kx_base"], dv["Out"])
        A["FBoutFull"] = (dv["kx_base"], dv["OutFull"])

        # field data (Fortran-ordered complex128 on the device)
        D = self.Data = {}
        sp = (A["Nx"], A["Nr"], A["Mtot"])
        fb = (A["Nx"], A["Nkr"], A["Mtot"])
        z = lambda shape: fortran_zeros(shape, device=self.device)  # noqa: E731
        D["EB"] = z(sp + (6,))
        D["J"] = z(sp + (3,))
        D["scl_spc"] = z(sp)
        D["EG_fb"] = z(fb + (6,))
        D["vec_fb"] = z(fb + (3,))
        D["scl_fb"] = z(fb)
        D["J_fb"] = z(fb + (3,))
        D["B_fb"] = z(fb + (3,))
        if "SpaceCharge" in A["Features"] or "StaticKick" in A["Features"]:
            msg.print_("sol/spcchrg")
            D["Rho"] = z(sp)
            D["Rho_fb"] = z(fb)
            D["gradRho_fb_nxt"] = z(fb + (3,))
            D["gradRho_fb_prv"] = z(fb + (3,))
        if "StillAsBackground" in A["Features"]:
            msg.print_("sol/stillspcs")
            D["BckGrndRho"] = z(sp)

        if "CoPropagative" in A:
            self.PSATD_coeffs(A["CoPropagative"])
        else:
            self.PSATD_coeffs()
        if "NoPoissonCorrection" in A["Features"]:
            msg.print_("sol/pois")
        self.log = "\n".join(msg.log)

    # ------------------------------------------------------------------
    def PSATD_coeffs(self, beta=1.):
        """PSATD coefficients (solvers.py:227-279), built in FP64 on the host."""
        A = self.Args
        w = A["w"]
        kx_g = beta * A["kx_g"][:, :, None]
        dt = A["TimeStep"]
        if "SpaceCharge" in A["Features"]:
            CE = np.zeros(w.shape + (5,), dtype="double", order="F")
        elif "KxShift" in A:
            CE = np.zeros(w.shape + (3,), dtype="complex", order="F")
        else:
            CE = np.zeros(w.shape + (3,), dtype="double", order="F")
        CG = np.zeros_like(CE)
        cdw, sdw = np.cos(dt * w), np.sin(dt * w)
        CE[..., 0] = cdw
        CE[..., 1] = sdw / w
        CG[..., 0] = -w * sdw
        CG[..., 1] = cdw
        if "KxShift" in A:
            den = w ** 2 - kx_g ** 2
            ph = np.exp(-0.5j * kx_g * dt)
            CE[..., 2] = ph * 1j * kx_g / den * (1.0 - np.exp(1j * kx_g * dt)
                                                 * (w / (1j * kx_g) * sdw + cdw))
            CG[..., 2] = ph * w ** 2 / den * (1.0 + np.exp(1j * kx_g * dt)
                                              * (1j * kx_g / w * sdw - cdw))
        else:
            CE[..., 2] = -sdw / w
            CG[..., 2] = 1 - cdw
        if "SpaceCharge" in A["Features"]:
            CE[..., 3] = (dt * w * cdw - sdw) / w ** 3 / dt
            CE[..., 4] = (sdw - dt * w) / w ** 3 / dt
            CG[..., 3] = (1 - cdw - dt * w * sdw) / w ** 2 / dt
            CG[..., 4] = (cdw - 1) / w ** 2 / dt
        dtype = torch.complex128 if np.iscomplexobj(CE) else torch.float64
        self.Data["PSATD_E"] = _dev_tensor(CE, dtype, self.device)
        self.Data["PSATD_G"] = _dev_tensor(CG, dtype, self.device)

    # ------------------------------------------------------------------
    # per-step operations (thin wrappers over the CUDA kernels)
    # ------------------------------------------------------------------
    def maxwell_solver(self):
        """solvers.py:281-299"""
        D = self.Data
        if "SpaceCharge" in self.Args["Features"]:
            D["EG_fb"] = chimera.maxwell_push_with_spchrg(D["EG_fb"], D["J_fb"], D["gradRho_fb_prv"],
                                                          D["gradRho_fb_nxt"], D["PSATD_E"],
                                                          D["PSATD_G"])
        else:
            D["EG_fb"] = chimera.maxwell_push_wo_spchrg(D["EG_fb"], D["J_fb"], D["PSATD_E"],
                                                        D["PSATD_G"])

    def poiss_corr(self, poiss_corr_num=3):
        """solvers.py:301-331"""
        if "NoPoissonCorrection" in self.Args["Features"]:
            return
        D = self.Data
        for _ in range(poiss_corr_num):
            D["vec_fb"].copy_(D["J_fb"])
            self.FBGradDiv()
            if "SpaceCharge" in self.Args["Features"]:
                D["J_fb"] = chimera.poiss_corr(D["J_fb"], D["vec_fb"], D["gradRho_fb_prv"],
                                               D["gradRho_fb_nxt"], self.Args["dt_inv"],
                                               self.dev["PoissFact"])
            else:
                D["vec_fb"] = chimera.omp_mult_vec(D["vec_fb"], self.dev["PoissFact"])
                D["J_fb"] = chimera.omp_add_vec(D["J_fb"], D["vec_fb"])

    def _stat_coeffs(self, px0):
        A = self.Args
        beta0 = px0 / np.sqrt(1 + px0 ** 2)
        kx_g = beta0 * A["kx_g"][:, :, None]
        w = A["w"]
        den = w ** 2 - kx_g ** 2
        C1 = np.zeros(w.shape + (2,), dtype="complex", order="F")
        C2 = np.zeros_like(C1)
        C1[..., 0] = 1.j * kx_g / den
        C1[..., 1] = -1. / den
        C2[..., 0] = w ** 2 / den
        C2[..., 1] = 1.j * kx_g / den
        return C1, C2

    def maxwell_solver_stat(self, px0):
        """solvers.py:333-362 (static space-charge field)"""
        if "SpaceCharge" not in self.Args["Features"] and "StaticKick" not in self.Args["Features"]:
            return
        C1, C2 = self._stat_coeffs(px0)
        D = self.Data
        D["EG_fb"] = chimera.maxwell_init_push(D["EG_fb"], D["J_fb"], D["gradRho_fb_nxt"],
                                               _dev_tensor(C1, torch.complex128, self.device),
                                               _dev_tensor(C2, torch.complex128, self.device))

    def poiss_corr_stat(self, px0):
        """solvers.py:364-387"""
        if "NoPoissonCorrection" in self.Args["Features"]:
            return
        DT = -1.j * px0 / np.sqrt(1 + px0 ** 2) * self.Args["kx"]
        D = self.Data
        D["vec_fb"].copy_(D["J_fb"])
        self.FBGradDiv()
        D["J_fb"] = chimera.poiss_corr_stat(D["J_fb"], D["vec_fb"], D["gradRho_fb_nxt"],
                                            _dev_tensor(DT, torch.complex128, self.device),
                                            self.dev["PoissFact"])

    def field_drift(self, px0):
        """solvers.py:389-405"""
        self.Data["EG_fb"] = chimera.field_drift(self.Data["EG_fb"], self.dev["kx"],
                                                 px0 / np.sqrt(1 + px0 ** 2),
                                                 self.Args["TimeStep"])

    def fb_curr_in(self):
        """solvers.py:407-420; the DepFact multiply is fused into the transform."""
        D = self.Data
        D["J_fb"] = chimera._fb_in(D["J_fb"], D["J"], self.Args["leftX"], *self.Args["FBCurrIn"],
                                   3, fact=self.dev["DepFact"])

    def fb_dens_in(self):
        """solvers.py:422-435 (DepFact fused)"""
        D = self.Data
        D["Rho_fb"] = chimera._fb_in(D["Rho_fb"], D["Rho"], self.Args["leftX"],
                                     *self.Args["FBCurrIn"], 1, fact=self.dev["DepFact"])

    def fb_scl_spc_in(self):
        """solvers.py:437-448"""
        D = self.Data
        D["scl_fb"] = chimera.fb_scl_in(D["scl_fb"], D["scl_spc"], self.Args["leftX"],
                                        *self.Args["FBIn"])

    def fb_fld_out(self):
        """solvers.py:450-465 (eb_correction fused into the inverse transform)"""
        D = self.Data
        D["EB"] = chimera.fb_eb_out(D["EB"], D["EG_fb"], D["B_fb"], self.Args["leftX"],
                                    *self.Args["FBout"],
                                    eb_mode=2 if "KxShift" in self.Args else 1)

    def FBGrad(self):
        """solvers.py:467-482"""
        f = chimera.fb_grad_env if "KxShift" in self.Args else chimera.fb_grad
        self.Data["vec_fb"] = f(self.Data["vec_fb"], self.Data["scl_fb"], *self.Args["FBDiff"])

    def FBDiv(self):
        """solvers.py:484-499"""
        f = chimera.fb_div_env if "KxShift" in self.Args else chimera.fb_div
        self.Data["scl_fb"] = f(self.Data["scl_fb"], self.Data["vec_fb"], *self.Args["FBDiff"])

    def FBGradDiv(self):
        """solvers.py:501-515"""
        f = chimera.fb_graddiv_env if "KxShift" in self.Args else chimera.fb_graddiv
        self.Data["vec_fb"] = f(self.Data["vec_fb"], *self.Args["FBDiff"])

    def FBGradDens(self):
        """solvers.py:517-534"""
        f = chimera.fb_grad_env if "KxShift" in self.Args else chimera.fb_grad
        self.Data["gradRho_fb_nxt"] = f(self.Data["gradRho_fb_nxt"], self.Data["Rho_fb"],
                                        *self.Args["FBDiff"])

    def G2B_FBRot(self):
        """solvers.py:536-553: B from G = rot(B)"""
        f = chimera.fb_rot_env if "KxShift" in self.Args else chimera.fb_rot
        D = self.Data
        D["B_fb"] = f(D["B_fb"], D["EG_fb"][:, :, :, 3:], *self.Args["FBDiff"])
        D["B_fb"] = chimera.omp_mult_vec(D["B_fb"], self.dev["PoissFact"])

    def FBRot(self):
        """solvers.py:634-642"""
        f = chimera.fb_rot_env if "KxShift" in self.Args else chimera.fb_rot
        out = torch.empty_like(self.Data["vec_fb"])
        self.Data["vec_fb"] = f(out, self.Data["vec_fb"], *self.Args["FBDiff"])

    def B2G_FBRot(self):
        """solvers.py:652-658"""
        f = chimera.fb_rot_env if "KxShift" in self.Args else chimera.fb_rot
        D = self.Data
        f(D["EG_fb"][:, :, :, 3:], D["B_fb"], *self.Args["FBDiff"])

    def div_clean(self, vec):
        """solvers.py:644-650: vec + PoissFact * grad(div(vec))"""
        D = self.Data
        D["vec_fb"].copy_(vec)
        self.FBGradDiv()
        D["vec_fb"] = chimera.omp_mult_vec(D["vec_fb"], self.dev["PoissFact"])
        return chimera.omp_add_vec(vec, D["vec_fb"])

    def divG_clean(self):
        """solvers.py:761-767"""
        D = self.Data
        D["vec_fb"].copy_(D["EG_fb"][:, :, :, 3:])
        self.FBGradDiv()
        D["vec_fb"] = chimera.omp_mult_vec(D["vec_fb"], self.dev["PoissFact"])
        chimera.omp_add_vec(D["EG_fb"][:, :, :, 3:], D["vec_fb"])

    def test_calibration(self):
        """solvers.py:769-779: Gauss-law residuals div E - rho, div G, div B."""
        D = self.Data
        D["vec_fb"].copy_(D["EG_fb"][:, :, :, :3])
        self.FBDiv()
        t1 = (D["scl_fb"] - D["Rho_fb"]).clone()
        D["vec_fb"].copy_(D["EG_fb"][:, :, :, 3:])
        self.FBDiv()
        t2 = D["scl_fb"].clone()
        D["vec_fb"].copy_(D["B_fb"])
        self.FBDiv()
        t3 = D["scl_fb"].clone()
        return t1, t2, t3

    # ------------------------------------------------------------------
    # initialisation helpers
    # ------------------------------------------------------------------
    def add_gauss_beam(self, S):
        """Gaussian laser pulse added in spectral space (solvers.py:555-610)."""
        A, D = self.Args, self.Data
        k0 = 2 * np.pi * S["k0"]
        a0 = 2 * np.pi * S["a0"]
        Xf = S["x0"] - S["x_foc"]
        kx_g, kr_g, w = A["kx_g"], A["kr_g"], A["w"]
        w4 = w[:, :, :, None]
        vec = D["vec_fb"]
        if "KxShift" in A:
            Nko = A["Nko"]
            e_s0 = a0 * 0.5 * np.pi ** 0.5 * S["Lx"] * S["LR"] ** 2 * A["dkx"] / A["lengthR"] ** 2
            krm = kr_g[:, :, Nko]
            val = (e_s0 / j1(A["lengthR"] * krm) ** 2 * np.exp(-1j * kx_g * S["x0"])
                   * np.exp(-0.25 * (kx_g - k0) ** 2 * S["Lx"] ** 2 - 0.25 * krm ** 2 * S["LR"] ** 2))
            vec[:, :, Nko, 2] = torch.from_numpy(np.ascontiguousarray(val)).to(self.device)
            DT = -1.j * w4
        else:
            X, R = A["Xgrid"][:, None], A["Rgrid"][None, :]
            prof = (a0 * np.cos(k0 * (X - S["x0"])) * np.exp(-(X - S["x0"]) ** 2 / S["Lx"] ** 2
                                                             - R ** 2 / S["LR"] ** 2)
                    * (abs(R) < 3.5 * S["LR"]) * (abs(X - S["x0"]) < 3.5 * S["Lx"]))
            prof[:, 0] = 0.0
            D["scl_spc"][:, :, 0] = torch.from_numpy(prof.astype(np.complex128)).to(self.device)
            self.fb_scl_spc_in()
            vec[:, :, :, 2] = D["scl_fb"] / A["Nx"]
            DT = -1.j * w4 * np.sign(kx_g[:, :, None, None] + (kx_g[:, :, None, None] == 0))
        EE = chimera.fortran_empty(vec.shape, device=self.device)
        EE.copy_(vec)
        EE = self.div_clean(EE)
        to = lambda a: torch.from_numpy(np.ascontiguousarray(  # noqa: E731
            np.broadcast_to(a, vec.shape).astype(np.complex128))).to(self.device)
        DTd = to(DT)
        GG = DTd * EE
        cw, sw = to(np.cos(w4 * Xf)), to(np.sin(w4 * Xf))
        wd = to(w4)
        vec.copy_(cw * EE + sw / wd * GG)
        GG = -wd * sw * EE + cw * GG
        EE.copy_(vec)
        ph = to(np.exp(1.j * kx_g[:, :, None, None] * Xf))
        EE = EE * ph
        GG = GG * ph
        D["EG_fb"][:, :, :, :3] += EE
        D["EG_fb"][:, :, :, 3:] += GG
        vec.zero_()
        D["scl_fb"].zero_()

    def get_damp_profile(self, Lf):
        """solvers.py:612-617"""
        n = int(Lf)
        g = np.arange(n)
        return (g >= 0.75 * n) * (0.5 - 0.5 * np.cos(np.pi * (g - 0.75 * n) / (0.25 * n))) ** 2

    def damp_field(self, config="left", damp_b=False):
        """solvers.py:619-632: absorbing layer on E and G (or B)."""
        mode = {"left": 0, "right": 1, "both": 2}[config]
        A, D = self.Args, self.Data
        prof = A["damp_profile"]
        if not isinstance(prof, torch.Tensor):
            prof = A["damp_profile"] = _dev_tensor(prof, device=self.device)
        chimera.fb_filtr(D["EG_fb"][:, :, :, :3], A["leftX"], self.dev["kx"], prof, mode)
        if damp_b:
            chimera.fb_filtr(D["B_fb"], A["leftX"], self.dev["kx"], prof, mode)
            self.B2G_FBRot()
        else:
            chimera.fb_filtr(D["EG_fb"][:, :, :, 3:], A["leftX"], self.dev["kx"], prof, mode)

    def antialias(self):
        """Band-pass and numerical-echo filter of the envelope solver
        (solvers.py:660-715)."""
        A = self.Args
        kx_env, kx, kx0, Nx = A["kx_env"], A["kx"], A["kx0"], A["Nx"]
        cut = 0.85

        def bandpass(x):
            return (x < cut) + (x >= cut) * np.cos(np.pi / 2 * (x - cut) / (1 - cut)) ** 2

        filt_bp = bandpass(np.abs(kx_env) / np.abs(kx_env.max()))[:, None, None]
        filt_aa = np.ones_like(filt_bp)
        if "NoAntiEcho" not in A["Features"]:
            msg.print_("sol/echo_intro")
            ae = A["Features"]["AntiEchoStrength"] if "AntiEchoStrength" in A["Features"] else 2
            n_echo = int(np.abs(kx).max() / np.abs(kx_env).max()) + 1
            cell_echos = np.abs(kx_env).max() / kx0 * np.arange(n_echo) - 1.
            band = np.array([kx.min() / kx0, kx.max() / kx0]) - 1.

            def notch(x, x0, a):
                return 1 - np.exp(-(x - x0) ** 2 / (a * (x0 + 1.) / Nx) ** 2)

            idx = 0
            for order, ce in enumerate(cell_echos, start=1):
                if not (band[0] < ce < band[1]):
                    continue
                ech = ce / abs(band).max()
                line = "**** {0:d}-th grid echo at {1:.5g} ".format(order, ech)
                a_loc = ae[idx] if isinstance(ae, (list, tuple)) else ae
                idx += 1
                if abs(ce) / abs(band).max() < 0.4:
                    line += "(close to resonance) "
                if a_loc <= 0:
                    print(line + "no correction")
                    continue
                filt_aa = filt_aa * notch(kx / kx0 - 1, ce, a_loc)[:, None, None]
                print(line + "correcting with strength {0:g}".format(a_loc))
        return filt_aa * filt_bp

    def get_spectral_operators(self, ext=0):
        """solvers.py:717-759"""
        return spectral_operators(self.Args, ext)
