"""CPU PIC step driver over the oracle kernels -- TEST INFRASTRUCTURE.

Restates the control flow of the reference's ``ChimeraRun.make_step``
(moduls/chimera_main.py:82-318) and the ``Solver`` / ``Specie`` wrappers it
calls (moduls/solvers.py:281-553, moduls/species.py:279-398) on numpy arrays,
with every kernel taken from the oracle (oracle/chimera_oracle.c).  It is
used (a) as the CPU baseline of bench.py (the reference's Fortran cannot be
built on either machine) and (b) by tests, where it is checked against the
golden runs of the reference's own step loop.

Supported subset (what the benchmark and the golden runs use): one plain
(non-envelope) solver with or without SpaceCharge / StillAsBackground /
NoPoissonCorrection, Still and moving species, FixedCell plasma, a moving
window with optional AbsorbLayer / AddPlasma / IonsOnTop, serial or
x-chunked deposition.  The FP64 operators come from the host-side operator
build (a Solver constructed on the CPU), which is itself pinned to the
reference's solvers.py by the golden operator fixtures.
"""
from __future__ import annotations

import numpy as np

from . import oracle as orc


def _f(a, dtype=np.float64):
    return np.asfortranarray(np.asarray(a), dtype=dtype)


class CpuSpecies:
    def __init__(self, specie):
        """specie: a chimera_gb300 Specie built on the CPU (its Args, generator
        and particles are copied to numpy)."""
        self.sp = specie
        self.Args = specie.Args
        d = specie.Data
        self.Data = {k: _f(d[k].cpu().numpy()) for k in ("coords", "coords_halfstep", "momenta",
                                                          "weights", "EB")}
        self.chunks = None

    @property
    def still(self):
        return "Still" in self.Args["Features"]

    def n(self):
        return self.Data["coords"].shape[1]

    def add(self, coords, momenta, weights):
        D = self.Data
        D["coords"] = _f(np.hstack([D["coords"], coords]))
        D["coords_halfstep"] = _f(np.hstack([D["coords_halfstep"], coords]))
        D["momenta"] = _f(np.hstack([D["momenta"], momenta]))
        D["weights"] = _f(np.concatenate([D["weights"], weights]))

    def chunk_and_damp(self, wind=None, SimDom=None, position="stag"):
        """species.py:351-398"""
        if self.n() == 0:
            return
        A = self.Args
        comp = {"cntr": "coords_halfstep", "stag": "coords"}
        if wind is None:
            wind = {"Features": (), "AbsorbLayer": 0.0}
        if SimDom is None:
            SimDom = _f([A["leftX"] + wind["AbsorbLayer"] * A["dx"], A["rightX"], 0.0,
                         A["upperR"] ** 2])
        if "Xchunked" in A and "NoSorting" not in wind["Features"]:
            ids, self.chunks, go = orc.chunk_coords_boundaries(self.Data[comp[position]], SimDom,
                                                               A["Xgrid"], A["Xchunked"][0])
            keep = np.argsort(ids, kind="stable")[go:]
        else:
            idx, num = orc.sortpartsout(self.Data["coords"], SimDom)
            keep = idx[:num]
        for k in ("coords", "coords_halfstep", "momenta"):
            self.Data[k] = _f(self.Data[k][:, keep])
        self.Data["weights"] = _f(self.Data["weights"][keep])


class CpuRun:
    """make_halfstep / make_step of the reference on numpy arrays."""

    def __init__(self, solver, species, window=None):
        """solver: a chimera_gb300 Solver built on the CPU (numpy operators in
        ``Args``); species: CpuSpecies list; window: moving-frame dict."""
        self.S = solver
        A = self.A = solver.Args
        self.Particles = species
        nx, nr, nkr, nm = A["Nx"], A["Nr"], A["Nkr"], A["Mtot"]
        z = lambda s: np.zeros(s, complex, order="F")  # noqa: E731
        self.D = {"EB": z((nx, nr, nm, 6)), "J": z((nx, nr, nm, 3)), "EG_fb": _f(
            solver.Data["EG_fb"].cpu().numpy(), complex), "vec_fb": z((nx, nkr, nm, 3)),
            "J_fb": z((nx, nkr, nm, 3)), "B_fb": z((nx, nkr, nm, 3))}
        self.space_charge = "SpaceCharge" in A["Features"]
        if self.space_charge:
            self.D.update(Rho=z((nx, nr, nm)), Rho_fb=z((nx, nkr, nm)),
                          gradRho_fb_nxt=z((nx, nkr, nm, 3)), gradRho_fb_prv=z((nx, nkr, nm, 3)))
        if "StillAsBackground" in A["Features"]:
            self.D["BckGrndRho"] = z((nx, nr, nm))
        self.CE = _f(solver.Data["PSATD_E"].cpu().numpy())
        self.CG = _f(solver.Data["PSATD_G"].cpu().numpy())
        self.wind = dict(window) if window else {}
        w = self.wind
        w.setdefault("Features", ())
        w.setdefault("TimeActive", (0.0, np.inf))
        w.setdefault("Velocity", 1.0)
        w.setdefault("TimeStep", 1.0)
        w.setdefault("Steps", 1)
        w["shiftX"] = (0.5 if "Staged" in w["Features"] else 1.0) * w["Velocity"] * w["TimeStep"] \
            * w["Steps"]
        if "AbsorbLayer" in w:
            A["damp_profile_np"] = solver.get_damp_profile(w["AbsorbLayer"])
        self.DP = [A["Rgrid"], A["dx_inv"], A["dr_inv"]]
        self.make_halfstep()

    # -- solver wrappers (solvers.py) ----------------------------------------
    def _fbdiff(self):
        return (self.A["DpS2S"], self.A["DmS2S"], self.A["kx"])

    def fb_curr_in(self):
        D, A = self.D, self.A
        D["J_fb"] = orc.fb_vec_in(D["J_fb"], D["J"], A["leftX"], A["kx"], A["InCurr"])
        D["J_fb"] = orc.omp_mult_vec(D["J_fb"], A["DepFact"])

    def project_current(self):
        D = self.D
        D["J"][:] = 0.0
        for sp in self.Particles:
            if sp.n() == 0 or sp.still:
                continue
            d = sp.Data
            if "Xchunked" in sp.Args:
                D["J"] = orc.dep_curr_chnk(d["coords_halfstep"], d["momenta"], d["weights"], D["J"],
                                           sp.chunks, sp.Args["Xchunked"][1], self.A["leftX"],
                                           *self.DP)
            else:
                D["J"] = orc.dep_curr(d["coords_halfstep"], d["momenta"], d["weights"], D["J"],
                                      self.A["leftX"], *self.DP)
        self.fb_curr_in()

    def _dep_dens(self, target, still):
        D = self.D
        for sp in self.Particles:
            if sp.n() == 0 or sp.still != still:
                continue
            d = sp.Data
            if "Xchunked" in sp.Args:
                D[target] = orc.dep_dens_chnk(d["coords"], d["weights"], D[target], sp.chunks,
                                              sp.Args["Xchunked"][1], self.A["leftX"], *self.DP)
            else:
                D[target] = orc.dep_dens(d["coords"], d["weights"], D[target], self.A["leftX"],
                                         *self.DP)

    def dep_dens(self):
        D = self.D
        D["Rho"][:] = 0.0
        if "BckGrndRho" in D:
            D["Rho"] += D["BckGrndRho"]
        self._dep_dens("Rho", False)

    def dep_bg(self):
        self.D["BckGrndRho"][:] = 0.0
        self._dep_dens("BckGrndRho", True)

    def project_density(self):
        if not self.space_charge:
            return
        D, A = self.D, self.A
        D["gradRho_fb_prv"][:] = D["gradRho_fb_nxt"]
        self.dep_dens()
        D["Rho_fb"] = orc.fb_scl_in(D["Rho_fb"], D["Rho"], A["leftX"], A["kx"], A["InCurr"])
        D["Rho_fb"] = orc.omp_mult_scl(D["Rho_fb"], A["DepFact"])
        D["gradRho_fb_nxt"] = orc.fb_grad(D["gradRho_fb_nxt"], D["Rho_fb"], *self._fbdiff())

    def update_fields(self):
        D, A = self.D, self.A
        if "NoPoissonCorrection" not in A["Features"]:
            for _ in range(3):
                D["vec_fb"][:] = D["J_fb"]
                D["vec_fb"] = orc.fb_graddiv(D["vec_fb"], *self._fbdiff())
                if self.space_charge:
                    D["J_fb"] = orc.poiss_corr(D["J_fb"], D["vec_fb"], D["gradRho_fb_prv"],
                                               D["gradRho_fb_nxt"], A["dt_inv"], A["PoissFact"])
                else:
                    D["vec_fb"] = orc.omp_mult_vec(D["vec_fb"], A["PoissFact"])
                    D["J_fb"] = orc.omp_add_vec(D["J_fb"], D["vec_fb"])
        if self.space_charge:
            D["EG_fb"] = orc.maxwell_push_with_spchrg(D["EG_fb"], D["J_fb"], D["gradRho_fb_prv"],
                                                      D["gradRho_fb_nxt"], self.CE, self.CG)
        else:
            D["EG_fb"] = orc.maxwell_push_wo_spchrg(D["EG_fb"], D["J_fb"], self.CE, self.CG)

    def project_fields(self):
        D, A = self.D, self.A
        for sp in self.Particles:
            if not sp.still:
                sp.Data["EB"] = np.zeros((6, sp.n()), order="F")
        D["B_fb"] = orc.fb_rot(D["B_fb"], _f(D["EG_fb"][:, :, :, 3:], complex), *self._fbdiff())
        D["B_fb"] = orc.omp_mult_vec(D["B_fb"], A["PoissFact"])
        D["EB"] = orc.fb_eb_out(D["EB"], D["EG_fb"], D["B_fb"], A["leftX"], A["kx"], A["Out"])
        D["EB"] = orc.eb_correction(D["EB"])
        for sp in self.Particles:
            if sp.n() == 0 or sp.still:
                continue
            d = sp.Data
            d["EB"] = orc.proj_fld(d["coords"], d["weights"], D["EB"], d["EB"], A["leftX"], *self.DP)

    def push_velocs(self, frac=1.0):
        for sp in self.Particles:
            if sp.n() and not sp.still:
                sp.Data["momenta"] = orc.push_velocs(sp.Data["momenta"], sp.Data["EB"],
                                                     sp.Args["push_fact"] * frac * sp.Args["TimeStep"])

    def push_coords(self):
        for sp in self.Particles:
            if sp.n() and not sp.still:
                sp.Data["coords"], sp.Data["coords_halfstep"] = orc.push_coords(
                    sp.Data["coords"], sp.Data["momenta"], sp.Data["coords_halfstep"],
                    sp.Args["TimeStep"])

    # -- window (chimera_main.py:250-304) --------------------------------------
    def move_frame(self):
        for args in [self.A] + [sp.Args for sp in self.Particles]:
            args["Xgrid"] = args["Xgrid"] + self.wind["shiftX"]
            args["leftX"] = args["Xgrid"][0]
            args["rightX"] = args["Xgrid"][-1]

    def frame_act(self, istep):
        w = self.wind
        if istep < w["TimeActive"][0] or istep > w["TimeActive"][1]:
            return
        if np.mod(istep - w["TimeActive"][0], w["Steps"]) != 0:
            return
        D, A = self.D, self.A
        if w.get("AbsorbLayer", 0) > 0:
            for sl in (slice(0, 3), slice(3, 6)):
                part = _f(D["EG_fb"][:, :, :, sl], complex)
                part = orc.fb_filtr(part, A["leftX"], A["kx"], A["damp_profile_np"], 0)
                D["EG_fb"][:, :, :, sl] = part
        self.move_frame()
        if "AddPlasma" in w:
            xsteps = int(w["shiftX"] / w["TimeStep"]) + 1
            if "IonsOnTop" in w["Features"]:
                s1, s2 = self.Particles[:2]
                parts = s1.sp.gen_parts(Xsteps=xsteps, ProfileFunc=w["AddPlasma"])
                s1.add(*parts)
                parts[-1] = parts[-1] * -1
                s2.add(*parts)
            else:
                for sp in self.Particles:
                    sp.add(*sp.sp.gen_parts(Xsteps=xsteps, ProfileFunc=w["AddPlasma"]))
        if "AbsorbLayer" in w:
            for sp in self.Particles:
                sp.chunk_and_damp(wind=w)
        if self.space_charge:
            if "BckGrndRho" in D:
                self.dep_bg()
            self.dep_dens()

    def chunk_particles(self, istep):
        for sp in self.Particles:
            if "Xchunked" not in sp.Args or "NoSorting" in sp.Args["Features"]:
                continue
            if np.mod(istep, sp.Args["Xchunked"][1] + 1) != 0 or sp.n() == 0:
                continue
            SimDom = _f([self.A["leftX"], self.A["rightX"], 0, self.A["Rgrid"].max() ** 2])
            sp.chunk_and_damp(SimDom=SimDom, position="cntr")

    def make_halfstep(self):
        A = self.A
        for sp in self.Particles:
            SimDom = _f([A["leftX"], A["rightX"], 0, A["upperR"] ** 2])
            if SimDom[0] != SimDom[1]:
                sp.chunk_and_damp(SimDom=SimDom)
        self.project_current()
        self.project_density()
        if self.space_charge:
            for sp in self.Particles:
                self._static(sp.Args["MomentaMeans"][0])
        self.project_fields()
        self.push_velocs(0.5)

    def _static(self, px0):
        A, D = self.A, self.D
        beta0 = px0 / np.sqrt(1 + px0 ** 2)
        kx_g = beta0 * A["kx_g"][:, :, None]
        w = A["w"]
        den = w ** 2 - kx_g ** 2
        C1 = np.zeros(w.shape + (2,), complex, order="F")
        C2 = np.zeros_like(C1)
        C1[..., 0], C1[..., 1] = 1.j * kx_g / den, -1. / den
        C2[..., 0], C2[..., 1] = w ** 2 / den, 1.j * kx_g / den
        D["EG_fb"] = orc.maxwell_init_push(D["EG_fb"], D["J_fb"], D["gradRho_fb_nxt"], C1, C2)

    def make_step(self, istep):
        self.frame_act(istep)
        self.push_coords()
        self.chunk_particles(istep)
        self.project_current()
        self.project_density()
        self.update_fields()
        self.project_fields()
        self.push_velocs()


def add_gauss_beam(solver, S):
    """Gaussian laser pulse added to solver.Data["EG_fb"] in spectral space,
    for the plain (non-envelope) solver, with the oracle's kernels: the
    reference's Solver.add_gauss_beam (moduls/solvers.py:555-610) restated on
    numpy.  solver: a Solver built on the CPU; S: the laser dict."""
    A = solver.Args
    k0, a0 = 2 * np.pi * S["k0"], 2 * np.pi * S["a0"]
    Xf = S["x0"] - S["x_foc"]
    nx, nkr, nm = A["Nx"], A["Nkr"], A["Mtot"]
    X, R = A["Xgrid"][:, None], A["Rgrid"][None, :]
    prof = (a0 * np.cos(k0 * (X - S["x0"])) * np.exp(-(X - S["x0"]) ** 2 / S["Lx"] ** 2
                                                     - R ** 2 / S["LR"] ** 2)
            * (abs(R) < 3.5 * S["LR"]) * (abs(X - S["x0"]) < 3.5 * S["Lx"]))
    prof[:, 0] = 0.0
    scl = np.zeros((nx, A["Nr"], nm), complex, order="F")
    scl[:, :, 0] = prof
    scl_fb = orc.fb_scl_in(np.zeros((nx, nkr, nm), complex, order="F"), scl, A["leftX"], A["kx"],
                           A["In"])
    EE = np.zeros((nx, nkr, nm, 3), complex, order="F")
    EE[:, :, :, 2] = scl_fb / nx
    # div_clean (solvers.py:644-650): EE + PoissFact grad(div(EE))
    v = orc.fb_graddiv(EE.copy(order="F"), A["DpS2S"], A["DmS2S"], A["kx"])
    v = orc.omp_mult_vec(v, A["PoissFact"])
    EE = orc.omp_add_vec(EE, v)
    kx_g = A["kx_g"][:, :, None, None]
    w4 = A["w"][:, :, :, None]
    DT = -1.j * w4 * np.sign(kx_g + (kx_g == 0))
    GG = DT * EE
    cw, sw = np.cos(w4 * Xf), np.sin(w4 * Xf)
    E1 = cw * EE + sw / w4 * GG
    G1 = -w4 * sw * EE + cw * GG
    ph = np.exp(1.j * kx_g * Xf)
    eg = solver.Data["EG_fb"]
    eg[:, :, :, :3] += torch_from(E1 * ph)
    eg[:, :, :, 3:] += torch_from(G1 * ph)


def torch_from(a):
    import torch
    return torch.from_numpy(np.ascontiguousarray(a))
