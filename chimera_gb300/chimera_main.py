"""Drop-in ``ChimeraRun`` step loop (the reference's moduls/chimera_main.py:23-318).

The control flow, the order of the kernel calls and the moving-window logic
follow the reference; every kernel is a CUDA launch on the current torch
stream, so a step issues no host synchronisation except where particles are
absorbed or injected (the new particle count is read back).

This module restates the reference's GPLv3-licensed Python layer
(hightower8083/chimera) statement by statement to keep its API as a
drop-in; it is a derivative of that code and is distributed under the GNU
General Public License, version 3 or later, as the reference is.
"""
from __future__ import annotations

import numpy as np

from . import fimera as chimera


class ChimeraRun:
    def __init__(self, SimComps):
        self.Particles = SimComps.get("Particles", ())
        self.Solvers = SimComps.get("Solvers", ())
        self.MovingFrames = SimComps.get("MovingFrames", ({},))
        self.init_Moving_Frames()
        self.init_damp_profile()
        self.make_halfstep()

    def init_Moving_Frames(self):
        """chimera_main.py:41-52"""
        for wind in self.MovingFrames:
            wind.setdefault("Features", ())
            wind.setdefault("TimeActive", (0.0, np.inf))
            wind.setdefault("Velocity", 1.0)
            wind.setdefault("TimeStep", 1.0)
            wind.setdefault("Steps", 1)
            shift = wind["Velocity"] * wind["TimeStep"] * wind["Steps"]
            wind["shiftX"] = 0.5 * shift if "Staged" in wind["Features"] else shift

    def init_damp_profile(self):
        """chimera_main.py:54-59"""
        for solver in self.Solvers:
            for wind in self.MovingFrames:
                if "AbsorbLayer" in wind:
                    solver.Args["damp_profile"] = solver.get_damp_profile(wind["AbsorbLayer"])

    def _args0(self):
        return self.Solvers[0].Args if len(self.Solvers) > 0 else self.Particles[0].Args

    def make_halfstep(self):
        """chimera_main.py:61-80"""
        for species in self.Particles:
            a = self._args0()
            SimDom = np.asfortranarray([a["leftX"], a["rightX"], 0, a["upperR"] ** 2])
            if SimDom[0] != SimDom[1]:
                species.chunk_and_damp(SimDom=SimDom)
        self.project_current()
        self.project_density()
        for solver in self.Solvers:
            for species in self.Particles:
                solver.maxwell_solver_stat(species.Args["MomentaMeans"][0])
        self.project_fields()
        for species in self.Particles:
            species.make_device()
        for species in self.Particles:
            species.push_velocs(dt_frac=0.5)

    def make_step(self, istep):
        """chimera_main.py:82-92: one PIC step."""
        self.frame_act(istep)
        for species in self.Particles:
            species.push_coords()
        self.chunk_particles(istep)
        self.project_current()
        self.frame_act(istep, "stage2")
        self.project_density()
        self.update_fields()
        self.project_fields()
        for species in self.Particles:
            species.make_device(istep)
        for species in self.Particles:
            species.push_velocs()

    def project_current(self):
        """chimera_main.py:94-101"""
        for solver in self.Solvers:
            if "NoCurrent" in solver.Args["Features"]:
                solver.Data["J"].zero_()
                solver.Data["J_fb"].zero_()
                continue
            self.dep_curr(solver)
            solver.fb_curr_in()

    def project_density(self):
        """chimera_main.py:103-114"""
        for solver in self.Solvers:
            feats = solver.Args["Features"]
            if "SpaceCharge" not in feats and "StaticKick" not in feats:
                continue
            if "StaticKick" not in feats:
                solver.Data["gradRho_fb_prv"].copy_(solver.Data["gradRho_fb_nxt"])
            self.dep_dens(solver)
            solver.fb_dens_in()
            solver.FBGradDens()

    def update_fields(self):
        """chimera_main.py:116-128"""
        for solver in self.Solvers:
            if "StaticKick" in solver.Args["Features"]:
                solver.Data["EG_fb"].zero_()
                for species in self.Particles:
                    w = species.Data["weights"]
                    px = float((species.Data["momenta"][0] * w).sum() / w.sum())
                    solver.poiss_corr_stat(px)
                    solver.maxwell_solver_stat(px)
                    solver.field_drift(px)
            else:
                solver.poiss_corr()
                solver.maxwell_solver()

    def project_fields(self, component="coords"):
        """chimera_main.py:130-151"""
        for species in self.Particles:
            species.make_field()
        for solver in self.Solvers:
            if "NoPush" in solver.Args["Features"]:
                solver.Data["EB"].zero_()
                continue
            solver.G2B_FBRot()
            solver.fb_fld_out()
            for species in self.Particles:
                if species.Data[component].shape[1] == 0 or "Still" in species.Args["Features"]:
                    continue
                f = chimera.proj_fld_env if "KxShift" in solver.Args else chimera.proj_fld
                species.Data["EB"] = f(species.Data[component], species.Data["weights"],
                                       solver.Data["EB"], species.Data["EB"], solver.Args["leftX"],
                                       *solver.Args["DepProj"])

    def _deposit(self, solver, target, component, still_only):
        """Shared body of dep_curr / dep_dens / dep_bg (chimera_main.py:153-248)."""
        env = "KxShift" in solver.Args
        curr = target == "J"
        for species in self.Particles:
            is_still = "Still" in species.Args["Features"]
            if species.Data[component].shape[1] == 0 or is_still != still_only:
                continue
            D = species.Data
            chunked = "Xchunked" in species.Args
            if curr:
                if chunked:
                    f = chimera.dep_curr_env_chnk if env else chimera.dep_curr_chnk
                    out = f(D["coords_halfstep"], D["momenta"], D["weights"], solver.Data[target],
                            species.chunks, species.Args["Xchunked"][1], solver.Args["leftX"],
                            *solver.Args["DepProj"])
                else:
                    f = chimera.dep_curr_env if env else chimera.dep_curr
                    out = f(D["coords_halfstep"], D["momenta"], D["weights"], solver.Data[target],
                            solver.Args["leftX"], *solver.Args["DepProj"])
            else:
                if chunked:
                    f = chimera.dep_dens_env_chnk if env else chimera.dep_dens_chnk
                    out = f(D[component], D["weights"], solver.Data[target], species.chunks,
                            species.Args["Xchunked"][1], solver.Args["leftX"],
                            *solver.Args["DepProj"])
                else:
                    f = chimera.dep_dens_env if env else chimera.dep_dens
                    out = f(D[component], D["weights"], solver.Data[target], solver.Args["leftX"],
                            *solver.Args["DepProj"])
            solver.Data[target] = out

    def dep_curr(self, solver):
        """chimera_main.py:153-181"""
        solver.Data["J"].zero_()
        self._deposit(solver, "J", "coords", still_only=False)

    def dep_dens(self, solver, component="coords"):
        """chimera_main.py:183-218"""
        solver.Data["Rho"].zero_()
        if "StaticKick" in solver.Args["Features"]:
            component = "coords_halfstep"
        if "StillAsBackground" in solver.Args["Features"]:
            solver.Data["Rho"] += solver.Data["BckGrndRho"]
        self._deposit(solver, "Rho", component, still_only=False)

    def dep_bg(self, solver):
        """chimera_main.py:220-248: density of the Still species."""
        solver.Data["BckGrndRho"].zero_()
        self._deposit(solver, "BckGrndRho", "coords", still_only=True)

    def damp_fields(self, wind):
        """chimera_main.py:250-255"""
        if "AbsorbLayer" not in wind or wind["AbsorbLayer"] <= 0:
            return
        for solver in self.Solvers:
            if "StaticKick" not in solver.Args["Features"]:
                solver.damp_field()

    def damp_plasma(self, wind):
        """chimera_main.py:257-259"""
        if "AbsorbLayer" not in wind:
            return
        for species in self.Particles:
            species.chunk_and_damp(wind=wind)

    def add_plasma(self, wind):
        """chimera_main.py:261-275"""
        if "AddPlasma" not in wind:
            return
        xsteps = int(wind["shiftX"] / wind["TimeStep"]) + 1
        if "IonsOnTop" in wind["Features"]:
            s1, s2 = self.Particles[:2]
            parts = s1.gen_parts(Xsteps=xsteps, ProfileFunc=wind["AddPlasma"])
            s1.add_particles(*parts)
            parts[-1] = parts[-1] * -1
            s2.add_particles(*parts)
        else:
            for species in self.Particles:
                species.add_particles(*species.gen_parts(Xsteps=xsteps,
                                                         ProfileFunc=wind["AddPlasma"]))

    def postframe_corr(self, wind):
        """chimera_main.py:277-284.  The reference's condition
        ``'AbsorbLayer' or 'AddPlasma' in wind`` is always true; kept."""
        for solver in self.Solvers:
            if "StaticKick" in solver.Args["Features"]:
                continue
            if "SpaceCharge" in solver.Args["Features"]:
                if "StillAsBackground" in solver.Args["Features"]:
                    self.dep_bg(solver)
                self.dep_dens(solver)

    def move_frame(self, wind):
        """chimera_main.py:286-290"""
        for comp in tuple(self.Solvers) + tuple(self.Particles):
            comp.Args["Xgrid"] = comp.Args["Xgrid"] + wind["shiftX"]
            comp.Args["leftX"] = comp.Args["Xgrid"][0]
            comp.Args["rightX"] = comp.Args["Xgrid"][-1]

    def frame_act(self, istep, act="stage1"):
        """chimera_main.py:292-304"""
        for wind in self.MovingFrames:
            if istep < wind["TimeActive"][0] or istep > wind["TimeActive"][1]:
                continue
            if np.mod(istep - wind["TimeActive"][0], wind["Steps"]) != 0:
                continue
            if act == "stage1":
                self.damp_fields(wind)
                self.move_frame(wind)
                self.add_plasma(wind)
                self.damp_plasma(wind)
                self.postframe_corr(wind)
            elif act == "stage2" and "Staged" in wind["Features"]:
                self.move_frame(wind)

    def chunk_particles(self, istep=0):
        """chimera_main.py:306-318"""
        for species in self.Particles:
            if "Xchunked" not in species.Args or "NoSorting" in species.Args["Features"]:
                continue
            if np.mod(istep, species.Args["Xchunked"][1] + 1) != 0:
                continue
            if species.Data["coords"].shape[-1] == 0:
                continue
            a = self._args0()
            SimDom = np.asfortranarray([a["leftX"], a["rightX"], 0, a["Rgrid"].max() ** 2])
            species.chunk_and_damp(SimDom=SimDom, position="cntr")

    # ------------------------------------------------------------------
    # checkpoints (chimera_main.py:325-410), as .npz
    def drop_snap(self, fname="./snap_", verbose=False):
        """chimera_main.py:325-369: write every storable Data / Args entry of
        the solvers and species; returns the file name."""
        from . import snapshot
        name = snapshot.snap_name(fname)
        return snapshot.write(name, snapshot.snap_arrays(self.Solvers, self.Particles, verbose))

    def read_snap(self, fname="./test.npz", verbose=False):
        """chimera_main.py:371-410: restore the solvers' and species' Data /
        Args from a drop_snap file."""
        from . import snapshot
        with np.load(fname, allow_pickle=False) as f:
            snapshot.read_into(f, self.Solvers, self.Particles, verbose)
