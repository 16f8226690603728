"""Diagnostics of a ChimeraRun (moduls/diagnostics.py), with the field
reductions on the device.

``Diagnostics(Chimera, diags, out_folder)`` takes the reference's diag dicts
(``{'Type': 'Fields'|'FieldsFB'|'Particles'|'Density'|'EnergyEM'|'Power',
'Step': n, 'Features': {...}}``) and ``do_diags(i)`` runs the ones due at
step i.  With ``'Return'`` in the features a diagnostic returns its data;
otherwise it writes the reference's files (``ee_*.npy``, ``dens_*.npy``,
``phs*.npy``, ``nrg_*.txt``, ``pwrX_*.txt``, ``pwrO_*.txt``) into
out_folder.

The energy and power diagnostics reduce the FP64 grids on the GPU in a fixed
summation order (``chm_em_energy``, ``chm_power_profile``,
``chm_intens_profo``); only their per-x (or per-angle) results, a few
kilobytes, come to the host.  Field-like returns (Fields, FieldsFB,
Density, Particles) are device tensors, as the ``Data`` entries they copy;
the energy and power profiles are numpy arrays, as the reference writes them
to text files.

This module restates the reference's GPLv3-licensed Python layer
(hightower8083/chimera) statement by statement to keep its API as a
drop-in; it is a derivative of that code and is distributed under the GNU
General Public License, version 3 or later, as the reference is.
"""
from __future__ import annotations

import os
import shutil

import numpy as np
import torch

from . import fimera as chimera

PwrFctr = 0.5 * 0.511e6 * 1.6022e-19 / 2.818e-13 * 2.9979e10  # diagnostics.py:24
Ntheta = 60                                                   # diagnostics.py:25


def _host(t):
    return t.detach().cpu().numpy() if isinstance(t, torch.Tensor) else np.asarray(t)


class Diagnostics:
    """diagnostics.py:27-237"""

    def __init__(self, Chimera, diags=(), out_folder=None):
        self.Chimera = Chimera
        self.diags = diags
        self._efact = {}
        if out_folder is not None:
            # the reference empties the folder (rm -rf, mkdir)
            self.out_folder = out_folder
            if os.path.isdir(out_folder):
                shutil.rmtree(out_folder)
            os.makedirs(out_folder)

    def do_diags(self, i):
        """diagnostics.py:36-49: the diags whose Step divides i."""
        for diag in self.diags:
            if np.mod(i, diag["Step"]) != 0:
                continue
            self.istr = str(i).rjust(7, "0")
            if "Features" not in diag:
                diag["Features"] = {}
            t = diag["Type"]
            if t == "Fields":
                self.fld_out(diag)
            if t == "FieldsFB":
                self.fldfb_out(diag)
            if t == "Particles":
                self.phs_out(diag)
            if t == "Density":
                self.dns_out(diag)
            if t == "EnergyEM":
                self.nrg_out(diag)
            if t == "Power":
                self.pwr_out(diag)

    # -- field dumps --------------------------------------------------------
    def _save(self, name, dat):
        np.save(os.path.join(self.out_folder, name), _host(dat))

    def fld_out(self, diag):
        """diagnostics.py:51-58: EB without the ghost row."""
        ret = "Return" in diag["Features"]
        out = []
        for jj, sol in enumerate(self.Chimera.Solvers):
            dat = sol.Data["EB"][:, 1:]
            if ret:
                out.append(dat.clone())
            else:
                self._save("ee_" + str(jj) + "_" + self.istr + ".npy", dat)
        if ret:
            return out

    def fldfb_out(self, diag):
        """diagnostics.py:60-68: the spectral E and G fields."""
        ret = "Return" in diag["Features"]
        out = []
        for jj, sol in enumerate(self.Chimera.Solvers):
            dat = sol.Data["EG_fb"]
            if ret:
                out.append(dat.clone())
            else:
                self._save("ee_" + str(jj) + "_" + self.istr + ".npy", dat)
        if ret:
            return out

    def dns_out(self, diag):
        """diagnostics.py:70-87: density of each moving species on the grid."""
        if "MaxMode" in diag["Features"]:
            modes = diag["Features"]["MaxMode"]
        elif len(self.Chimera.Solvers) > 0:
            modes = self.Chimera.Solvers[0].Args["MaxAzimuthMode"]
        else:
            modes = 0
        ret = "Return" in diag["Features"]
        out = []
        for jj, sp in enumerate(self.Chimera.Particles):
            if "Still" in sp.Args["Features"]:
                continue
            dat = sp.get_dens_on_grid(modes)[:, 1:]
            if ret:
                out.append(dat.clone())
            else:
                self._save("dens_" + str(jj) + "_" + self.istr + ".npy", dat)
        if ret:
            return out

    def phs_out(self, diag):
        """diagnostics.py:89-107: phase space of the particles above the LPA
        filter 1 + |p|^2 > 20^2 (coords_halfstep, momenta, weights)."""
        ret = "Return" in diag["Features"]
        out = []
        for jj, sp in enumerate(self.Chimera.Particles):
            if "Still" in sp.Args["Features"]:
                continue
            p = sp.Data["momenta"]
            indx = torch.nonzero((1.0 + p ** 2).sum(0) > 20.0 ** 2).flatten()
            pack = torch.cat((sp.Data["coords_halfstep"][:, indx], p[:, indx],
                              sp.Data["weights"][indx][None, :]), dim=0)
            if ret:
                out.append(pack)
            else:
                self._save("phs" + str(jj) + "_" + self.istr + ".npy", pack)
        if ret:
            return out

    # -- device reductions --------------------------------------------------
    def _energy_fact(self, sol):
        key = id(sol)
        ef = self._efact.get(key)
        if ef is None:
            ef = chimera.to_device(sol.Args["EnergyFact"], torch.float64,
                                   sol.Data["EG_fb"].device)
            self._efact[key] = ef
        return ef

    def nrg_out(self, diag):
        """diagnostics.py:109-122: energy of the E field per kx (EnergyFact
        weighted, summed over kr and modes on the device), reordered as
        r_[dat[N/2+1:], dat[:N/2+1]]."""
        ret = "Return" in diag["Features"]
        out = []
        for jj, sol in enumerate(self.Chimera.Solvers):
            dat = chimera.em_energy(sol.Data["EG_fb"], self._energy_fact(sol))
            n = dat.shape[0]
            dat = _host(torch.cat((dat[n // 2 + 1:], dat[:n // 2 + 1])))
            if ret:
                out.append(dat.copy())
            else:
                with open(os.path.join(self.out_folder, "nrg_" + str(jj) + ".txt"), "a") as f:
                    np.savetxt(f, dat[None, :])
        if ret:
            return out

    def _power(self, sol):
        Rgrid, dr = sol.Args["RgridFull"], sol.Args["dr"]
        dat = chimera.fb_vec_out(sol.Data["EG_fb"][:, :, :, :3], sol.Args["leftX"],
                                 *sol.Args["FBoutFull"])
        pwr = _host(chimera.power_profile(dat, Rgrid, PwrFctr * 2 * dr))
        return dat, pwr

    def pwr_out(self, diag):
        """diagnostics.py:124-149: laser power per x, and with 'Spot' the
        intensity over Ntheta angles and r (intens_profO)."""
        ret = "Return" in diag["Features"]
        spot = "Spot" in diag["Features"]
        out = []
        for jj, sol in enumerate(self.Chimera.Solvers):
            dat, pwr = self._power(sol)
            if ret:
                if spot:
                    out.append([pwr, _host(chimera.intens_profo(dat, Ntheta))])
                else:
                    out.append(pwr)
            else:
                with open(os.path.join(self.out_folder, "pwrX_" + str(jj) + ".txt"), "a") as f:
                    np.savetxt(f, pwr[None])
                if spot:
                    spot_val = _host(chimera.intens_profo(dat, Ntheta))
                    with open(os.path.join(self.out_folder, "pwrO_" + str(jj) + ".txt"), "a") as f:
                        np.savetxt(f, spot_val.ravel()[None])
        if ret:
            return out

    def get_spot_cartesian(self, val=None, solver_index=0, bins=(200, 200), th_part=1.0):
        """diagnostics.py:151-177: the intensity profile on a Cartesian grid
        (host interpolation of the device intens_profO result)."""
        from scipy.interpolate import griddata
        sol = self.Chimera.Solvers[solver_index]
        if val is None:
            dat = chimera.fb_vec_out(sol.Data["EG_fb"][:, :, :, :3], sol.Args["leftX"],
                                     *sol.Args["FBoutFull"])
            val = _host(chimera.intens_profo(dat, Ntheta))
        val = np.asarray(val)
        r_max = np.asarray(sol.Args["RgridFull"]).max()
        rr = np.r_[0:r_max:val.shape[1] * 1j]
        ph = 2 * np.pi / (Ntheta - 1.0) * np.arange(1, Ntheta + 1)
        ph, rr = np.meshgrid(ph, rr)
        coord = ((rr * np.cos(ph)).flatten(), (rr * np.sin(ph)).flatten())
        r_max = th_part * r_max
        new_coord = np.mgrid[-r_max:r_max:bins[0] * 1j, -r_max:r_max:bins[1] * 1j]
        val = griddata(coord, val.T.flatten(), (new_coord[0].flatten(), new_coord[1].flatten()),
                       fill_value=0.0, method="linear").reshape(new_coord[0].shape)
        ext = np.array([-r_max, r_max, -r_max, r_max])
        return val, ext

    def get_beam_envelops(self):
        """diagnostics.py:179-211: weighted centroid, rms size and emittance
        of each moving species (device reductions)."""
        out = []
        for sp in self.Chimera.Particles:
            if "Still" in sp.Args["Features"]:
                continue
            x, y, z = sp.Data["coords_halfstep"]
            px, py, pz = sp.Data["momenta"]
            w = sp.Data["weights"]
            ws = w.sum()
            c0 = [(a * w).sum() / ws for a in (x, y, z)]
            rms = [torch.sqrt((a ** 2 * w).sum() / ws - m ** 2) for a, m in zip((x, y, z), c0)]
            emit = [torch.sqrt((a ** 2 * w).sum() / ws * (b ** 2 * w).sum() / ws
                               - (a * b * w).sum() ** 2 / ws ** 2)
                    for a, b in ((x, px), (y, py), (z, pz))]
            out.append(np.array([[float(v) for v in c0], [float(v) for v in rms],
                                 [float(v) for v in emit]]))
        return out
