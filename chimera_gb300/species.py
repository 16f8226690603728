"""Drop-in ``Specie`` (the reference's moduls/species.py:24-486) on GB300.

Particles live on the device in structure-of-arrays buffers with a capacity
(``ParticleStore``): ``Data['coords']`` etc. are (3, Np) float64 CUDA views
with part stride 1, re-bound whenever particles are added or removed.
Generation (``gen_parts``) runs on the host in numpy with the reference's
random-number call sequence, so a seeded ``np.random`` gives the same
particles as the reference; pushing, sorting, absorption and compaction run
as CUDA kernels through ``chimera_gb300.fimera``.

This module restates the reference's GPLv3-licensed Python layer
(hightower8083/chimera) statement by statement to keep its API as a
drop-in; it is a derivative of that code and is distributed under the GNU
General Public License, version 3 or later, as the reference is.
"""
from __future__ import annotations

import inspect

import numpy as np
import torch
from scipy.constants import c, e, epsilon_0, m_e

from . import _lib
from . import fimera as chimera

_VEC = ("coords", "coords_halfstep", "momenta", "coords_init")


class ParticleStore:
    """Capacity-allocated SoA buffers (ncomp, capacity) for one species.

    ``views()`` returns the (ncomp, n) views; a permutation (compaction /
    sort) gathers into the spare buffers and swaps them, so it never
    reallocates while the capacity suffices."""

    def __init__(self, names, device, capacity=0):
        self.device = device
        self.names = dict(names)  # name -> ncomp
        self.n = 0
        self.cap = 0
        self.buf: dict[str, torch.Tensor] = {}
        self.spare: dict[str, torch.Tensor] = {}
        self.reserve(max(int(capacity), 1))

    def _alloc(self, cap):
        return {k: torch.zeros((nc, cap), dtype=torch.float64, device=self.device)
                for k, nc in self.names.items()}

    def reserve(self, cap):
        cap = int(cap)
        if cap <= self.cap:
            return
        new, spare = self._alloc(cap), self._alloc(cap)
        for k in self.names:
            if self.n:
                new[k][:, : self.n].copy_(self.buf[k][:, : self.n])
        self.buf, self.spare, self.cap = new, spare, cap

    def views(self):
        out = {}
        for k, nc in self.names.items():
            v = self.buf[k][:, : self.n]
            out[k] = v[0] if nc == 1 else v
        return out

    def append(self, arrays: dict):
        add = next(iter(arrays.values()))
        m = int(add.shape[-1])
        if m == 0:
            return
        if self.n + m > self.cap:
            self.reserve(max(self.n + m, int(1.5 * self.cap) + 1024))
        for k, nc in self.names.items():
            a = arrays[k]
            if isinstance(a, torch.Tensor):
                t = a
            else:
                t = torch.from_numpy(np.ascontiguousarray(np.asarray(a, dtype=np.float64)))
                if self.device.type == "cuda":
                    chimera.io_bytes["h2d"] += t.numel() * 8
                    # pinned staging: an asynchronous copy (a pageable one
                    # would wait for the work queued on the stream)
                    t = t.pin_memory()
            t = t.to(self.device, torch.float64, non_blocking=True).reshape(nc, m)
            self.buf[k][:, self.n: self.n + m].copy_(t)
        self.n += m

    def permute(self, idx: torch.Tensor, names=None):
        """Keep particles idx (device int64), in that order."""
        n = int(idx.shape[0])
        for k in (names or self.names):
            nc = self.names[k]
            src = self.buf[k][:, : self.n]
            dst = self.spare[k][:, :n]
            if nc == 1:
                chimera.align_data_scl_into(dst[0], src[0], idx)
            else:
                chimera.align_data_vec_into(dst, src, idx)
            self.buf[k], self.spare[k] = self.spare[k], self.buf[k]
        self.n = n

    def resize(self, n):
        if n > self.cap:
            self.reserve(n)
        self.n = int(n)


class Specie:
    """A species of macro-particles (species.py:24)."""

    def __init__(self, specie_in, device=None):
        self.device = torch.device(device or "cuda")
        A = self.Args = specie_in
        A.setdefault("Features", ())
        A.setdefault("Charge", -1.0)
        A.setdefault("Mass", 1.0)
        A.setdefault("Density", 0.0)
        A.setdefault("MomentaMeans", (0.0, 0.0, 0.0))
        A.setdefault("MomentaSpreads", (0.0, 0.0, 0.0))
        A.setdefault("Grid", (0.0, 0.0, 0.0, 1.0, 1.0))
        self.Devices = A["Devices"] if "Devices" in A else ()

        A["leftX"], A["rightX"], A["lengthR"], A["dx"], A["dr"] = A["Grid"]
        A["push_fact"] = 2 * np.pi * A["Charge"] / A["Mass"]
        A["weight2pC"] = 4 * np.pi ** 2 * m_e * c ** 2 * epsilon_0 * 1e6 / e

        if "Xchunked" in A:
            A["nthrds"] = int(A["Xchunked"][0])
            A["Nx"] = 2 * A["nthrds"] * int(np.round(0.5 / A["dx"] / A["nthrds"]
                                                     * (A["rightX"] - A["leftX"])))
        else:
            A["Nx"] = 2 * int(np.round(0.5 / A["dx"] * (A["rightX"] - A["leftX"])))
        A["Xgrid"] = (A["rightX"] - A["dx"] * np.arange(A["Nx"])[::-1] if A["Nx"] > 0
                      else np.array([0.]))
        A["leftX"] = A["Xgrid"][0]

        A["Nr"] = int(np.round(A["lengthR"] / A["dr"]))
        A["Rgrid"] = A["dr"] * (np.arange(A["Nr"]) - 0.5) if A["Nr"] > 0 else np.array([0.])
        A["lowerR"] = (A["Rgrid"] * (A["Rgrid"] >= 0)).min()
        A["upperR"] = A["Rgrid"].max()

        # per-cell generator patterns (species.py:95-118)
        if "FixedCell" in A:
            fc = A["FixedCell"]
            A["Num_p"] = int(np.prod(fc))
            px, pr, po = np.mgrid[1:fc[0]:fc[0] * 1j, 1:fc[1]:fc[1] * 1j, 1:fc[2]:fc[2] * 1j]
            A["Pax"] = (np.asfortranarray((px.ravel() - 0.5) / fc[0]),
                        np.asfortranarray((pr.ravel() - 0.5) / fc[1]),
                        np.asfortranarray(np.exp(2.j * np.pi * (po.ravel() - 1) / fc[2])))
        elif "RandCell" in A:
            A["Num_p"] = A["RandCell"]
        else:
            A["Num_p"] = 0
        A["wght0"] = (A["Charge"] * A["Density"] * A["dr"] * A["dx"] * 2 * np.pi / A["Num_p"]
                      if A["Num_p"] != 0 else 0.0)
        A["NpSlice"] = A["Nx"] * A["Num_p"]

        names = {"coords": 3, "coords_halfstep": 3, "momenta": 3, "weights": 1, "EB": 6}
        if "KeepInitPos" in A["Features"]:
            names["coords_init"] = 3
        self.store = ParticleStore(names, self.device)
        self.Data = {}
        self.chunks = None
        self._sync()

    # ------------------------------------------------------------------
    def _sync(self):
        self.Data.update(self.store.views())

    @property
    def num_particles(self) -> int:
        return self.store.n

    def gen_parts(self, Domain=None, Xsteps=None, ProfileFunc=None):
        """Macro-particle generator (species.py:132-215); host numpy, returns
        [coords (3,Np), momenta (3,Np), weights (Np,)] as numpy arrays."""
        A = self.Args
        Xgrid, Rgrid = A["Xgrid"], A["Rgrid"]
        if Domain is not None:
            p_left, p_right, p_low, p_up = Domain
            if (A["leftX"] > p_right or A["rightX"] < p_left or p_up < A["lowerR"]
                    or p_low > A["upperR"]):
                return np.zeros((8, 0), order="F")
            ixb, ixe = (Xgrid < p_left).sum() - 1, (Xgrid < p_right).sum() + 1
            Xgrid = Xgrid[ixb:ixe]
            irb = 0 if p_low <= Rgrid.min() else (Rgrid < p_low).sum() - 1
            ire = Rgrid.shape[0] if p_up >= Rgrid.max() else (Rgrid < p_up).sum() + 1
            Rgrid = Rgrid[irb:ire]
        elif Xsteps is not None:
            Xgrid = Xgrid[-2 * Xsteps:-Xsteps]

        if "FixedCell" in A:
            rand_o = np.random.rand(Xgrid.shape[0], Rgrid.shape[0]).astype("d", order="F")
            coords = fixed_cell_particles(Xgrid, Rgrid, rand_o, *A["Pax"])
        elif "RandCell" in A:
            coords = self.gen_randcell(Xgrid, Rgrid)
        else:
            coords = np.zeros((4, 0))
        num = coords.shape[1]

        if ProfileFunc is None:
            coords[-1] *= A["wght0"]
        else:
            nargs = len(inspect.signature(ProfileFunc).parameters)
            if nargs == 1:
                coords[-1] *= A["wght0"] * ProfileFunc(coords[0])
            elif nargs == 2:
                coords[-1] *= A["wght0"] * ProfileFunc(coords[0], np.sqrt((coords[1:3] ** 2).sum(0)))
            elif nargs == 3:
                coords[-1] *= A["wght0"] * ProfileFunc(*coords[0:3])
            else:
                print("can't understand the ProfileFunc")

        if "FlatSpectrum" in A["Features"]:
            rnd = 2 * np.random.rand(3, num) - 1.0
        else:
            rnd = np.random.randn(3, num)
        mom = np.vstack([A["MomentaMeans"][k] + A["MomentaSpreads"][k] * rnd[k] for k in range(3)])
        return [np.asfortranarray(coords[0:3], dtype="d"), np.asfortranarray(mom, dtype="d"),
                np.asfortranarray(coords[-1], dtype="d")]

    def gen_parts_device(self, Xsteps=None, ProfileFunc=None):
        """gen_parts(Xsteps=..., ProfileFunc=...) with the particles built on
        the device (chm_gen_fixed_cell): the same random numbers are drawn on
        the host in the same order (rand_o, then the momenta), the pattern
        positions and the profile are evaluated on the host on the few
        distinct values, and only rand_o (and non-constant momenta) go to
        the device.  Returns device tensors [coords (3,Np), momenta (3,Np),
        weights (Np,)] in gen_parts' particle order.  Only for FixedCell
        species and a profile of x alone (or none); otherwise the host
        generator's arrays are uploaded."""
        A = self.Args
        nargs = (len(inspect.signature(ProfileFunc).parameters)
                 if ProfileFunc is not None else 0)
        if "FixedCell" not in A or nargs > 1 or Xsteps is None:
            c, p, w = self.gen_parts(Xsteps=Xsteps, ProfileFunc=ProfileFunc)
            up = lambda a: torch.from_numpy(np.ascontiguousarray(a)).to(self.device)  # noqa: E731
            return [up(c), up(p), up(w)]
        Xgrid = A["Xgrid"][-2 * Xsteps:-Xsteps]
        Rgrid = A["Rgrid"]
        nxg, nrg = Xgrid.shape[0], Rgrid.shape[0]
        rand_o = np.random.rand(nxg, nrg).astype("d", order="F")  # the RNG stream of gen_parts
        packx, packr, packo = A["Pax"]
        npc = packx.shape[0]
        dev = self.device
        if nxg < 2 or nrg < 2:
            num = 0
        else:
            cx, cr, keep, count, rank, base = fixed_cell_tables(Xgrid, Rgrid, packx, packr)
            nxc = nxg - 1
            num = int(count.sum()) * nxc
        if "FlatSpectrum" in A["Features"]:
            rnd = 2 * np.random.rand(3, num) - 1.0
        else:
            rnd = np.random.randn(3, num)
        coords = torch.empty((3, num), dtype=torch.float64, device=dev)
        weights = torch.empty(num, dtype=torch.float64, device=dev)
        spreads = A.get("MomentaSpreads", (0.0, 0.0, 0.0))
        if all(float(sp_) == 0.0 for sp_ in spreads):
            momenta = torch.empty((3, num), dtype=torch.float64, device=dev)
            for k in range(3):  # means + 0 * rnd
                momenta[k].fill_(float(A["MomentaMeans"][k]))
        else:
            mom = np.vstack([A["MomentaMeans"][k] + spreads[k] * rnd[k] for k in range(3)])
            momenta = torch.from_numpy(np.ascontiguousarray(mom)).pin_memory().to(
                dev, non_blocking=True)
            chimera.io_bytes["h2d"] += mom.nbytes
        if num == 0:
            return [coords, momenta, weights]
        # the particles' (x, r) pattern positions in output order, for the
        # caller's particle ordering (host values; no device read)
        keep3 = np.broadcast_to(keep[:, None, :], (nrg - 1, nxc, npc))
        self.last_gen_xr = (np.broadcast_to(cx[None, :, :], keep3.shape)[keep3],
                            np.broadcast_to(cr[:, None, :], keep3.shape)[keep3])
        prof = ProfileFunc(cx) if ProfileFunc is not None else 1.0
        wfac = np.asfortranarray(np.broadcast_to(A["wght0"] * prof, cx.shape), dtype=np.float64)

        def up(a, dt=None):
            a = np.asfortranarray(a) if dt is None else np.asfortranarray(a, dtype=dt)
            chimera.io_bytes["h2d"] += a.nbytes
            return torch.from_numpy(a.ravel(order="F").copy()).pin_memory().to(dev, non_blocking=True)

        t = [up(np.asfortranarray(cx)), up(np.asfortranarray(cr)), up(wfac),
             up(packo.astype(np.complex128)), up(rand_o), up(base, np.int64), up(rank, np.int32),
             up(count, np.int32)]
        _lib.call("chm_gen_fixed_cell", coords.data_ptr(), num, weights.data_ptr(), t[0].data_ptr(),
                  t[1].data_ptr(), t[2].data_ptr(), t[3].data_ptr(), t[4].data_ptr(), nxg,
                  t[5].data_ptr(), t[6].data_ptr(), t[7].data_ptr(), nxc, nrg - 1, npc,
                  torch.cuda.current_stream(dev).cuda_stream)
        return [coords, momenta, weights]

    def gen_randcell(self, Xgrid, Rgrid):
        """Random in-cell particles (species.py:429-471), same RNG sequence."""
        n = self.Args["Num_p"]
        dx, dr = self.Args["dx"], self.Args["dr"]
        out = np.zeros((4, max(0, (Xgrid.shape[0] - 1) * (Rgrid.shape[0] - 1) * n)))
        ip = 0
        base = np.arange(n)
        for ix in range(Xgrid.shape[0] - 1):
            for ir in range(Rgrid.shape[0] - 1):
                rc = 2 * (np.random.rand(3, n) - 0.5)
                xx = Xgrid[ix] + dx * (base + 0.5 * rc[0]) / n
                rr = Rgrid[ir] + dr * (base + 0.5 * rc[1]) / n
                oo = 2 * np.pi * (base + 0.5 * rc[2]) / n
                np.random.shuffle(xx)
                np.random.shuffle(rr)
                np.random.shuffle(oo)
                out[0, ip:ip + n] = xx
                out[1, ip:ip + n] = rr * np.cos(oo)
                out[2, ip:ip + n] = rr * np.sin(oo)
                out[3, ip:ip + n] = rr
                ip += n
        return out[:, :ip]

    def add_particles(self, coords, momenta, weights):
        """species.py:217-244: append particles (numpy or torch arrays)."""
        arrs = {"coords": coords, "coords_halfstep": coords, "momenta": momenta,
                "weights": weights, "EB": None}
        m = int(coords.shape[-1])
        arrs["EB"] = torch.zeros((6, m), dtype=torch.float64, device=self.device)
        if "coords_init" in self.store.names:
            arrs["coords_init"] = coords
        self.store.append(arrs)
        self._sync()

    def make_field(self):
        """species.py:246-256: zero the per-particle E, B container."""
        if "Still" in self.Args["Features"]:
            return
        self.Data["EB"].zero_()

    def make_device(self, i_step=0):
        """species.py:258-277: external fields from the devices."""
        if "Still" in self.Args["Features"]:
            return
        for device in self.Devices:
            self.Data["EB"] = device[0](self.Data["coords"], self.Data["EB"],
                                        i_step * self.Args["TimeStep"], *device[1:])

    def push_velocs(self, dt_frac=1.):
        """species.py:279-298 (Boris)"""
        if self.store.n == 0 or "Still" in self.Args["Features"]:
            return
        chimera.push_velocs(self.Data["momenta"], self.Data["EB"],
                            self.Args["push_fact"] * dt_frac * self.Args["TimeStep"])

    def push_coords(self, dt_frac=1.):
        """species.py:300-320 (leap-frog)"""
        if self.store.n == 0 or "Still" in self.Args["Features"]:
            return
        chimera.push_coords(self.Data["coords"], self.Data["momenta"], self.Data["coords_halfstep"],
                            dt_frac * self.Args["TimeStep"])

    def denoise(self, WaveNums2Kill):
        """species.py:322-349: mirrored anti-phase copies suppress shot noise."""
        for k in WaveNums2Kill:
            d = {key: v.clone() for key, v in self.Data.items()}
            n = self.store.n
            for key in ("coords", "coords_halfstep"):
                d[key][0] += 0.5 / k
            self.store.append({key: d[key] for key in self.store.names})
            w = self.store.buf["weights"][0, : 2 * n]
            w *= 0.5
            self._sync()

    def chunk_and_damp(self, wind=None, SimDom=None, position="stag"):
        """species.py:351-398: absorb particles outside SimDom and, with
        Xchunked, order the rest by x-chunk (stable counting sort)."""
        if self.store.n == 0:
            return
        A = self.Args
        comp = {"cntr": "coords_halfstep", "stag": "coords"}
        if wind is None:
            wind = {"Features": (), "AbsorbLayer": 0.0}
        if SimDom is None:
            SimDom = np.asfortranarray([A["leftX"] + wind["AbsorbLayer"] * A["dx"], A["rightX"],
                                        0.0, A["upperR"] ** 2])
        if "Xchunked" in A and "NoSorting" not in wind.get("Features", ()):
            ids, self.chunks, _ = chimera.chunk_coords_boundaries(
                self.Data[comp[position]], SimDom, A["Xgrid"], A["Xchunked"][0])
            idx = chimera.chunk_order(ids, A["Xchunked"][0])
        else:
            idx, num = chimera.sortpartsout(self.Data["coords"], SimDom)
            idx = idx[:num]
        names = [k for k in self.store.names if k != "EB"]
        self.store.permute(idx, names)
        self._sync()

    def get_dens_on_grid(self, Nko=0):
        """species.py:400-427: density of the species on its grid."""
        A = self.Args
        V = 2 * np.pi * A["dx"] * A["dr"] * A["Rgrid"]
        V = (V + (A["Rgrid"] == 0)) ** -1 * (A["Rgrid"] > 0.0)
        dens = chimera.fortran_zeros((A["Nx"], A["Nr"], Nko + 1), device=self.device)
        dens = chimera.dep_dens(self.Data["coords"], self.Data["weights"], dens, A["leftX"],
                                A["Rgrid"], 1. / A["dx"], 1 / A["dr"])
        return dens * torch.from_numpy(V).to(self.device)[None, :, None]

    def beam_focus(self, x_foc):
        """species.py:473-486: drift the beam back from its focus."""
        D = self.Data
        gg = (1 + D["momenta"] ** 2).sum(0) ** 0.5
        pzmean = (D["momenta"][0] * D["weights"]).sum() / D["weights"].sum()
        D["coords"][0] -= x_foc * (D["momenta"][0] - pzmean) / pzmean / gg ** 2
        D["coords"][1:3] -= D["momenta"][1:3] / pzmean * x_foc
        D["coords_halfstep"].copy_(D["coords"])


def fixed_cell_tables(Xgrid, Rgrid, packx, packr):
    """The tables of the device generator (chm_gen_fixed_cell): the pattern
    x positions cx (nx-1, npc) and radii cr (nr-1, npc) with the expressions
    of fixed_cell_particles, the kept points (cr > 0), their count and rank
    per r row, and each r row's first output index (rows of (nx-1) cells)."""
    dr_2 = 0.5 * (Rgrid[1] - Rgrid[0])
    rs = Rgrid + dr_2
    cx = Xgrid[:-1][:, None] + (Xgrid[1:] - Xgrid[:-1])[:, None] * packx[None, :]
    cr = rs[:-1][:, None] + (rs[1:] - rs[:-1])[:, None] * packr[None, :]
    keep = cr > 0
    count = keep.sum(1).astype(np.int32)
    rank = np.where(keep, np.cumsum(keep, 1) - 1, -1).astype(np.int32)
    base = np.concatenate([[0], np.cumsum(count.astype(np.int64) * (Xgrid.shape[0] - 1))[:-1]])
    return cx, cr, keep, count, rank, base


def fixed_cell_particles(Xgrid, Rgrid, rand_o, packx, packr, packo):
    """Host restatement of particle_tools.f90:84-128 (genparts): the fixed
    per-cell pattern rotated by a random angle per cell, cells in (r, x)
    order; returns (4, Np) = (x, y, z, r)."""
    nx, nr = Xgrid.shape[0], Rgrid.shape[0]
    if nx < 2 or nr < 2:
        return np.zeros((4, 0))
    dr_2 = 0.5 * (Rgrid[1] - Rgrid[0])
    rs = Rgrid + dr_2
    r0, r1 = rs[:-1][:, None, None], rs[1:][:, None, None]
    x0, x1 = Xgrid[:-1][None, :, None], Xgrid[1:][None, :, None]
    cx = x0 + (x1 - x0) * packx[None, None, :]
    cr = r0 + (r1 - r0) * packr[None, None, :]
    ang = 2.0 * np.pi * rand_o[: nx - 1, : nr - 1].T[:, :, None]
    oc = packo[None, None, :] * (np.cos(ang) + 1j * np.sin(ang))
    cx, cr, oc = np.broadcast_arrays(cx, cr, oc)
    keep = (cr > 0).ravel()
    cx, cr, oc = cx.ravel()[keep], cr.ravel()[keep], oc.ravel()[keep]
    return np.vstack([cx, cr * oc.imag, cr * oc.real, cr])
