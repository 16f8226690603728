"""Checkpoints of a run: the reference's drop_snap / read_snap
(moduls/chimera_main.py:325-410) with the same key layout, written as a
numpy ``.npz`` archive instead of HDF5 (h5py is not a dependency).

Keys: ``solver<i>/Data/<key>``, ``solver<i>/Args/<key>``,
``specie<i>/Data/<key>``, ``specie<i>/Args/<key>``, ``NumSolvers``,
``NumSpecies``, ``NumThreads``, and ``specie<i>/chunks`` (the x-chunk
boundaries, which the reference leaves out).  As in the reference, list /
tuple / set / dict values are skipped; so are values numpy cannot store
without pickling (functions, None, objects).  Device tensors are copied to
the host.

Reading restores every stored key of the run's current ``Data`` / ``Args``:
grids are copied into the existing device tensors (their Fortran layout is
kept), particle stores are resized to the stored particle count, arrays and
scalars of ``Args`` are replaced.

This module restates the reference's GPLv3-licensed Python layer
(hightower8083/chimera) statement by statement to keep its API as a
drop-in; it is a derivative of that code and is distributed under the GNU
General Public License, version 3 or later, as the reference is.
"""
from __future__ import annotations

import os
import time

import numpy as np
import torch

_SKIP = (list, tuple, set, dict)


def skipped(v) -> bool:
    """True for the values drop_snap does not write."""
    if isinstance(v, _SKIP) or v is None or callable(v):
        return True
    if isinstance(v, torch.Tensor):
        return False
    if isinstance(v, np.ndarray):
        return v.dtype == object
    return not isinstance(v, (bool, int, float, complex, str, np.generic))


def storable(v):
    """The value drop_snap writes for v, or None when v is skipped."""
    if skipped(v):
        return None
    if isinstance(v, torch.Tensor):
        return v.detach().cpu().numpy()
    if isinstance(v, np.ndarray):
        return None if v.dtype == object else v
    if isinstance(v, (bool, int, float, complex, str, np.generic)):
        return np.asarray(v)
    return None


def snap_arrays(solvers, species, verbose=False) -> dict:
    """name -> array for every storable Data / Args entry (drop_snap's keys)."""
    out = {}
    for kind, comps in (("solver", solvers), ("specie", species)):
        for i, comp in enumerate(comps):
            for part in ("Data", "Args"):
                for key, val in getattr(comp, part).items():
                    v = storable(val)
                    if v is None:
                        continue
                    name = f"{kind}{i}/{part}/{key}"
                    if verbose:
                        print("/" + name)
                    out[name] = v
            # the x-chunk boundaries of a chunked species (an attribute, not
            # Data: stored too, so that a restart deposits with them)
            ch = storable(getattr(comp, "chunks", None)) if kind == "specie" else None
            if ch is not None:
                out[f"specie{i}/chunks"] = ch
    out["NumSolvers"] = np.asarray(len(solvers))
    out["NumSpecies"] = np.asarray(len(species))
    out["NumThreads"] = np.asarray(int(os.environ.get("OMP_NUM_THREADS", os.cpu_count() or 1)))
    return out


def snap_name(fname: str) -> str:
    """drop_snap's file name: the prefix, the local time, '.npz'."""
    return fname + time.ctime().replace(" ", "_").replace(":", "-") + ".npz"


def write(fname: str, arrays: dict) -> str:
    with open(fname, "wb") as f:
        np.savez(f, **arrays)
    return fname


def _restore_arg(old, new: np.ndarray):
    if isinstance(old, np.ndarray):
        return np.asfortranarray(new) if new.ndim > 1 else np.array(new)
    if isinstance(old, torch.Tensor):
        t = torch.from_numpy(np.ascontiguousarray(new)).to(old.device, old.dtype)
        return t
    if new.ndim == 0:
        v = new.item()
        if isinstance(old, bool):
            return bool(v)
        if isinstance(old, int) and not isinstance(old, bool):
            return int(v)
        if isinstance(old, float):
            return float(v)
        if isinstance(old, str):
            return str(v)
        return v
    return new


def _copy_into(t: torch.Tensor, a: np.ndarray, what: str):
    if tuple(t.shape) != tuple(a.shape):
        raise ValueError(f"{what}: stored shape {a.shape} differs from the run's {tuple(t.shape)}")
    t.copy_(torch.from_numpy(np.ascontiguousarray(a)).to(t.dtype))


def read_into(f, solvers, species, verbose=False):
    """read_snap: restore the stored entries of Data / Args (f: an NpzFile)."""
    ns, nsp = int(f["NumSolvers"]), int(f["NumSpecies"])
    for i in range(ns):
        solver = solvers[i]
        name = f"solver{i}/"
        for key, val in list(solver.Data.items()):
            k = name + "Data/" + key
            if skipped(val) or k not in f.files:
                continue
            if verbose:
                print("/" + k)
            if isinstance(val, torch.Tensor):
                _copy_into(val, f[k], k)
            else:
                solver.Data[key] = _restore_arg(val, f[k])
        for key, val in list(solver.Args.items()):
            k = name + "Args/" + key
            if skipped(val) or k not in f.files:
                continue
            if verbose:
                print("/" + k)
            solver.Args[key] = _restore_arg(val, f[k])
    for i in range(nsp):
        sp = species[i]
        name = f"specie{i}/"
        n = int(f[name + "Data/weights"].shape[-1])
        sp.store.resize(n)
        sp._sync()
        for key, val in list(sp.Data.items()):
            k = name + "Data/" + key
            if skipped(val) or k not in f.files:
                continue
            if verbose:
                print("/" + k)
            if isinstance(val, torch.Tensor):
                _copy_into(val, f[k], k)
            else:
                sp.Data[key] = _restore_arg(val, f[k])
        for key, val in list(sp.Args.items()):
            k = name + "Args/" + key
            if skipped(val) or k not in f.files:
                continue
            if verbose:
                print("/" + k)
            sp.Args[key] = _restore_arg(val, f[k])
        k = name + "chunks"
        if k in f.files:
            sp.chunks = torch.from_numpy(np.ascontiguousarray(f[k])).to(sp.device)
        else:
            sp.chunks = None
