"""Drop-in replacement of the reference's f2py module ``chimera.moduls.fimera``.

Same function names, argument order and f2py return convention
(``intent(in,out)`` arrays are returned; callers rebind them, e.g.
``Data['J'] = fimera.dep_curr(...)``), but every array argument is a torch
CUDA tensor and every call launches sm_103a kernels of libchimera_gb300.so
through its C ABI on the current torch CUDA stream.

Array conventions (those of the reference's Python layer):
  - particle arrays are (3, Np) / (6, Np) / (Np,) float64 tensors with any
    strides (the structure-of-arrays buffers of ``Specie`` use part stride 1);
  - grid / spectral arrays are complex128 tensors in Fortran order
    (``chimera_gb300.fortran_empty``); a non-Fortran-ordered grid raises
    instead of being silently copied (f2py would copy);
  - small parameter arrays (Rgrid, kx, In/Out, DpS2S, lims, ...) may be numpy
    arrays; they are uploaded on every call, so hot loops pass device copies.

There is no CPU path: a call with CPU tensors or without the built library
raises.
"""
from __future__ import annotations

import ctypes as C

import numpy as np
import torch

from . import _lib
from ._lib import ChimeraError

__all__ = [
    "push_velocs", "push_coords", "proj_fld", "proj_fld_env", "eb_correction",
    "eb_correction_env", "dep_curr", "dep_dens", "dep_curr_env", "dep_dens_env",
    "dep_curr_chnk", "dep_dens_chnk", "dep_curr_env_chnk", "dep_dens_env_chnk",
    "fb_vec_in", "fb_scl_in", "fb_vec_out", "fb_scl_out", "fb_eb_out", "fb_filtr",
    "fb_rot", "fb_grad", "fb_div", "fb_graddiv", "fb_rot_env", "fb_grad_env",
    "fb_div_env", "fb_graddiv_env", "maxwell_push_with_spchrg",
    "maxwell_push_wo_spchrg", "maxwell_init_push", "poiss_corr", "poiss_corr_stat",
    "field_drift", "omp_mult_vec", "omp_mult_scl", "omp_add_vec", "omp_add_scl",
    "undul_analytic", "undul_analytic_taper", "undul_mapped", "undul_mapped_tap",
    "planewave", "gaussbeam", "sortpartsout", "chunk_coords_boundaries",
    "align_data_vec", "align_data_scl", "chunk_order", "intens_profo",
]


# ---------------------------------------------------------------------------
# tensor helpers
# ---------------------------------------------------------------------------

def fortran_empty(shape, dtype=torch.complex128, device="cuda"):
    """Uninitialised tensor with Fortran (column-major) strides."""
    shape = tuple(int(s) for s in shape)
    return torch.empty(shape[::-1], dtype=dtype, device=device).permute(
        *reversed(range(len(shape))))


def fortran_zeros(shape, dtype=torch.complex128, device="cuda"):
    t = fortran_empty(shape, dtype, device)
    t.zero_()
    return t


def is_fortran(t: torch.Tensor) -> bool:
    exp = 1
    for size, st in zip(t.shape, t.stride()):
        if size != 1 and st != exp:
            return False
        exp *= size
    return True


def to_device(a, dtype, device=None) -> torch.Tensor:
    """Tensor on the CUDA device in Fortran order (numpy inputs uploaded)."""
    device = device or torch.device("cuda", torch.cuda.current_device())
    if isinstance(a, torch.Tensor):
        t = a
        if t.device.type != "cuda":
            t = t.to(device)
        if t.dtype != dtype:
            raise ChimeraError(f"expected dtype {dtype}, got {t.dtype}")
        if not is_fortran(t):
            raise ChimeraError("array must be Fortran-contiguous")
        return t
    arr = np.asfortranarray(np.asarray(a), dtype=_np_dtype(dtype))
    return torch.from_numpy(arr).to(device)


def _np_dtype(dtype):
    return {torch.float64: np.float64, torch.complex128: np.complex128,
            torch.int32: np.int32, torch.int64: np.int64, torch.int8: np.int8}[dtype]


def _cuda(t: torch.Tensor, what: str, dtype=torch.float64) -> torch.Tensor:
    if not isinstance(t, torch.Tensor) or t.device.type != "cuda":
        raise ChimeraError(f"{what}: expected a CUDA tensor (there is no CPU path)")
    if t.dtype != dtype:
        raise ChimeraError(f"{what}: expected {dtype}, got {t.dtype}")
    return t


def _parts(t: torch.Tensor, ncomp: int, what: str):
    """(ptr, comp_stride, part_stride, np) of a (ncomp, Np) particle array."""
    _cuda(t, what)
    if t.dim() != 2 or t.shape[0] != ncomp:
        raise ChimeraError(f"{what}: expected shape ({ncomp}, Np), got {tuple(t.shape)}")
    return t.data_ptr(), t.stride(0), t.stride(1), t.shape[1]


def _vec1(t: torch.Tensor, what: str):
    _cuda(t, what)
    if t.dim() != 1:
        raise ChimeraError(f"{what}: expected a 1-d array")
    return t.data_ptr(), t.stride(0), t.shape[0]


def _grid(t: torch.Tensor, what: str, ndim=(3, 4)):
    _cuda(t, what, torch.complex128)
    if t.dim() not in ndim:
        raise ChimeraError(f"{what}: expected {ndim}-d grid, got {tuple(t.shape)}")
    if not is_fortran(t):
        raise ChimeraError(f"{what}: grid must be Fortran-contiguous (fortran_empty)")
    return t


def _stream():
    return torch.cuda.current_stream().cuda_stream


_ws_cache: dict = {}

# host<->device bytes moved by the shim and the drop-in classes (particle
# injection, particle counts read back); the benchmark reports them.
io_bytes = {"h2d": 0, "d2h": 0}


def workspace(nbytes: int, device=None) -> torch.Tensor:
    """Scratch buffer for the C ABI (grown on demand, reused across calls)."""
    device = device or torch.device("cuda", torch.cuda.current_device())
    key = (device.index, torch.cuda.current_stream(device).cuda_stream)
    buf = _ws_cache.get(key)
    if buf is None or buf.numel() < nbytes:
        buf = torch.empty(max(int(nbytes), 256), dtype=torch.uint8, device=device)
        _ws_cache[key] = buf
    return buf


def _check_same_np(*nps):
    if len(set(nps)) != 1:
        raise ChimeraError(f"particle arrays disagree on Np: {nps}")


# ---------------------------------------------------------------------------
# particle_tools.f90
# ---------------------------------------------------------------------------

def push_velocs(momenta, Fld, dt):
    """particle_tools.f90:18-56"""
    p, pcs, pps, n = _parts(momenta, 3, "momenta")
    f, fcs, fps, nf = _parts(Fld, 6, "Fld")
    _check_same_np(n, nf)
    _lib.call("chm_push_velocs", p, pcs, pps, f, fcs, fps, float(dt), n, _stream())
    return momenta


def push_coords(coord, momenta, coord_cntr, dt):
    """particle_tools.f90:58-82"""
    x, xcs, xps, n = _parts(coord, 3, "coord")
    p, pcs, pps, n2 = _parts(momenta, 3, "momenta")
    h, hcs, hps, n3 = _parts(coord_cntr, 3, "coord_cntr")
    _check_same_np(n, n2, n3)
    _lib.call("chm_push_coords", x, xcs, xps, p, pcs, pps, h, hcs, hps, float(dt), n, _stream())
    return coord, coord_cntr


def sortpartsout(coord, lims):
    """particle_tools.f90:130-153 -> (indx2stay int64 CUDA tensor, num2stay)"""
    x, xcs, xps, n = _parts(coord, 3, "coord")
    idx = torch.zeros(max(n, 1), dtype=torch.int64, device=coord.device)[:n]
    num = C.c_int64(0)
    limsh = np.ascontiguousarray(np.asarray(lims, dtype=np.float64).ravel()[:4])
    ws = workspace(_lib.query("chm_sortpartsout_ws_bytes", n))
    _lib.call("chm_sortpartsout", idx.data_ptr(), C.addressof(num), x, xcs, xps,
              limsh.ctypes.data, n, ws.data_ptr(), ws.numel(), _stream())
    io_bytes["d2h"] += 4
    return idx, int(num.value)


def chunk_coords_boundaries(coord, lims, Xgrid, nchnk):
    """particle_tools.f90:155-208 -> (chunked_indx int8, IndInChnk int32, GoOut)"""
    x, xcs, xps, n = _parts(coord, 3, "coord")
    xg = np.asarray(Xgrid.cpu() if isinstance(Xgrid, torch.Tensor) else Xgrid, dtype=np.float64)
    nx = xg.size - 1
    nchnk = int(nchnk)
    xgc = xg[(nx + 1) // nchnk] if nchnk > 1 else xg[nx]
    ids = torch.empty(max(n, 1), dtype=torch.int8, device=coord.device)[:n]
    ind = torch.zeros(nchnk + 1, dtype=torch.int32, device=coord.device)
    go = C.c_int64(0)
    limsh = np.ascontiguousarray(np.asarray(lims, dtype=np.float64).ravel()[:4])
    ws = workspace(4 * (nchnk + 2) + 256)
    _lib.call("chm_chunk_coords_boundaries", ids.data_ptr(), ind.data_ptr(), C.addressof(go), x,
              xcs, xps, limsh.ctypes.data, float(xg[0]), float(xgc), nchnk, n, ws.data_ptr(),
              ws.numel(), _stream())
    io_bytes["d2h"] += 4
    return ids, ind, int(go.value)


def chunk_order(chunked_indx, nchnk):
    """Stable ``chunked_indx.argsort()[go_out:]`` (species.py:379-383)."""
    _cuda(chunked_indx, "chunked_indx", torch.int8)
    n = chunked_indx.shape[0]
    idx = torch.empty(max(n, 1), dtype=torch.int64, device=chunked_indx.device)
    kept = C.c_int64(0)
    ws = workspace(_lib.query("chm_chunk_order_ws_bytes", n, int(nchnk)))
    _lib.call("chm_chunk_order", idx.data_ptr(), C.addressof(kept), chunked_indx.data_ptr(),
              int(nchnk), n, ws.data_ptr(), ws.numel(), _stream())
    io_bytes["d2h"] += 4
    return idx[: kept.value]


def _align(dat, idx, ncomp):
    idx = idx if isinstance(idx, torch.Tensor) else torch.as_tensor(np.asarray(idx, np.int64))
    idx = idx.to(device=dat.device, dtype=torch.int64).contiguous()
    n = idx.shape[0]
    src = dat.clone()
    if ncomp == 1:
        d, dps, _ = _vec1(dat, "dat")
        s, sps, _ = _vec1(src, "dat")
        dcs = scs = 0
    else:
        d, dcs, dps, _ = _parts(dat, ncomp, "dat")
        s, scs, sps, _ = _parts(src, ncomp, "dat")
    _lib.call("chm_align_data", d, dcs, dps, s, scs, sps, ncomp, idx.data_ptr(), n, _stream())
    return dat


def _align_into(dst, src, idx, ncomp):
    idx = idx.to(device=src.device, dtype=torch.int64).contiguous()
    n = idx.shape[0]
    if ncomp == 1:
        d, dps, nd = _vec1(dst, "dst")
        s, sps, _ = _vec1(src, "src")
        dcs = scs = 0
    else:
        d, dcs, dps, nd = _parts(dst, ncomp, "dst")
        s, scs, sps, _ = _parts(src, ncomp, "src")
    if nd < n:
        raise ChimeraError("align_data: destination too small")
    _lib.call("chm_align_data", d, dcs, dps, s, scs, sps, ncomp, idx.data_ptr(), n, _stream())
    return dst


def align_data_vec_into(dst, src, idx):
    """dst(:, i) = src(:, idx(i)) for i < len(idx); dst and src distinct."""
    return _align_into(dst, src, idx, 3)


def align_data_scl_into(dst, src, idx):
    return _align_into(dst, src, idx, 1)


def align_data_vec(dat, chunked_indx):
    """particle_tools.f90:270-296: dat(:, i) = dat(:, idx(i)) for i < len(idx)"""
    return _align(dat, chunked_indx, 3)


def align_data_scl(dat, chunked_indx):
    """particle_tools.f90:298-324"""
    return _align(dat, chunked_indx, 1)


# ---------------------------------------------------------------------------
# grid_deps*.f90
# ---------------------------------------------------------------------------

def _dims(g):
    return g.shape[0], g.shape[1], g.shape[2]


def _dep(kind, coord, momenta, wghts, grid, leftX, Rgrid, dx_inv, dr_inv, kx0=None,
         IndInChunk=None, guards=0):
    ncomp = 3 if kind.startswith("curr") else 1
    g = _grid(grid, "grid", (4,) if ncomp == 3 else (3,))
    x, xcs, xps, n = _parts(coord, 3, "coord")
    w, wps, nw = _vec1(wghts, "wghts")
    _check_same_np(n, nw)
    nx, nr, nm = _dims(g)
    rg = to_device(Rgrid, torch.float64, g.device)
    if rg.numel() != nr:
        raise ChimeraError(f"Rgrid has {rg.numel()} entries, grid has nr={nr}")
    ws = workspace(_lib.query("chm_dep_ws_bytes", nx, nr, nm, ncomp, n))
    args = [x, xcs, xps]
    if ncomp == 3:
        p, pcs, pps, n2 = _parts(momenta, 3, "momenta")
        _check_same_np(n, n2)
        args += [p, pcs, pps]
    args += [w, wps, g.data_ptr()]
    name = "chm_dep_" + kind
    if IndInChunk is not None:
        ind = to_device(IndInChunk, torch.int32, g.device)
        args += [ind.data_ptr(), ind.numel() - 1, int(guards)]
        name += "_chnk"
    args += [float(leftX), rg.data_ptr(), float(dx_inv), float(dr_inv)]
    if kx0 is not None:
        args += [float(kx0)]
    args += [n, nx, nr, nm, ws.data_ptr(), ws.numel(), _stream()]
    _lib.call(name, *args)
    return grid


def dep_curr(coord, momenta, wghts, curr, leftX, Rgrid, dx_inv, dr_inv):
    """grid_deps.f90:18-87"""
    return _dep("curr", coord, momenta, wghts, curr, leftX, Rgrid, dx_inv, dr_inv)


def dep_dens(coord, wghts, dens, leftX, Rgrid, dx_inv, dr_inv):
    """grid_deps.f90:89-147"""
    return _dep("dens", coord, None, wghts, dens, leftX, Rgrid, dx_inv, dr_inv)


def dep_curr_env(coord, momenta, wghts, curr, leftX, Rgrid, dx_inv, dr_inv, kx0):
    """grid_deps_env.f90:18-95"""
    return _dep("curr_env", coord, momenta, wghts, curr, leftX, Rgrid, dx_inv, dr_inv, kx0)


def dep_dens_env(coord, wghts, dens, leftX, Rgrid, dx_inv, dr_inv, kx0):
    """grid_deps_env.f90:97-162"""
    return _dep("dens_env", coord, None, wghts, dens, leftX, Rgrid, dx_inv, dr_inv, kx0)


def dep_curr_chnk(coord, momenta, wghts, curr, IndInChunk, guards, leftX, Rgrid, dx_inv,
                  dr_inv):
    """grid_deps_chnk.f90:18-130"""
    return _dep("curr", coord, momenta, wghts, curr, leftX, Rgrid, dx_inv, dr_inv,
                IndInChunk=IndInChunk, guards=guards)


def dep_dens_chnk(coord, wghts, dens, IndInChunk, guards, leftX, Rgrid, dx_inv, dr_inv):
    """grid_deps_chnk.f90:132-234"""
    return _dep("dens", coord, None, wghts, dens, leftX, Rgrid, dx_inv, dr_inv,
                IndInChunk=IndInChunk, guards=guards)


def dep_curr_env_chnk(coord, momenta, wghts, curr, IndInChunk, guards, leftX, Rgrid, dx_inv,
                      dr_inv, kx0):
    """grid_deps_env_chnk.f90:18-145"""
    return _dep("curr_env", coord, momenta, wghts, curr, leftX, Rgrid, dx_inv, dr_inv, kx0,
                IndInChunk=IndInChunk, guards=guards)


def dep_dens_env_chnk(coord, wghts, dens, IndInChunk, guards, leftX, Rgrid, dx_inv, dr_inv,
                      kx0):
    """grid_deps_env_chnk.f90:147-261"""
    return _dep("dens_env", coord, None, wghts, dens, leftX, Rgrid, dx_inv, dr_inv, kx0,
                IndInChunk=IndInChunk, guards=guards)


def _proj(env, coord, wghts, Fld, Fld_tot, leftX, Rgrid, dx_inv, dr_inv, kx0=0.0):
    g = _grid(Fld, "Fld", (4,))
    x, xcs, xps, n = _parts(coord, 3, "coord")
    w, wps, nw = _vec1(wghts, "wghts")
    f, fcs, fps, nf = _parts(Fld_tot, 6, "Fld_tot")
    _check_same_np(n, nw, nf)
    nx, nr, nm = _dims(g)
    rg = to_device(Rgrid, torch.float64, g.device)
    if env:
        _lib.call("chm_proj_fld_env", x, xcs, xps, w, wps, g.data_ptr(), f, fcs, fps,
                  float(leftX), rg.data_ptr(), float(dx_inv), float(dr_inv), float(kx0), n, nx,
                  nr, nm, _stream())
    else:
        _lib.call("chm_proj_fld", x, xcs, xps, w, wps, g.data_ptr(), f, fcs, fps, float(leftX),
                  rg.data_ptr(), float(dx_inv), float(dr_inv), n, nx, nr, nm, _stream())
    return Fld_tot


def proj_fld(coord, wghts, Fld, Fld_tot, leftX, Rgrid, dx_inv, dr_inv):
    """grid_deps.f90:149-217"""
    return _proj(False, coord, wghts, Fld, Fld_tot, leftX, Rgrid, dx_inv, dr_inv)


def proj_fld_env(coord, wghts, Fld, Fld_tot, leftX, Rgrid, dx_inv, dr_inv, kx0):
    """grid_deps_env.f90:164-238"""
    return _proj(True, coord, wghts, Fld, Fld_tot, leftX, Rgrid, dx_inv, dr_inv, kx0)


def eb_correction(eb_spc):
    """grid_deps.f90:219-266"""
    g = _grid(eb_spc, "eb_spc", (4,))
    _lib.call("chm_eb_correction", g.data_ptr(), *_dims(g), _stream())
    return eb_spc


def eb_correction_env(eb_spc):
    """grid_deps_env.f90:240-283"""
    g = _grid(eb_spc, "eb_spc", (4,))
    _lib.call("chm_eb_correction_env", g.data_ptr(), *_dims(g), _stream())
    return eb_spc


# ---------------------------------------------------------------------------
# fb_io.f90
# ---------------------------------------------------------------------------

def _fb_in(vec_fb, vec, leftX, kx, In, ncomp, fact=None):
    out = _grid(vec_fb, "vec_fb")
    v = _grid(vec, "vec")
    nx, nr, nm = _dims(v)
    In_ = to_device(In, torch.float64, v.device)
    nkr = In_.shape[1]
    if tuple(out.shape[:3]) != (nx, nkr, nm) or In_.shape[0] != nr - 1:
        raise ChimeraError("fb_in: inconsistent shapes")
    kx_ = to_device(kx, torch.float64, v.device)
    # device copies stay bound until the call is enqueued (a freed temporary
    # could be handed to the workspace allocation below)
    fac_t = to_device(fact, torch.float64, v.device) if fact is not None else None
    ws = workspace(_lib.query("chm_fb_ws_bytes", nx, nr, nkr, nm, ncomp))
    _lib.call("chm_fb_in", out.data_ptr(), v.data_ptr(), float(leftX), kx_.data_ptr(),
              In_.data_ptr(), fac_t.data_ptr() if fac_t is not None else None, nx, nr, nkr, nm,
              ncomp, ws.data_ptr(), ws.numel(), _stream())
    return vec_fb


def fb_vec_in(vec_fb, vec, leftX, kx, In):
    """fb_io.f90:18-59"""
    return _fb_in(vec_fb, vec, leftX, kx, In, 3)


def fb_scl_in(scl_fb, scl, leftX, kx, In):
    """fb_io.f90:61-98"""
    return _fb_in(scl_fb, scl, leftX, kx, In, 1)


def _fb_out(vec_fb, leftX, kx, Out, ncomp, out=None, eb_mode=0):
    vfb = _grid(vec_fb, "vec_fb")
    nx, nkr, nm = _dims(vfb)
    Out_ = to_device(Out, torch.float64, vfb.device)
    nr = Out_.shape[1] + 1
    if out is None:
        out = fortran_empty((nx, nr, nm) + ((ncomp,) if ncomp > 1 else ()), device=vfb.device)
    kx_ = to_device(kx, torch.float64, vfb.device)
    ws = workspace(_lib.query("chm_fb_ws_bytes", nx, nr, nkr, nm, ncomp))
    _lib.call("chm_fb_out", out.data_ptr(), vfb.data_ptr(), float(leftX), kx_.data_ptr(),
              Out_.data_ptr(), nx, nr, nkr, nm, ncomp, int(eb_mode), ws.data_ptr(), ws.numel(),
              _stream())
    return out


def fb_vec_out(vec_fb, leftX, kx, Out):
    """fb_io.f90:100-140 (intent(out) vec)"""
    return _fb_out(vec_fb, leftX, kx, Out, 3)


def fb_scl_out(scl_fb, leftX, kx, Out):
    """fb_io.f90:142-180"""
    return _fb_out(scl_fb, leftX, kx, Out, 1)


def fb_eb_out(eb_spc, e_fb, b_fb, leftX, kx, Out, eb_mode=0):
    """fb_io.f90:182-228.  ``eb_mode`` 1/2 fuses eb_correction(_env)."""
    eb = _grid(eb_spc, "eb_spc", (4,))
    e = _grid(e_fb, "e_fb", (4,))
    b = _grid(b_fb, "b_fb", (4,))
    nx, nr, nm = _dims(eb)
    nkr = e.shape[1]
    Out_ = to_device(Out, torch.float64, eb.device)
    kx_ = to_device(kx, torch.float64, eb.device)
    ws = workspace(_lib.query("chm_fb_ws_bytes", nx, nr, nkr, nm, 3))
    _lib.call("chm_fb_eb_out", eb.data_ptr(), e.data_ptr(), b.data_ptr(), float(leftX),
              kx_.data_ptr(), Out_.data_ptr(), nx, nr, nkr, nm, int(eb_mode), ws.data_ptr(),
              ws.numel(), _stream())
    return eb_spc


def fb_filtr(vec, leftX, kx, filtr, modefilt):
    """fb_io.f90:230-308"""
    v = _grid(vec, "vec", (4,))
    nx, nkr, nm = _dims(v)
    f = to_device(filtr, torch.float64, v.device)
    kx_ = to_device(kx, torch.float64, v.device)
    ws = workspace(2 * 16 * nx + 1024)
    _lib.call("chm_fb_filtr", v.data_ptr(), float(leftX), kx_.data_ptr(), f.data_ptr(),
              f.numel(), int(modefilt), nx, nkr, nm, v.shape[3], ws.data_ptr(), ws.numel(),
              _stream())
    return vec


# ---------------------------------------------------------------------------
# fb_math*.f90
# ---------------------------------------------------------------------------

def _fbm(name, env, out, inp, DpS2S, DmS2S, kx):
    o = _grid(out, "out")
    i = _grid(inp, "in")
    nx, nkr, nm = _dims(i)
    Dp = to_device(DpS2S, torch.float64, i.device)
    Dm = to_device(DmS2S, torch.float64, i.device)
    kx_ = to_device(kx, torch.float64, i.device)
    need = nm + (2 if env else 1)
    if Dp.shape[2] < need or Dm.shape[2] < need or Dp.shape[0] != nkr:
        raise ChimeraError(f"{name}: DpS2S/DmS2S need ({nkr},{nkr},>={need}) modes")
    ws = workspace(_lib.query("chm_fbmath_ws_bytes", nx, nkr, nm))
    _lib.call(name, o.data_ptr(), i.data_ptr(), Dp.data_ptr(), Dm.data_ptr(), kx_.data_ptr(),
              nx, nkr, nm, int(env), ws.data_ptr(), ws.numel(), _stream())
    return out


def fb_rot(vec_fb_loc, vec_fb, DpS2S, DmS2S, kx):
    """fb_math.f90:18-94"""
    return _fbm("chm_fb_rot", 0, vec_fb_loc, vec_fb, DpS2S, DmS2S, kx)


def fb_grad(vec_fb_loc, scl_fb, DpS2S, DmS2S, kx):
    """fb_math.f90:96-149"""
    return _fbm("chm_fb_grad", 0, vec_fb_loc, scl_fb, DpS2S, DmS2S, kx)


def fb_div(scl_fb_loc, vec_fb, DpS2S, DmS2S, kx):
    """fb_math.f90:151-199"""
    return _fbm("chm_fb_div", 0, scl_fb_loc, vec_fb, DpS2S, DmS2S, kx)


def fb_rot_env(vec_fb_loc, vec_fb, DpS2S, DmS2S, kx):
    """fb_math_env.f90:106-162"""
    return _fbm("chm_fb_rot", 1, vec_fb_loc, vec_fb, DpS2S, DmS2S, kx)


def fb_grad_env(vec_fb_loc, scl_fb, DpS2S, DmS2S, kx):
    """fb_math_env.f90:18-61"""
    return _fbm("chm_fb_grad", 1, vec_fb_loc, scl_fb, DpS2S, DmS2S, kx)


def fb_div_env(scl_fb_loc, vec_fb, DpS2S, DmS2S, kx):
    """fb_math_env.f90:63-104"""
    return _fbm("chm_fb_div", 1, scl_fb_loc, vec_fb, DpS2S, DmS2S, kx)


def _graddiv(env, vec_fb, DpS2S, DmS2S, kx):
    v = _grid(vec_fb, "vec_fb", (4,))
    nx, nkr, nm = _dims(v)
    Dp = to_device(DpS2S, torch.float64, v.device)
    Dm = to_device(DmS2S, torch.float64, v.device)
    kx_ = to_device(kx, torch.float64, v.device)
    ws = workspace(_lib.query("chm_fbmath_ws_bytes", nx, nkr, nm))
    _lib.call("chm_fb_graddiv", v.data_ptr(), Dp.data_ptr(), Dm.data_ptr(), kx_.data_ptr(), nx,
              nkr, nm, int(env), ws.data_ptr(), ws.numel(), _stream())
    return vec_fb


def fb_graddiv(vec_fb, DpS2S, DmS2S, kx):
    """fb_math.f90:201-293"""
    return _graddiv(0, vec_fb, DpS2S, DmS2S, kx)


def fb_graddiv_env(vec_fb, DpS2S, DmS2S, kx):
    """fb_math_env.f90:164-233"""
    return _graddiv(1, vec_fb, DpS2S, DmS2S, kx)


# ---------------------------------------------------------------------------
# maxwell_solvers.f90
# ---------------------------------------------------------------------------

def _spec(t, what):
    g = _grid(t, what, (4,))
    return g.data_ptr(), g.shape[0], g.shape[1], g.shape[2]


def maxwell_push_with_spchrg(EG_fb, j_fb, grad_rho_n_fb, grad_rho_np1_fb, C1, C2):
    """maxwell_solvers.f90:18-60 (real C1, C2)"""
    eg, nx, nkr, nm = _spec(EG_fb, "EG_fb")
    c1 = to_device(C1, torch.float64, EG_fb.device)
    c2 = to_device(C2, torch.float64, EG_fb.device)
    _lib.call("chm_maxwell_push_with_spchrg", eg, _grid(j_fb, "j").data_ptr(),
              _grid(grad_rho_n_fb, "gn").data_ptr(), _grid(grad_rho_np1_fb, "gnp1").data_ptr(),
              c1.data_ptr(), c2.data_ptr(), nx, nkr, nm, _stream())
    return EG_fb


def _complex_coef(C, dev):
    if isinstance(C, torch.Tensor) and C.dtype == torch.float64:
        C = C.to(torch.complex128)
        if not is_fortran(C):
            C = to_device(C.cpu().numpy(), torch.complex128, dev)
    return to_device(C, torch.complex128, dev)


def maxwell_push_wo_spchrg(EG_fb, j_fb, C1, C2):
    """maxwell_solvers.f90:62-96 (complex C1, C2; real ones are cast as f2py does)"""
    eg, nx, nkr, nm = _spec(EG_fb, "EG_fb")
    c1 = _complex_coef(C1, EG_fb.device)
    c2 = _complex_coef(C2, EG_fb.device)
    _lib.call("chm_maxwell_push_wo_spchrg", eg, _grid(j_fb, "j").data_ptr(), c1.data_ptr(),
              c2.data_ptr(), nx, nkr, nm, _stream())
    return EG_fb


def maxwell_init_push(EG_fb, j_fb, grad_rho_n_fb, C1, C2):
    """maxwell_solvers.f90:98-129"""
    eg, nx, nkr, nm = _spec(EG_fb, "EG_fb")
    c1 = _complex_coef(C1, EG_fb.device)
    c2 = _complex_coef(C2, EG_fb.device)
    _lib.call("chm_maxwell_init_push", eg, _grid(j_fb, "j").data_ptr(),
              _grid(grad_rho_n_fb, "gn").data_ptr(), c1.data_ptr(), c2.data_ptr(), nx, nkr, nm,
              _stream())
    return EG_fb


def poiss_corr(j_fb, grad_div_j_fb, grad_rho_n_fb, grad_rho_np1_fb, dt_inv, w2_inv):
    """maxwell_solvers.f90:131-164"""
    j, nx, nkr, nm = _spec(j_fb, "j_fb")
    w2 = to_device(w2_inv, torch.float64, j_fb.device)
    _lib.call("chm_poiss_corr", j, _grid(grad_div_j_fb, "gdj").data_ptr(),
              _grid(grad_rho_n_fb, "gn").data_ptr(), _grid(grad_rho_np1_fb, "gnp1").data_ptr(),
              float(dt_inv), w2.data_ptr(), nx, nkr, nm, _stream())
    return j_fb


def poiss_corr_stat(j_fb, grad_div_j_fb, grad_rho_n_fb, DT, w2_inv):
    """maxwell_solvers.f90:166-197"""
    j, nx, nkr, nm = _spec(j_fb, "j_fb")
    w2 = to_device(w2_inv, torch.float64, j_fb.device)
    dt = to_device(DT, torch.complex128, j_fb.device)
    _lib.call("chm_poiss_corr_stat", j, _grid(grad_div_j_fb, "gdj").data_ptr(),
              _grid(grad_rho_n_fb, "gn").data_ptr(), dt.data_ptr(), w2.data_ptr(), nx, nkr, nm,
              _stream())
    return j_fb


def field_drift(EG_fb, kx, beta0, dt):
    """maxwell_solvers.f90:199-226"""
    eg, nx, nkr, nm = _spec(EG_fb, "EG_fb")
    kx_ = to_device(kx, torch.float64, EG_fb.device)
    _lib.call("chm_field_drift", eg, kx_.data_ptr(), float(beta0), float(dt), nx, nkr, nm,
              _stream())
    return EG_fb


def _mult(v, A, ncomp):
    g = _grid(v, "vec_fb")
    a = to_device(A, torch.float64, v.device)
    P = a.numel()
    if g.numel() != P * ncomp:
        raise ChimeraError("omp_mult: shape mismatch")
    _lib.call("chm_omp_mult", g.data_ptr(), a.data_ptr(), P, ncomp, _stream())
    return v


def omp_mult_vec(vec_fb, A):
    """maxwell_solvers.f90:228-250"""
    return _mult(vec_fb, A, 3)


def omp_mult_scl(scl_fb, A):
    """maxwell_solvers.f90:252-272"""
    return _mult(scl_fb, A, 1)


def omp_add_vec(vec_fb, A):
    """maxwell_solvers.f90:274-296"""
    g = _grid(vec_fb, "vec_fb")
    a = _grid(A, "A") if isinstance(A, torch.Tensor) else to_device(A, torch.complex128, g.device)
    if a.numel() != g.numel():
        raise ChimeraError("omp_add: shape mismatch")
    _lib.call("chm_omp_add", g.data_ptr(), a.data_ptr(), g.numel(), _stream())
    return vec_fb


def omp_add_scl(scl_fb, A):
    """maxwell_solvers.f90:298-318"""
    return omp_add_vec(scl_fb, A)


# ---------------------------------------------------------------------------
# devices.f90
# ---------------------------------------------------------------------------

def _host_params(params, n):
    p = np.zeros(8, dtype=np.float64)
    a = np.asarray(params.cpu() if isinstance(params, torch.Tensor) else params,
                   dtype=np.float64).ravel()
    if a.size < n:
        raise ChimeraError(f"device needs {n} parameters, got {a.size}")
    p[: min(8, a.size)] = a[:8]
    return p


def _device(name, nparams, coord, Fld, t, params, extra=()):
    x, xcs, xps, n = _parts(coord, 3, "coord")
    f, fcs, fps, nf = _parts(Fld, 6, "Fld")
    _check_same_np(n, nf)
    p = _host_params(params, nparams)
    _lib.call(name, x, xcs, xps, f, fcs, fps, float(t), *extra, p.ctypes.data, n, _stream())
    return Fld


def undul_analytic(coord, Fld, t, params):
    """devices.f90:162-203"""
    return _device("chm_undul_analytic", 4, coord, Fld, t, params)


def undul_analytic_taper(coord, Fld, t, params):
    """devices.f90:117-160"""
    return _device("chm_undul_analytic_taper", 5, coord, Fld, t, params)


def undul_mapped(coord, Fld, t, a0, params):
    """devices.f90:18-62"""
    a = to_device(a0, torch.float64, Fld.device)
    return _device("chm_undul_mapped", 3, coord, Fld, t, params, (a.data_ptr(), a.shape[1]))


def undul_mapped_tap(coord, Fld, t, a0, params):
    """devices.f90:64-115"""
    a = to_device(a0, torch.float64, Fld.device)
    return _device("chm_undul_mapped_tap", 5, coord, Fld, t, params, (a.data_ptr(), a.shape[1]))


def planewave(coord, Fld, t, params):
    """devices.f90:205-252"""
    return _device("chm_planewave", 7, coord, Fld, t, params)


def gaussbeam(coord, Fld, time, a0, params):
    """devices.f90:254-297"""
    x, xcs, xps, n = _parts(coord, 3, "coord")
    f, fcs, fps, nf = _parts(Fld, 6, "Fld")
    _check_same_np(n, nf)
    p = _host_params(params, 8)
    _lib.call("chm_gaussbeam", x, xcs, xps, f, fcs, fps, float(time), float(a0), p.ctypes.data,
              n, _stream())
    return Fld


# ---------------------------------------------------------------------------
# utils.f90 and the Diagnostics reductions
# ---------------------------------------------------------------------------

def intens_profo(Fld, NO):
    """utils.f90:18-57: PWR_RO (NO, nr) float64 from Fld (nx+1, nr+1,
    2 nkO + 1, 3) complex128 (f2py infers nkO, so the mode extent is odd)."""
    f = _grid(Fld, "Fld", (4,))
    NX, NR, NM, nc = f.shape
    if nc != 3 or NM % 2 != 1:
        raise ChimeraError("intens_profo: Fld must be (nx+1, nr+1, 2*nkO+1, 3)")
    out = fortran_empty((int(NO), NR - 1), dtype=torch.float64, device=f.device)
    _lib.call("chm_intens_profo", out.data_ptr(), f.data_ptr(), int(NO), NX, NR, NM, _stream())
    return out


def em_energy(EG_fb, EnergyFact):
    """Electromagnetic energy per kx of diagnostics.py:112-114 (before its
    reordering): sum over kr and modes of EnergyFact * sum_{l<3} |E_l|^2."""
    eg = _grid(EG_fb, "EG_fb", (4,))
    nx, nkr, nm = _dims(eg)
    ef = to_device(EnergyFact, torch.float64, eg.device)
    if tuple(ef.shape) != (nx, nkr, nm):
        raise ChimeraError(f"EnergyFact has shape {tuple(ef.shape)}, expected {(nx, nkr, nm)}")
    out = torch.empty(nx, dtype=torch.float64, device=eg.device)
    _lib.call("chm_em_energy", out.data_ptr(), eg.data_ptr(), ef.data_ptr(), nx, nkr, nm,
              eg.shape[3], _stream())
    return out


def power_profile(dat, Rgrid, fac):
    """Power per x of diagnostics.py:134-143: fac * sum_r Rgrid[r] *
    sum_{m, l} |dat(x, r, m, l)|^2 for a spatial vector field (nx, nr, nm, 3)."""
    v = _grid(dat, "dat", (4,))
    nx, nr, nm = _dims(v)
    if v.shape[3] != 3:
        raise ChimeraError("power_profile: expected a 3-component field")
    rg = to_device(Rgrid, torch.float64, v.device)
    if rg.numel() != nr:
        raise ChimeraError(f"Rgrid has {rg.numel()} entries, field has nr={nr}")
    out = torch.empty(nx, dtype=torch.float64, device=v.device)
    _lib.call("chm_power_profile", out.data_ptr(), v.data_ptr(), rg.data_ptr(), float(fac), nx, nr,
              nm, _stream())
    return out
