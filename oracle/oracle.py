"""CPU FP64 oracle for CHIMERA's per-step PIC kernels -- TEST INFRASTRUCTURE.

This module is the checker.  Only ``tests/``, ``__graft_entry__.smoke()`` and
the ``cpu_baseline`` / ``--impl reference`` legs of ``bench.py`` import it; the
product package ``chimera_gb300`` never does.

It exposes the reference's f2py module surface (``chimera.moduls.fimera``):
the same function names, argument order, ``intent(in,out)`` return
convention and in-place semantics for Fortran-contiguous arrays of the right
dtype, over ``oracle/_build/libchimera_oracle.so`` (``chimera_oracle.c``, a
restatement of the reference's ``f90/*.f90``).  Because of that it can stand
in for the Fortran extension when the reference's own Python layer is run to
produce golden vectors (``tests/golden/make_golden.py``).
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_SO = os.path.join(_HERE, "_build", "libchimera_oracle.so")

c_dp = C.POINTER(C.c_double)
c_i64 = C.c_longlong


def build(force: bool = False) -> str:
    """Compile the oracle with the committed Makefile (gcc + OpenMP)."""
    src = os.path.join(_HERE, "chimera_oracle.c")
    if force or not os.path.exists(_SO) or os.path.getmtime(_SO) < os.path.getmtime(src):
        subprocess.check_call(["make", "-s", "-C", _HERE], stdout=subprocess.DEVNULL)
    return _SO


_lib = None


def lib():
    global _lib
    if _lib is None:
        build()
        _lib = C.CDLL(_SO)
    return _lib


# ---------------------------------------------------------------------------
# helpers
# ---------------------------------------------------------------------------

def _inout(a, dtype):
    """f2py intent(in,out): use the array itself when it is Fortran-contiguous
    with the right dtype, otherwise a Fortran-ordered copy."""
    a = np.asarray(a)
    if a.dtype == np.dtype(dtype) and a.flags.f_contiguous:
        return a
    return np.asfortranarray(a, dtype=dtype)


def _in(a, dtype):
    return np.asfortranarray(a, dtype=dtype)


def _p(a):
    return a.ctypes.data_as(c_dp)


def _vp(a):
    # data_as keeps the array alive for as long as the pointer object lives,
    # so temporaries created inline in a call stay valid during the call
    return a.ctypes.data_as(C.c_void_p)


def _d(x):
    return C.c_double(float(x))


def _n(x):
    return c_i64(int(x))


def _np(coord):
    return coord.shape[1] if coord.ndim == 2 else 0


# ---------------------------------------------------------------------------
# particle_tools.f90
# ---------------------------------------------------------------------------

def push_velocs(momenta, Fld, dt):
    m = _inout(momenta, np.float64)
    f = _in(Fld, np.float64)
    lib().orc_push_velocs(_p(m), _p(f), _d(dt), _n(_np(m)))
    return m


def push_coords(coord, momenta, coord_cntr, dt):
    x = _inout(coord, np.float64)
    p = _in(momenta, np.float64)
    xc = _inout(coord_cntr, np.float64)
    lib().orc_push_coords(_p(x), _p(p), _p(xc), _d(dt), _n(_np(x)))
    return x, xc


def genparts(coord, Xgrid, Rgrid, RandPackO, PackX, PackR, PackO):
    c = _inout(coord, np.float64)
    xg = _in(Xgrid, np.float64)
    rg = _in(Rgrid, np.float64)
    rp = _in(RandPackO, np.float64)
    px = _in(PackX, np.float64)
    pr = _in(PackR, np.float64)
    po = _in(PackO, np.complex128)
    f = lib().orc_genparts
    f.restype = c_i64
    n = f(_p(c), _n(c.shape[1]), _p(xg), _n(xg.size), _p(rg), _n(rg.size), _p(rp),
          _p(px), _p(pr), _vp(po), _n(px.size))
    if n < 0:
        raise ValueError("genparts: coordinate container too small")
    return c, int(n)


def sortpartsout(coord, lims):
    c = _in(coord, np.float64)
    idx = np.zeros(_np(c), dtype=np.int64)
    f = lib().orc_sortpartsout
    f.restype = c_i64
    n = f(_vp(idx), _p(c), _p(_in(lims, np.float64)), _n(_np(c)))
    return idx.astype(np.int32), int(n)


def chunk_coords_boundaries(coord, lims, Xgrid, nchnk):
    c = _in(coord, np.float64)
    xg = _in(Xgrid, np.float64)
    ci = np.zeros(_np(c), dtype=np.int8)
    ind = np.zeros(int(nchnk) + 1, dtype=np.int32)
    f = lib().orc_chunk_coords_boundaries
    f.restype = c_i64
    go = f(_vp(ci), _vp(ind), _p(c), _p(_in(lims, np.float64)), _p(xg), _n(xg.size),
           _n(nchnk), _n(_np(c)))
    return ci, ind, int(go)


def align_data_vec(dat, chunked_indx):
    d = _inout(dat, np.float64)
    idx = np.ascontiguousarray(chunked_indx, dtype=np.int64)
    if idx.size:
        lib().orc_align_data(_p(d), _n(3), _vp(idx), _n(idx.size))
    return d


def align_data_scl(dat, chunked_indx):
    d = _inout(dat, np.float64)
    idx = np.ascontiguousarray(chunked_indx, dtype=np.int64)
    if idx.size:
        lib().orc_align_data(_p(d), _n(1), _vp(idx), _n(idx.size))
    return d


# ---------------------------------------------------------------------------
# grid_deps*.f90
# ---------------------------------------------------------------------------

def _grid_dims(g):
    nx, nr, nm = g.shape[0], g.shape[1], g.shape[2]
    return _n(nx), _n(nr), _n(nm)


def dep_curr(coord, momenta, wghts, curr, leftX, Rgrid, dx_inv, dr_inv):
    g = _inout(curr, np.complex128)
    c = _in(coord, np.float64)
    lib().orc_dep_curr(_p(c), _p(_in(momenta, np.float64)), _p(_in(wghts, np.float64)),
                       _vp(g), _d(leftX), _p(_in(Rgrid, np.float64)), _d(dx_inv),
                       _d(dr_inv), _n(_np(c)), *_grid_dims(g))
    return g


def dep_dens(coord, wghts, dens, leftX, Rgrid, dx_inv, dr_inv):
    g = _inout(dens, np.complex128)
    c = _in(coord, np.float64)
    lib().orc_dep_dens(_p(c), _p(_in(wghts, np.float64)), _vp(g), _d(leftX),
                       _p(_in(Rgrid, np.float64)), _d(dx_inv), _d(dr_inv), _n(_np(c)),
                       *_grid_dims(g))
    return g


def dep_curr_env(coord, momenta, wghts, curr, leftX, Rgrid, dx_inv, dr_inv, kx0):
    g = _inout(curr, np.complex128)
    c = _in(coord, np.float64)
    lib().orc_dep_curr_env(_p(c), _p(_in(momenta, np.float64)), _p(_in(wghts, np.float64)),
                           _vp(g), _d(leftX), _p(_in(Rgrid, np.float64)), _d(dx_inv),
                           _d(dr_inv), _d(kx0), _n(_np(c)), *_grid_dims(g))
    return g


def dep_dens_env(coord, wghts, dens, leftX, Rgrid, dx_inv, dr_inv, kx0):
    g = _inout(dens, np.complex128)
    c = _in(coord, np.float64)
    lib().orc_dep_dens_env(_p(c), _p(_in(wghts, np.float64)), _vp(g), _d(leftX),
                           _p(_in(Rgrid, np.float64)), _d(dx_inv), _d(dr_inv), _d(kx0),
                           _n(_np(c)), *_grid_dims(g))
    return g


def _ind(IndInChunk):
    return np.ascontiguousarray(IndInChunk, dtype=np.int32)


def dep_curr_chnk(coord, momenta, wghts, curr, IndInChunk, guards, leftX, Rgrid,
                  dx_inv, dr_inv):
    g = _inout(curr, np.complex128)
    ind = _ind(IndInChunk)
    lib().orc_dep_curr_chnk(_p(_in(coord, np.float64)), _p(_in(momenta, np.float64)),
                            _p(_in(wghts, np.float64)), _vp(g), _vp(ind), _n(ind.size - 1),
                            _n(guards), _d(leftX), _p(_in(Rgrid, np.float64)), _d(dx_inv),
                            _d(dr_inv), *_grid_dims(g))
    return g


def dep_dens_chnk(coord, wghts, dens, IndInChunk, guards, leftX, Rgrid, dx_inv, dr_inv):
    g = _inout(dens, np.complex128)
    ind = _ind(IndInChunk)
    lib().orc_dep_dens_chnk(_p(_in(coord, np.float64)), _p(_in(wghts, np.float64)), _vp(g),
                            _vp(ind), _n(ind.size - 1), _n(guards), _d(leftX),
                            _p(_in(Rgrid, np.float64)), _d(dx_inv), _d(dr_inv),
                            *_grid_dims(g))
    return g


def dep_curr_env_chnk(coord, momenta, wghts, curr, IndInChunk, guards, leftX, Rgrid,
                      dx_inv, dr_inv, kx0):
    g = _inout(curr, np.complex128)
    ind = _ind(IndInChunk)
    lib().orc_dep_curr_env_chnk(_p(_in(coord, np.float64)), _p(_in(momenta, np.float64)),
                                _p(_in(wghts, np.float64)), _vp(g), _vp(ind),
                                _n(ind.size - 1), _n(guards), _d(leftX),
                                _p(_in(Rgrid, np.float64)), _d(dx_inv), _d(dr_inv),
                                _d(kx0), *_grid_dims(g))
    return g


def dep_dens_env_chnk(coord, wghts, dens, IndInChunk, guards, leftX, Rgrid, dx_inv,
                      dr_inv, kx0):
    g = _inout(dens, np.complex128)
    ind = _ind(IndInChunk)
    lib().orc_dep_dens_env_chnk(_p(_in(coord, np.float64)), _p(_in(wghts, np.float64)),
                                _vp(g), _vp(ind), _n(ind.size - 1), _n(guards), _d(leftX),
                                _p(_in(Rgrid, np.float64)), _d(dx_inv), _d(dr_inv),
                                _d(kx0), *_grid_dims(g))
    return g


def proj_fld(coord, wghts, Fld, Fld_tot, leftX, Rgrid, dx_inv, dr_inv):
    ft = _inout(Fld_tot, np.float64)
    g = _in(Fld, np.complex128)
    c = _in(coord, np.float64)
    lib().orc_proj_fld(_p(c), _p(_in(wghts, np.float64)), _vp(g), _p(ft), _d(leftX),
                       _p(_in(Rgrid, np.float64)), _d(dx_inv), _d(dr_inv), _n(_np(c)),
                       *_grid_dims(g))
    return ft


def proj_fld_env(coord, wghts, Fld, Fld_tot, leftX, Rgrid, dx_inv, dr_inv, kx0):
    ft = _inout(Fld_tot, np.float64)
    g = _in(Fld, np.complex128)
    c = _in(coord, np.float64)
    lib().orc_proj_fld_env(_p(c), _p(_in(wghts, np.float64)), _vp(g), _p(ft), _d(leftX),
                           _p(_in(Rgrid, np.float64)), _d(dx_inv), _d(dr_inv), _d(kx0),
                           _n(_np(c)), *_grid_dims(g))
    return ft


def eb_correction(eb_spc):
    g = _inout(eb_spc, np.complex128)
    lib().orc_eb_correction(_vp(g), *_grid_dims(g), C.c_int(0))
    return g


def eb_correction_env(eb_spc):
    g = _inout(eb_spc, np.complex128)
    lib().orc_eb_correction(_vp(g), *_grid_dims(g), C.c_int(1))
    return g


# ---------------------------------------------------------------------------
# fb_io.f90
# ---------------------------------------------------------------------------

def _fb_in(vec_fb, vec, leftX, kx, In, ncomp):
    out = _inout(vec_fb, np.complex128)
    v = _in(vec, np.complex128)
    In_ = _in(In, np.float64)
    nx, nr, nm = v.shape[0], v.shape[1], v.shape[2]
    nkr = In_.shape[1]
    lib().orc_fb_in(_vp(out), _vp(v), _d(leftX), _p(_in(kx, np.float64)), _p(In_),
                    _n(nx), _n(nr), _n(nm), _n(nkr), _n(ncomp))
    return out


def fb_vec_in(vec_fb, vec, leftX, kx, In):
    return _fb_in(vec_fb, vec, leftX, kx, In, 3)


def fb_scl_in(scl_fb, scl, leftX, kx, In):
    return _fb_in(scl_fb, scl, leftX, kx, In, 1)


def _fb_out(vec_fb, leftX, kx, Out, ncomp, out=None):
    vfb = _in(vec_fb, np.complex128)
    Out_ = _in(Out, np.float64)
    nx, nkr, nm = vfb.shape[0], vfb.shape[1], vfb.shape[2]
    nr = Out_.shape[1] + 1
    if out is None:
        shape = (nx, nr, nm) + ((ncomp,) if ncomp > 1 else ())
        out = np.zeros(shape, dtype=np.complex128, order="F")
    lib().orc_fb_out(_vp(out), _vp(vfb), _d(leftX), _p(_in(kx, np.float64)), _p(Out_),
                     _n(nx), _n(nr), _n(nm), _n(nkr), _n(ncomp))
    return out


def fb_vec_out(vec_fb, leftX, kx, Out):
    return _fb_out(vec_fb, leftX, kx, Out, 3)


def fb_scl_out(scl_fb, leftX, kx, Out):
    return _fb_out(scl_fb, leftX, kx, Out, 1)


def fb_eb_out(eb_spc, e_fb, b_fb, leftX, kx, Out):
    eb = _inout(eb_spc, np.complex128)
    eb[...] = 0.0
    nx, nr, nm = eb.shape[0], eb.shape[1], eb.shape[2]
    half = nx * nr * nm * 3
    flat = eb.reshape(-1, order="F")
    e = np.asfortranarray(np.asarray(e_fb)[..., :3], dtype=np.complex128)
    lo = np.zeros((nx, nr, nm, 3), dtype=np.complex128, order="F")
    hi = np.zeros((nx, nr, nm, 3), dtype=np.complex128, order="F")
    _fb_out(e, leftX, kx, Out, 3, out=lo)
    _fb_out(b_fb, leftX, kx, Out, 3, out=hi)
    flat[:half] = lo.reshape(-1, order="F")
    flat[half:] = hi.reshape(-1, order="F")
    return eb


def fb_filtr(vec, leftX, kx, filtr, modefilt):
    v = _inout(vec, np.complex128)
    f = _in(filtr, np.float64)
    nx, nkr, nm = v.shape[0], v.shape[1], v.shape[2]
    lib().orc_fb_filtr(_vp(v), _d(leftX), _p(_in(kx, np.float64)), _p(f), _n(f.size),
                       C.c_int(int(modefilt)), _n(nx), _n(nkr), _n(nm), _n(3))
    return v


# ---------------------------------------------------------------------------
# fb_math*.f90
# ---------------------------------------------------------------------------

def _fbm(name, out, inp, DpS2S, DmS2S, kx, out_scalar=False):
    o = _inout(out, np.complex128)
    i = _in(inp, np.complex128)
    Dp = _in(DpS2S, np.float64)
    Dm = _in(DmS2S, np.float64)
    nx, nkr, nm = i.shape[0], i.shape[1], i.shape[2]
    nkl = Dp.shape[1]
    getattr(lib(), name)(_vp(o), _vp(i), _p(Dp), _p(Dm), _p(_in(kx, np.float64)),
                         _n(nx), _n(nkr), _n(nm), _n(nkl))
    return o


def fb_rot(vec_fb_loc, vec_fb, DpS2S, DmS2S, kx):
    return _fbm("orc_fb_rot", vec_fb_loc, vec_fb, DpS2S, DmS2S, kx)


def fb_grad(vec_fb_loc, scl_fb, DpS2S, DmS2S, kx):
    return _fbm("orc_fb_grad", vec_fb_loc, scl_fb, DpS2S, DmS2S, kx)


def fb_div(scl_fb_loc, vec_fb, DpS2S, DmS2S, kx):
    return _fbm("orc_fb_div", scl_fb_loc, vec_fb, DpS2S, DmS2S, kx)


def fb_rot_env(vec_fb_loc, vec_fb, DpS2S, DmS2S, kx):
    return _fbm("orc_fb_rot_env", vec_fb_loc, vec_fb, DpS2S, DmS2S, kx)


def fb_grad_env(vec_fb_loc, scl_fb, DpS2S, DmS2S, kx):
    return _fbm("orc_fb_grad_env", vec_fb_loc, scl_fb, DpS2S, DmS2S, kx)


def fb_div_env(scl_fb_loc, vec_fb, DpS2S, DmS2S, kx):
    return _fbm("orc_fb_div_env", scl_fb_loc, vec_fb, DpS2S, DmS2S, kx)


def _graddiv(name, vec_fb, DpS2S, DmS2S, kx):
    v = _inout(vec_fb, np.complex128)
    Dp = _in(DpS2S, np.float64)
    Dm = _in(DmS2S, np.float64)
    nx, nkr, nm = v.shape[0], v.shape[1], v.shape[2]
    getattr(lib(), name)(_vp(v), _p(Dp), _p(Dm), _p(_in(kx, np.float64)), _n(nx), _n(nkr),
                         _n(nm), _n(Dp.shape[1]))
    return v


def fb_graddiv(vec_fb, DpS2S, DmS2S, kx):
    return _graddiv("orc_fb_graddiv", vec_fb, DpS2S, DmS2S, kx)


def fb_graddiv_env(vec_fb, DpS2S, DmS2S, kx):
    return _graddiv("orc_fb_graddiv_env", vec_fb, DpS2S, DmS2S, kx)


# ---------------------------------------------------------------------------
# maxwell_solvers.f90
# ---------------------------------------------------------------------------

def _spec_dims(a):
    return _n(a.shape[0]), _n(a.shape[1]), _n(a.shape[2])


def maxwell_push_with_spchrg(EG_fb, j_fb, grad_rho_n_fb, grad_rho_np1_fb, C1, C2):
    eg = _inout(EG_fb, np.complex128)
    lib().orc_maxwell_push_with_spchrg(
        _vp(eg), _vp(_in(j_fb, np.complex128)), _vp(_in(grad_rho_n_fb, np.complex128)),
        _vp(_in(grad_rho_np1_fb, np.complex128)), _p(_in(C1, np.float64)),
        _p(_in(C2, np.float64)), *_spec_dims(eg))
    return eg


def maxwell_push_wo_spchrg(EG_fb, j_fb, C1, C2):
    eg = _inout(EG_fb, np.complex128)
    lib().orc_maxwell_push_wo_spchrg(_vp(eg), _vp(_in(j_fb, np.complex128)),
                                     _vp(_in(C1, np.complex128)), _vp(_in(C2, np.complex128)),
                                     *_spec_dims(eg))
    return eg


def maxwell_init_push(EG_fb, j_fb, grad_rho_n_fb, C1, C2):
    eg = _inout(EG_fb, np.complex128)
    lib().orc_maxwell_init_push(_vp(eg), _vp(_in(j_fb, np.complex128)),
                                _vp(_in(grad_rho_n_fb, np.complex128)),
                                _vp(_in(C1, np.complex128)), _vp(_in(C2, np.complex128)),
                                *_spec_dims(eg))
    return eg


def poiss_corr(j_fb, grad_div_j_fb, grad_rho_n_fb, grad_rho_np1_fb, dt_inv, w2_inv):
    j = _inout(j_fb, np.complex128)
    lib().orc_poiss_corr(_vp(j), _vp(_in(grad_div_j_fb, np.complex128)),
                         _vp(_in(grad_rho_n_fb, np.complex128)),
                         _vp(_in(grad_rho_np1_fb, np.complex128)), _d(dt_inv),
                         _p(_in(w2_inv, np.float64)), *_spec_dims(j))
    return j


def poiss_corr_stat(j_fb, grad_div_j_fb, grad_rho_n_fb, DT, w2_inv):
    j = _inout(j_fb, np.complex128)
    lib().orc_poiss_corr_stat(_vp(j), _vp(_in(grad_div_j_fb, np.complex128)),
                              _vp(_in(grad_rho_n_fb, np.complex128)),
                              _vp(_in(DT, np.complex128)), _p(_in(w2_inv, np.float64)),
                              *_spec_dims(j))
    return j


def field_drift(EG_fb, kx, beta0, dt):
    eg = _inout(EG_fb, np.complex128)
    lib().orc_field_drift(_vp(eg), _p(_in(kx, np.float64)), _d(beta0), _d(dt),
                          *_spec_dims(eg))
    return eg


def omp_mult_vec(vec_fb, A):
    v = _inout(vec_fb, np.complex128)
    a = _in(A, np.float64)
    lib().orc_mult(_vp(v), _p(a), _n(a.size), _n(3))
    return v


def omp_mult_scl(scl_fb, A):
    v = _inout(scl_fb, np.complex128)
    a = _in(A, np.float64)
    lib().orc_mult(_vp(v), _p(a), _n(a.size), _n(1))
    return v


def omp_add_vec(vec_fb, A):
    v = _inout(vec_fb, np.complex128)
    lib().orc_add(_vp(v), _vp(_in(A, np.complex128)), _n(v.size))
    return v


def omp_add_scl(scl_fb, A):
    return omp_add_vec(scl_fb, A)


# ---------------------------------------------------------------------------
# devices.f90
# ---------------------------------------------------------------------------

def undul_analytic(coord, Fld, t, params):
    f = _inout(Fld, np.float64)
    c = _in(coord, np.float64)
    lib().orc_undul_analytic(_p(c), _p(f), _d(t), _p(_in(params, np.float64)), _n(_np(c)))
    return f


def undul_analytic_taper(coord, Fld, t, params):
    f = _inout(Fld, np.float64)
    c = _in(coord, np.float64)
    lib().orc_undul_analytic_taper(_p(c), _p(f), _d(t), _p(_in(params, np.float64)),
                                   _n(_np(c)))
    return f


def undul_mapped(coord, Fld, t, a0, params):
    f = _inout(Fld, np.float64)
    c = _in(coord, np.float64)
    a = _in(a0, np.float64)
    lib().orc_undul_mapped(_p(c), _p(f), _d(t), _p(a), _n(a.shape[1]),
                           _p(_in(params, np.float64)), C.c_int(0), _n(_np(c)))
    return f


def undul_mapped_tap(coord, Fld, t, a0, params):
    f = _inout(Fld, np.float64)
    c = _in(coord, np.float64)
    a = _in(a0, np.float64)
    lib().orc_undul_mapped(_p(c), _p(f), _d(t), _p(a), _n(a.shape[1]),
                           _p(_in(params, np.float64)), C.c_int(1), _n(_np(c)))
    return f


def planewave(coord, Fld, t, params):
    f = _inout(Fld, np.float64)
    c = _in(coord, np.float64)
    lib().orc_planewave(_p(c), _p(f), _d(t), _p(_in(params, np.float64)), _n(_np(c)))
    return f


def gaussbeam(coord, Fld, time, a0, params):
    f = _inout(Fld, np.float64)
    c = _in(coord, np.float64)
    lib().orc_gaussbeam(_p(c), _p(f), _d(time), _d(a0), _p(_in(params, np.float64)),
                        _n(_np(c)))
    return f


def fft(a, sign=-1):
    """The oracle's own mixed-radix DFT (unnormalised), for its tests."""
    a = np.ascontiguousarray(a, dtype=np.complex128)
    out = np.empty_like(a)
    lib().orc_fft(_vp(a), _vp(out), _n(a.size), C.c_int(sign))
    return out


# ---------------------------------------------------------------------------
# utils.f90 and diagnostics.py reductions
# ---------------------------------------------------------------------------

def intens_profo(Fld, NO):
    """utils.f90:18-57: PWR_RO (NO, nr) from Fld (nx+1, nr+1, 2 nkO + 1, 3).
    As f2py, nkO is inferred from the mode extent, which must be odd."""
    f = _in(Fld, np.complex128)
    NX, NR, NM, nc = f.shape
    if nc != 3 or NM % 2 != 1:
        raise ValueError("intens_profo: Fld must be (nx+1, nr+1, 2*nkO+1, 3)")
    out = np.zeros((int(NO), NR - 1), dtype=np.float64, order="F")
    lib().orc_intens_profo(_p(out), _vp(f), _n(NO), _n(NX), _n(NR), _n(NM))
    return out


def em_energy(EG_fb, EnergyFact):
    """diagnostics.py:112-114 before the reordering, in the reference's
    numpy order: (|E|^2 summed over the 3 components) * EnergyFact, summed
    over modes, then over kr."""
    eg = np.asarray(EG_fb)
    return ((np.abs(eg[:, :, :, :3]) ** 2).sum(-1) * np.asarray(EnergyFact)).sum(-1).sum(-1)


def power_profile(dat, Rgrid, fac):
    """diagnostics.py:134-143: fac * sum_r Rgrid * sum_{m, l} |dat|^2."""
    dat = np.asarray(dat)
    return fac * ((np.abs(dat) ** 2).sum(-1).sum(-1) * np.asarray(Rgrid)[None, :]).sum(-1)
