"""The C ABI library: it loads, exports every symbol include/*.h declares, and
rejects bad arguments with status codes (host-side checks, no GPU needed)."""
import ctypes as C
import glob
import os
import re
import subprocess

import pytest

from conftest import ROOT


def _declared():
    names = []
    for h in glob.glob(os.path.join(ROOT, "include", "*.h")):
        text = re.sub(r"/\*.*?\*/", " ", open(h).read(), flags=re.S)
        names += re.findall(r"\b(chm_\w+)\s*\(", text)
    return sorted(set(names))


def test_library_builds_and_exports_every_declared_symbol():
    from chimera_gb300 import _lib, buildlib as build
    path = build.build()
    lib = C.CDLL(path)
    declared = _declared()
    assert len(declared) >= 40
    for name in declared:
        assert hasattr(lib, name), name
    out = subprocess.run(["nm", "-D", "--defined-only", path], capture_output=True, text=True)
    if out.returncode == 0:
        exported = set(re.findall(r"\b(chm_\w+)\b", out.stdout))
        assert set(declared) <= exported
    assert set(_lib.exported_symbols()) == set(declared)


def test_status_codes_without_gpu():
    from chimera_gb300 import _lib
    lib = _lib.load()
    assert lib.chm_push_velocs(None, 1, 3, None, 1, 6, 0.1, -1, None) == 1  # CHM_ERR_ARG
    assert b"np < 0" in lib.chm_last_error()
    # workspace too small is reported before any device work
    fake = C.c_void_p(256)
    rc = lib.chm_dep_curr(fake, 1, 3, fake, 1, 3, fake, 1, fake, 0.0, fake, 1.0, 1.0, 10, 16, 9,
                          2, fake, 8, None)
    assert rc == 3  # CHM_ERR_WS
    rc = lib.chm_fb_in(fake, fake, 0.0, fake, fake, None, 16, 9, 8, 2, 3, fake, 8, None)
    assert rc == 3
    rc = lib.chm_fb_filtr(fake, 0.0, fake, fake, 4, 7, 16, 8, 2, 3, fake, 1 << 20, None)
    assert rc == 1  # bad modefilt
    assert lib.chm_dep_ws_bytes(16, 9, 2, 3, 10) >= 16 * 9 * 2 * 3 * 2 * 8


def test_envelope_gather_rejects_bad_undulators_without_gpu():
    """chm_sp_gather_push_env checks its undulator and carrier arguments on
    the host: a mapped undulator without a map, with no columns or a
    misaligned map, an unknown kind and a short carrier table."""
    from chimera_gb300 import _lib
    lib = _lib.load()
    fake = C.c_void_p(256)
    und = (C.c_double * 5)(1.0, 0.0, 0.35, 10.0, 0.1)

    def call(kind, amap, nmap, ntab=20):
        return lib.chm_sp_gather_push_env(*[fake] * 8, 100, 0, 0.0, 1.0, fake, 16, 9, 3, 0.1,
                                          fake, ntab, 0.1, kind, und, amap, nmap, 0.0, 0.1,
                                          None, None)

    for kind, amap, nmap in ((3, None, 10), (4, fake, 0), (3, C.c_void_p(260), 10),
                             (5, fake, 10)):
        assert call(kind, amap, nmap) == 1, (kind, amap, nmap)  # CHM_ERR_ARG
        assert b"undulator" in lib.chm_last_error()
    assert call(3, fake, 10, ntab=19) == 1
    assert b"carrier table" in lib.chm_last_error()


def test_fimera_has_every_reference_kernel_name():
    """Every f2py routine the reference's Python calls exists in the shim."""
    from chimera_gb300 import fimera
    names = ["push_velocs", "push_coords", "genparts", "sortpartsout", "chunk_coords_boundaries",
             "align_data_vec", "align_data_scl", "dep_curr", "dep_dens", "dep_curr_chnk",
             "dep_dens_chnk", "dep_curr_env", "dep_dens_env", "dep_curr_env_chnk",
             "dep_dens_env_chnk", "proj_fld", "proj_fld_env", "eb_correction",
             "eb_correction_env", "fb_vec_in", "fb_scl_in", "fb_vec_out", "fb_scl_out",
             "fb_eb_out", "fb_filtr", "fb_rot", "fb_grad", "fb_div", "fb_graddiv", "fb_rot_env",
             "fb_grad_env", "fb_div_env", "fb_graddiv_env", "maxwell_push_with_spchrg",
             "maxwell_push_wo_spchrg", "maxwell_init_push", "poiss_corr", "poiss_corr_stat",
             "field_drift", "omp_mult_vec", "omp_mult_scl", "omp_add_vec", "omp_add_scl",
             "undul_analytic", "undul_analytic_taper", "undul_mapped", "undul_mapped_tap",
             "planewave", "gaussbeam"]
    missing = [n for n in names if not hasattr(fimera, n)]
    assert missing == ["genparts"] or missing == []


def test_fimera_rejects_cpu_tensors():
    import torch
    from chimera_gb300 import fimera
    with pytest.raises(fimera.ChimeraError):
        fimera.push_velocs(torch.zeros(3, 4, dtype=torch.float64),
                           torch.zeros(6, 4, dtype=torch.float64), 0.1)


def test_empty_species_without_gpu():
    """A species with no particles (n = 0) is a no-op for the particle entry
    points of both forms: status 0 with null particle arrays, before any
    device work (the Fortran loops run zero times)."""
    from chimera_gb300 import _lib
    lib = _lib.load()
    N = None
    und = (C.c_double * 5)(1.0, 0.0, 0.35, 10.0, 0.1)
    calls = {
        "chm_push_velocs": (N, 1, 3, N, 1, 6, 0.1, 0, N),
        "chm_push_coords": (N, 1, 3, N, 1, 3, N, 1, 3, 0.1, 0, N),
        "chm_sp_push_deposit": (*[N] * 8, 0, 0, 0.0, 1.0, 1.0, 0.1, 16, 9, 3, 1,
                                *[N] * 6),
        "chm_sp_gather_push": (*[N] * 8, 0, 0, 0.0, 1.0, N, 16, 9, 3, 0.1, N, N),
        "chm_sp_push_deposit_env": (*[N] * 8, 0, 0, 0.0, 1.0, 1.0, 0.1, 0.1, 16, 9, 3, N, N, N,
                                    20, 0.1, N, N),
        "chm_sp_gather_push_env": (*[N] * 8, 0, 0, 0.0, 1.0, N, 16, 9, 3, 0.1, N, 20, 0.1, 0,
                                   und, N, 0, 0.0, 0.1, N, N),
    }
    for name, args in calls.items():
        assert getattr(lib, name)(*args) == 0, (name, lib.chm_last_error())
