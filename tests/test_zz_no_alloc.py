"""The allocation-free current deposit, through the C ABI.

chm_dep_curr_noalloc serves callers that cannot allocate device memory by
keeping its scratch in a static device array.  It must give the same grid
as chm_dep_curr (which takes a caller workspace), also on a second call in a
row (the shared array keeps the previous call's contents and must be cleared
by the call itself).  This file is collected last on purpose."""
import numpy as np
import pytest

from conftest import rel_l2

pytestmark = pytest.mark.gpu
TOL = 1e-12  # FP64 deposit tolerance used by the other GPU tests


def _particles(seed, n, leftX, nx, dx, rmax):
    rng = np.random.default_rng(seed)
    x = rng.uniform(leftX, leftX + (nx - 1) * dx, n)
    r = np.sqrt(rng.uniform(0, (0.95 * rmax) ** 2, n))
    th = rng.uniform(0, 2 * np.pi, n)
    c = np.vstack([x, r * np.cos(th), r * np.sin(th)])
    p = rng.standard_normal((3, n))
    w = rng.uniform(0.5, 1.5, n)
    return c, p, w


def test_no_alloc_deposit_matches_workspace_deposit(cuda):
    import torch
    from chimera_gb300 import _lib, fimera
    st = torch.cuda.current_stream().cuda_stream
    nx, nr, nm = 256, 33, 2
    dx, dr = 0.05, 0.25
    leftX = -3.0
    rgrid = torch.from_numpy(dr * (np.arange(nr) - 0.5)).cuda()
    assert _lib.load().chm_dep_noalloc_max_bytes() >= _lib.query("chm_dep_ws_bytes", nx, nr, nm, 3, 0)
    ws = torch.empty(_lib.query("chm_dep_ws_bytes", nx, nr, nm, 3, 0), dtype=torch.uint8,
                     device="cuda")
    for call, seed in enumerate((11, 12)):
        c, p, w = _particles(seed, 20000 + 1000 * call, leftX, nx, dx, rgrid[-1].item())
        xc = torch.from_numpy(np.ascontiguousarray(c)).cuda()
        pc = torch.from_numpy(np.ascontiguousarray(p)).cuda()
        wc = torch.from_numpy(w).cuda()
        n = wc.numel()
        ref = fimera.fortran_zeros((nx, nr, nm, 3))
        got = fimera.fortran_zeros((nx, nr, nm, 3))
        _lib.call("chm_dep_curr", xc.data_ptr(), xc.stride(0), xc.stride(1), pc.data_ptr(),
                  pc.stride(0), pc.stride(1), wc.data_ptr(), 1, ref.data_ptr(), leftX,
                  rgrid.data_ptr(), 1 / dx, 1 / dr, n, nx, nr, nm, ws.data_ptr(), ws.numel(), st)
        _lib.call("chm_dep_curr_noalloc", xc.data_ptr(), xc.stride(0), xc.stride(1), pc.data_ptr(),
                  pc.stride(0), pc.stride(1), wc.data_ptr(), 1, got.data_ptr(), leftX,
                  rgrid.data_ptr(), 1 / dx, 1 / dr, n, nx, nr, nm, st)
        torch.cuda.synchronize()
        r, g = ref.cpu().numpy(), got.cpu().numpy()
        assert np.abs(r).max() > 0
        assert rel_l2(g, r) <= TOL, f"call {call}: {rel_l2(g, r):.3e}"


def test_no_alloc_deposit_rejects_oversized_grid(cuda):
    from chimera_gb300 import _lib
    lib = _lib.load()
    # a grid whose accumulator alone exceeds the static array; rejected before any device work
    rc = lib.chm_dep_curr_noalloc(None, 1, 3, None, 1, 3, None, 1, None, 0.0, None, 1.0, 1.0, 0,
                                  4096, 513, 3, None)
    assert rc == 5  # CHM_ERR_RANGE
    assert b"static array" in lib.chm_last_error()


def test_no_alloc_deposit_rejects_bad_and_overflowing_dims(cuda):
    from chimera_gb300 import _lib
    lib = _lib.load()
    # dimensions whose product wraps a 64-bit integer are rejected as too large
    rc = lib.chm_dep_curr_noalloc(None, 1, 3, None, 1, 3, None, 1, None, 0.0, None, 1.0, 1.0, 0,
                                  1 << 40, 1 << 20, 1 << 10, None)
    assert rc == 5 and b"static array" in lib.chm_last_error()
    # grids the deposit does not accept get their own message
    for dims in ((0, 33, 2), (256, 1, 2), (256, 33, 0), (-5, 33, 2)):
        rc = lib.chm_dep_curr_noalloc(None, 1, 3, None, 1, 3, None, 1, None, 0.0, None, 1.0, 1.0,
                                      0, *dims, None)
        assert rc == 1 and b"bad grid" in lib.chm_last_error(), dims
