"""GPU parity: every fimera kernel (CUDA, through the C ABI) against the
oracle on the same seeded inputs.  FP64 tolerance: 1e-12 relative L2 per
kernel (the plain form's budget is 1e-10 per step)."""
import numpy as np
import pytest

from conftest import rel_l2

pytestmark = pytest.mark.gpu
TOL = 1e-12


@pytest.fixture(scope="module")
def fm(cuda):
    from chimera_gb300 import fimera
    return fimera


def T(a, soa=True):
    """numpy -> CUDA tensor; particle arrays as SoA (part stride 1) unless
    soa=False (the reference's F-ordered (3, Np) layout)."""
    import torch
    a = np.asarray(a)
    if a.dtype.kind == "c" or a.ndim > 2 or not soa:
        return torch.from_numpy(np.asfortranarray(a)).cuda()
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


def H(t):
    return t.cpu().numpy()


def ops(golden, name):
    return {k.split("/")[-1]: golden[k] for k in golden.files if k.startswith(f"op/{name}/Args/")}


def parts(n, seed, x0, x1, rmax, rmin=0.0, pscale=1.0):
    rng = np.random.default_rng(seed)
    x = rng.uniform(x0, x1, n)
    r = np.sqrt(rng.uniform(rmin ** 2, rmax ** 2, n))
    th = rng.uniform(0, 2 * np.pi, n)
    c = np.vstack([x, r * np.cos(th), r * np.sin(th)])
    p = pscale * rng.standard_normal((3, n))
    w = rng.uniform(0.5, 1.5, n)
    w[:: 17] = 0.0  # zero weights are skipped
    return np.asfortranarray(c), np.asfortranarray(p), w


def rand_c(shape, seed):
    rng = np.random.default_rng(seed)
    return np.asfortranarray(rng.standard_normal(shape) + 1j * rng.standard_normal(shape))


@pytest.mark.parametrize("soa", [True, False])
def test_push_velocs(fm, orc, soa):
    rng = np.random.default_rng(1)
    p = np.asfortranarray(rng.standard_normal((3, 5000)))
    F = np.asfortranarray(rng.standard_normal((6, 5000)))
    ref = orc.push_velocs(p.copy(order="F"), F, 0.37)
    got = fm.push_velocs(T(p, soa), T(F, soa), 0.37)
    assert rel_l2(H(got), ref) < TOL


def test_push_coords(fm, orc):
    rng = np.random.default_rng(2)
    x = np.asfortranarray(rng.standard_normal((3, 4097)))
    p = np.asfortranarray(rng.standard_normal((3, 4097)))
    h = np.zeros_like(x, order="F")
    rx, rh = orc.push_coords(x.copy(order="F"), p, h.copy(order="F"), 0.04)
    gx, gh = fm.push_coords(T(x), T(p), T(h), 0.04)
    assert rel_l2(H(gx), rx) < TOL and rel_l2(H(gh), rh) < TOL


@pytest.mark.parametrize("name,env", [("lpa_m2", False), ("lpa_m3_chunked", False),
                                      ("fel_env_k1", True)])
def test_proj_fld(fm, orc, golden, name, env):
    g = ops(golden, name)
    nx, nr, nm = int(g["Nx"]), int(g["Nr"]), int(g["Mtot"])
    leftX, dx, dr = float(g["leftX"]), g["Xgrid"][1] - g["Xgrid"][0], g["Rgrid"][2] - g["Rgrid"][1]
    c, _, w = parts(6000, 3, leftX - 0.2, leftX + (nx + 1) * dx, g["Rgrid"][-1] * 1.05)
    c[1:, :5] = 0.0  # on-axis particles
    fld = rand_c((nx, nr, nm, 6), 4)
    ft = np.asfortranarray(np.random.default_rng(5).standard_normal((6, c.shape[1])))
    args = (leftX, g["Rgrid"], 1 / dx, 1 / dr) + ((float(g["kx0"]),) if env else ())
    f_o, f_g = (orc.proj_fld_env, fm.proj_fld_env) if env else (orc.proj_fld, fm.proj_fld)
    ref = f_o(c, w, fld, ft.copy(order="F"), *args)
    got = f_g(T(c), T(w), T(fld), T(ft), *args)
    assert rel_l2(H(got), ref) < TOL


@pytest.mark.parametrize("env", [False, True])
def test_eb_correction(fm, orc, env):
    for nm in ((1, 3) if env else (1, 2, 3)):
        eb = rand_c((32, 9, nm, 6), 6)
        f_o, f_g = (orc.eb_correction_env, fm.eb_correction_env) if env else (orc.eb_correction, fm.eb_correction)
        ref = f_o(eb.copy(order="F"))
        got = f_g(T(eb))
        assert rel_l2(H(got), ref) < TOL


DEP_CASES = [("dep_curr", False, False), ("dep_dens", False, False),
             ("dep_curr_env", True, False), ("dep_dens_env", True, False),
             ("dep_curr_chnk", False, True), ("dep_dens_chnk", False, True),
             ("dep_curr_env_chnk", True, True), ("dep_dens_env_chnk", True, True)]


@pytest.mark.parametrize("kind,env,chnk", DEP_CASES)
def test_deposits(fm, orc, golden, kind, env, chnk):
    g = ops(golden, "fel_env_k1" if env else "lpa_m3_chunked")
    nx, nr, nm = int(g["Nx"]), int(g["Nr"]), int(g["Mtot"])
    leftX, dx = float(g["leftX"]), g["Xgrid"][1] - g["Xgrid"][0]
    dr = g["Rgrid"][2] - g["Rgrid"][1]
    c, p, w = parts(20000, 7, leftX - 0.5 * dx, leftX + (nx - 0.5) * dx, g["Rgrid"][-1] * 1.02)
    c[1:, :3] = 0.0
    p[:, 3] = 0.0
    curr = kind.startswith("dep_curr")
    shape = (nx, nr, nm, 3) if curr else (nx, nr, nm)
    grid0 = rand_c(shape, 8) * 0.1
    extra = (float(g["kx0"]),) if env else ()
    base = (leftX, g["Rgrid"], 1 / dx, 1 / dr) + extra
    if chnk:
        nch = 4
        xg = g["Xgrid"]
        ids, ind, go = orc.chunk_coords_boundaries(c, np.array([xg[0], xg[-1], 0, 1e9]), xg, nch)
        order = np.argsort(ids, kind="stable")[go:]
        c, p, w = (np.asfortranarray(a[..., order]) for a in (c, p, w))
        mid = (ind, 2)
    else:
        mid = ()
    pa = (c, p, w) if curr else (c, w)
    ref = getattr(orc, kind)(*pa, grid0.copy(order="F"), *mid, *base)
    gpa = tuple(T(a) for a in pa)
    gmid = (T(ind), 2) if chnk else ()
    got = getattr(fm, kind)(*gpa, T(grid0), *gmid, *base)
    assert rel_l2(H(got), ref) < TOL
    # bitwise determinism: the same inputs deposit the same bits
    again = getattr(fm, kind)(*gpa, T(grid0), *gmid, *base)
    assert np.array_equal(H(got), H(again))


@pytest.mark.parametrize("name", ["lpa_m2", "lpa_m3_chunked", "fel_env_k1"])
def test_fb_transforms(fm, orc, golden, name):
    g = ops(golden, name)
    nx, nr, nkr, nm = int(g["Nx"]), int(g["Nr"]), int(g["Nkr"]), int(g["Mtot"])
    leftX = float(g["leftX"]) + 0.37
    kx = g["kx_env"] if "KxShift" in name or name.startswith("fel") else g["kx"]
    v = rand_c((nx, nr, nm, 3), 9)
    ref = orc.fb_vec_in(np.zeros((nx, nkr, nm, 3), complex, order="F"), v, leftX, kx, g["InCurr"])
    got = fm.fb_vec_in(T(np.zeros((nx, nkr, nm, 3), complex, order="F")), T(v), leftX, kx, g["InCurr"])
    assert rel_l2(H(got), ref) < TOL
    s = rand_c((nx, nr, nm), 10)
    ref = orc.fb_scl_in(np.zeros((nx, nkr, nm), complex, order="F"), s, leftX, kx, g["In"])
    got = fm.fb_scl_in(T(np.zeros((nx, nkr, nm), complex, order="F")), T(s), leftX, kx, g["In"])
    assert rel_l2(H(got), ref) < TOL
    vfb = rand_c((nx, nkr, nm, 3), 11)
    assert rel_l2(H(fm.fb_vec_out(T(vfb), leftX, kx, g["Out"])),
                  orc.fb_vec_out(vfb, leftX, kx, g["Out"])) < TOL
    assert rel_l2(H(fm.fb_scl_out(T(vfb[..., 0].copy(order="F")), leftX, kx, g["Out"])),
                  orc.fb_scl_out(vfb[..., 0].copy(order="F"), leftX, kx, g["Out"])) < TOL
    e = rand_c((nx, nkr, nm, 6), 12)
    b = rand_c((nx, nkr, nm, 3), 13)
    eb0 = np.zeros((nx, nr, nm, 6), complex, order="F")
    ref = orc.fb_eb_out(eb0.copy(order="F"), e, b, leftX, kx, g["Out"])
    got = fm.fb_eb_out(T(eb0), T(e), T(b), leftX, kx, g["Out"])
    assert rel_l2(H(got), ref) < TOL
    # fused eb_correction
    envc = name.startswith("fel")
    ref_c = (orc.eb_correction_env if envc else orc.eb_correction)(ref.copy(order="F"))
    got_c = fm.fb_eb_out(T(eb0), T(e), T(b), leftX, kx, g["Out"], eb_mode=2 if envc else 1)
    assert rel_l2(H(got_c), ref_c) < TOL


@pytest.mark.parametrize("mode", [0, 1, 2])
def test_fb_filtr(fm, orc, golden, mode):
    g = ops(golden, "lpa_m2")
    nx, nkr, nm = int(g["Nx"]), int(g["Nkr"]), int(g["Mtot"])
    v = rand_c((nx, nkr, nm, 3), 14)
    prof = np.linspace(0.0, 1.0, 9) ** 2
    ref = orc.fb_filtr(v.copy(order="F"), float(g["leftX"]), g["kx"], prof, mode)
    got = fm.fb_filtr(T(v), float(g["leftX"]), g["kx"], prof, mode)
    assert rel_l2(H(got), ref) < TOL


FBM = [("fb_rot", "vec", "vec"), ("fb_grad", "scl", "vec"), ("fb_div", "vec", "scl")]


@pytest.mark.parametrize("name", ["lpa_m2", "lpa_m3_chunked", "plain_m1_vacuum", "fel_env_k1"])
@pytest.mark.parametrize("op,inp,out", FBM)
def test_fb_math(fm, orc, golden, name, op, inp, out):
    g = ops(golden, name)
    env = name.startswith("fel")
    nx, nkr, nm = int(g["Nx"]), int(g["Nkr"]), int(g["Mtot"])
    x = rand_c((nx, nkr, nm, 3) if inp == "vec" else (nx, nkr, nm), 15)
    o = np.zeros((nx, nkr, nm, 3) if out == "vec" else (nx, nkr, nm), complex, order="F")
    fn = op + ("_env" if env else "")
    ref = getattr(orc, fn)(o.copy(order="F"), x, g["DpS2S"], g["DmS2S"], g["kx"])
    got = getattr(fm, fn)(T(o), T(x), g["DpS2S"], g["DmS2S"], g["kx"])
    assert rel_l2(H(got), ref) < TOL


@pytest.mark.parametrize("name", ["lpa_m2", "lpa_m3_chunked", "plain_m1_vacuum", "fel_env_k1"])
def test_fb_graddiv(fm, orc, golden, name):
    g = ops(golden, name)
    env = name.startswith("fel")
    nx, nkr, nm = int(g["Nx"]), int(g["Nkr"]), int(g["Mtot"])
    v = rand_c((nx, nkr, nm, 3), 16)
    fn = "fb_graddiv_env" if env else "fb_graddiv"
    ref = getattr(orc, fn)(v.copy(order="F"), g["DpS2S"], g["DmS2S"], g["kx"])
    got = getattr(fm, fn)(T(v), g["DpS2S"], g["DmS2S"], g["kx"])
    assert rel_l2(H(got), ref) < TOL


def test_maxwell_and_elementwise(fm, orc, golden):
    g = ops(golden, "lpa_m2")
    nx, nkr, nm = int(g["Nx"]), int(g["Nkr"]), int(g["Mtot"])
    rng = np.random.default_rng(17)
    eg = rand_c((nx, nkr, nm, 6), 18)
    j, a, b = (rand_c((nx, nkr, nm, 3), s) for s in (19, 20, 21))
    C1 = np.asfortranarray(rng.standard_normal((nx, nkr, nm, 5)))
    C2 = np.asfortranarray(rng.standard_normal((nx, nkr, nm, 5)))
    ref = orc.maxwell_push_with_spchrg(eg.copy(order="F"), j, a, b, C1, C2)
    got = fm.maxwell_push_with_spchrg(T(eg), T(j), T(a), T(b), C1, C2)
    assert rel_l2(H(got), ref) < TOL
    Cc1, Cc2 = rand_c((nx, nkr, nm, 3), 22), rand_c((nx, nkr, nm, 3), 23)
    ref = orc.maxwell_push_wo_spchrg(eg.copy(order="F"), j, Cc1, Cc2)
    got = fm.maxwell_push_wo_spchrg(T(eg), T(j), Cc1, Cc2)
    assert rel_l2(H(got), ref) < TOL
    # real coefficients are cast to complex, as f2py does for the plain solver
    ref = orc.maxwell_push_wo_spchrg(eg.copy(order="F"), j, C1[..., :3].copy(order="F"),
                                     C2[..., :3].copy(order="F"))
    got = fm.maxwell_push_wo_spchrg(T(eg), T(j), C1[..., :3].copy(order="F"),
                                    C2[..., :3].copy(order="F"))
    assert rel_l2(H(got), ref) < TOL
    Ci1, Ci2 = rand_c((nx, nkr, nm, 2), 24), rand_c((nx, nkr, nm, 2), 25)
    ref = orc.maxwell_init_push(eg.copy(order="F"), j, a, Ci1, Ci2)
    got = fm.maxwell_init_push(T(eg), T(j), T(a), Ci1, Ci2)
    assert rel_l2(H(got), ref) < TOL
    w2 = np.asfortranarray(rng.uniform(0.1, 2.0, (nx, nkr, nm)))
    ref = orc.poiss_corr(j.copy(order="F"), a, b, eg[..., :3].copy(order="F"), 7.0, w2)
    got = fm.poiss_corr(T(j), T(a), T(b), T(eg[..., :3].copy(order="F")), 7.0, w2)
    assert rel_l2(H(got), ref) < TOL
    DT = rand_c((nx,), 26)
    ref = orc.poiss_corr_stat(j.copy(order="F"), a, b, DT, w2)
    got = fm.poiss_corr_stat(T(j), T(a), T(b), DT, w2)
    assert rel_l2(H(got), ref) < TOL
    ref = orc.field_drift(eg.copy(order="F"), g["kx"], 0.93, 0.1)
    got = fm.field_drift(T(eg), g["kx"], 0.93, 0.1)
    assert rel_l2(H(got), ref) < TOL
    ref = orc.omp_mult_vec(j.copy(order="F"), w2)
    assert rel_l2(H(fm.omp_mult_vec(T(j), w2)), ref) < TOL
    ref = orc.omp_mult_scl(a[..., 0].copy(order="F"), w2)
    assert rel_l2(H(fm.omp_mult_scl(T(a[..., 0].copy(order="F")), w2)), ref) < TOL
    ref = orc.omp_add_vec(j.copy(order="F"), a)
    assert rel_l2(H(fm.omp_add_vec(T(j), T(a))), ref) < TOL


DEVICES = [("undul_analytic", [1.2, 0.8, -1.0, 6.0]),
           ("undul_analytic_taper", [1.2, 0.8, -1.0, 6.0, 0.05]),
           ("planewave", [0.3, 1.1, -1.5, 5.0, 0.7, 0.2, 0.4])]


@pytest.mark.parametrize("name,params", DEVICES)
def test_devices(fm, orc, name, params):
    c, _, _ = parts(3000, 27, -2.0, 5.5, 0.5)
    F = np.asfortranarray(np.random.default_rng(28).standard_normal((6, 3000)))
    ref = getattr(orc, name)(c, F.copy(order="F"), 0.77, np.array(params))
    got = getattr(fm, name)(T(c), T(F), 0.77, np.array(params))
    assert rel_l2(H(got), ref) < TOL


@pytest.mark.parametrize("tap", [False, True])
def test_undul_mapped(fm, orc, tap):
    c, _, _ = parts(3000, 29, -0.5, 10.5, 0.3)
    F = np.zeros((6, 3000), order="F")
    a0 = np.asfortranarray(np.random.default_rng(30).standard_normal((2, 200)))
    params = np.array([1.5, -0.2, 0.05, 8.0, 0.1])
    name = "undul_mapped_tap" if tap else "undul_mapped"
    ref = getattr(orc, name)(c, F.copy(order="F"), 0.0, a0, params)
    got = getattr(fm, name)(T(c), T(F), 0.0, a0, params)
    assert rel_l2(H(got), ref) < TOL


def test_gaussbeam(fm, orc):
    c, _, _ = parts(3000, 31, -2.0, 2.0, 1.5)
    F = np.zeros((6, 3000), order="F")
    params = np.array([1.0, 1.0, 0.1, 0.0, 0.0, 1.0, 0.8, 0.8])
    ref = orc.gaussbeam(c, F.copy(order="F"), 0.3, 0.5, params)
    got = fm.gaussbeam(T(c), T(F), 0.3, 0.5, params)
    assert rel_l2(H(got), ref) < TOL


def test_sorting_and_alignment(fm, orc):
    c, p, w = parts(50000, 32, -3.0, 3.0, 2.0)
    lims = np.array([-2.5, 2.5, 0.0, 1.5 ** 2])
    ref_idx, ref_n = orc.sortpartsout(c, lims)
    idx, n = fm.sortpartsout(T(c), lims)
    assert n == ref_n and np.array_equal(H(idx)[:n], ref_idx[:n])
    xg = -3.0 + 0.05 * np.arange(121)
    ids_r, ind_r, go_r = orc.chunk_coords_boundaries(c, lims, xg, 6)
    ids, ind, go = fm.chunk_coords_boundaries(T(c), lims, xg, 6)
    assert go == go_r and np.array_equal(H(ids), ids_r) and np.array_equal(H(ind), ind_r)
    order = fm.chunk_order(ids, 6)
    assert np.array_equal(H(order), np.argsort(ids_r, kind="stable")[go_r:])
    dat = T(c)
    fm.align_data_vec(dat, order)
    assert np.array_equal(H(dat)[:, : order.shape[0]], c[:, np.argsort(ids_r, kind="stable")[go_r:]])


def test_empty_and_single_particle_inputs(fm, orc, golden):
    import torch
    g = ops(golden, "lpa_m2")
    nx, nr, nm = int(g["Nx"]), int(g["Nr"]), int(g["Mtot"])
    z3 = torch.zeros((3, 0), dtype=torch.float64, device="cuda")
    z1 = torch.zeros((0,), dtype=torch.float64, device="cuda")
    grid = T(rand_c((nx, nr, nm, 3), 33))
    before = H(grid).copy()
    fm.dep_curr(z3, z3, z1, grid, float(g["leftX"]), g["Rgrid"], 10.0, 4.0)
    ref = orc.dep_curr(np.zeros((3, 0), order="F"), np.zeros((3, 0), order="F"), np.zeros(0),
                       before.copy(order="F"), float(g["leftX"]), g["Rgrid"], 10.0, 4.0)
    assert rel_l2(H(grid), ref) < TOL
    fm.push_velocs(z3, torch.zeros((6, 0), dtype=torch.float64, device="cuda"), 0.1)
