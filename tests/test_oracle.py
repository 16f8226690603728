"""The CPU oracle against numpy and the reference's own mathematics
(known-answer tests; the reference ships no golden kernel outputs)."""
import numpy as np
import pytest

from conftest import rel_l2


@pytest.mark.parametrize("n", [1, 2, 12, 64, 131, 524, 1408, 2048])
def test_fft_matches_numpy(orc, n):
    rng = np.random.default_rng(n)
    x = rng.standard_normal(n) + 1j * rng.standard_normal(n)
    assert rel_l2(orc.fft(x, -1), np.fft.fft(x)) < 1e-14
    assert rel_l2(orc.fft(x, +1), np.fft.ifft(x) * n) < 1e-14


def _ops(golden, name):
    g = {k.split("/")[-1]: golden[k] for k in golden.files if k.startswith(f"op/{name}/Args/")}
    return g


def test_fb_round_trip(orc, golden):
    """In = inv(Out) (solvers.py:743): fb_scl_in followed by fb_scl_out is Nx
    times the identity on rows 1..Nr-1."""
    g = _ops(golden, "lpa_m2")
    nx, nr, nm = int(g["Nx"]), int(g["Nr"]), int(g["Mtot"])
    rng = np.random.default_rng(0)
    v = np.asfortranarray(rng.standard_normal((nx, nr, nm)) + 1j * rng.standard_normal((nx, nr, nm)))
    v[:, 0] = 0
    vfb = np.zeros((nx, int(g["Nkr"]), nm), complex, order="F")
    vfb = orc.fb_scl_in(vfb, v, float(g["leftX"]), g["kx"], g["In"])
    back = orc.fb_scl_out(vfb, float(g["leftX"]), g["kx"], g["Out"])
    assert rel_l2(back[:, 1:], nx * v[:, 1:]) < 1e-12


def test_fb_transforms_vs_numpy(orc, golden):
    """fb_io.f90:18-228 restated with numpy's FFT (FFTW_FORWARD = fft,
    FFTW_BACKWARD = n ifft): fb_vec_in sums In(r, k, m) over rows 1..Nr-1
    (the ghost row skipped), transforms along x and multiplies by
    e^{-i kx leftX}; fb_vec_out multiplies the Out sum by e^{+i kx leftX}
    and transforms back unnormalised into rows 1..Nr-1 (row 0 zero);
    fb_eb_out does that for E (e_fb's first three components) and B into
    the six components of a zeroed grid."""
    g = _ops(golden, "lpa_m2")
    nx, nr, nk, nm = int(g["Nx"]), int(g["Nr"]), int(g["Nkr"]), int(g["Mtot"])
    leftX, kx, In, Out = float(g["leftX"]) + 0.37, g["kx"], g["In"], g["Out"]
    v = _rand_fb((nx, nr, nm, 3), 6)
    got = orc.fb_vec_in(np.zeros((nx, nk, nm, 3), complex, order="F"), v, leftX, kx, In)
    A = np.einsum("rkm,xrml->xkml", In, v[:, 1:])
    want = np.fft.fft(A, axis=0) * np.exp(-1j * kx * leftX)[:, None, None, None]
    assert rel_l2(got, want) < 1e-13
    vf = _rand_fb((nx, nk, nm, 3), 7)
    got = orc.fb_vec_out(vf, leftX, kx, Out)
    B = np.einsum("krm,xkml->xrml", Out, vf) * np.exp(1j * kx * leftX)[:, None, None, None]
    want = np.zeros((nx, nr, nm, 3), complex)
    want[:, 1:] = nx * np.fft.ifft(B, axis=0)
    assert rel_l2(got, want) < 1e-13 and np.all(got[:, 0] == 0)
    e_fb = _rand_fb((nx, nk, nm, 6), 8)
    eb = orc.fb_eb_out(_rand_fb((nx, nr, nm, 6), 9), e_fb, vf, leftX, kx, Out)
    want6 = np.concatenate([orc.fb_vec_out(np.asfortranarray(e_fb[..., :3]), leftX, kx, Out),
                            orc.fb_vec_out(vf, leftX, kx, Out)], axis=-1)
    assert np.array_equal(eb, want6)


@pytest.mark.parametrize("modefilt", [0, 1, 2])
def test_fb_filtr_vs_numpy(orc, golden, modefilt):
    """fb_io.f90:230-308: back to x (unnormalised, with e^{+i kx leftX}),
    the first nxfilt cells times the profile (mode 0), the last nxfilt times
    the reversed profile (mode 1), both (mode 2), forward again and divided
    by nx e^{+i kx leftX}."""
    g = _ops(golden, "lpa_m2")
    nx, nk, nm = int(g["Nx"]), int(g["Nkr"]), int(g["Mtot"])
    leftX, kx = float(g["leftX"]) - 0.21, g["kx"]
    prof = np.linspace(0.0, 1.0, 9)[1:]
    nf = prof.size
    v = _rand_fb((nx, nk, nm, 3), 10)
    sh = np.exp(1j * kx * leftX)[:, None, None, None]
    a = nx * np.fft.ifft(v * sh, axis=0)
    if modefilt in (0, 2):
        a[:nf] *= prof[:, None, None, None]
    if modefilt in (1, 2):
        a[nx - nf:] *= prof[::-1, None, None, None]
    want = np.fft.fft(a, axis=0) / (nx * sh)
    got = orc.fb_filtr(v.copy(order="F"), leftX, kx, prof, modefilt)
    assert rel_l2(got, want) < 1e-13


def _rand_fb(shape, seed):
    rng = np.random.default_rng(seed)
    return np.asfortranarray(rng.standard_normal(shape) + 1j * rng.standard_normal(shape))


def _np_grad(s, Dp, Dm, kx, env):
    """numpy restatement of fb_grad (fb_math.f90:96-149 / fb_math_env.f90:18-61)."""
    nx, nk, nm = s.shape
    out = np.zeros((nx, nk, nm, 3), complex)
    K = (nm - 1) // 2
    for mi in range(nm):
        md = mi + 1 if env else mi
        out[:, :, mi, 0] = 1j * kx[:, None] * s[:, :, mi]
        lo = None
        if env:
            if mi > 0:
                lo = s[:, :, mi - 1]
        else:
            lo = s[:, :, mi - 1] if mi > 0 else (-np.conj(s[(-np.arange(nx)) % nx, :, 1]) if nm > 1 else 0 * s[:, :, 0])
        if lo is not None:
            sl = lo @ Dm[:, :, md]
            out[:, :, mi, 1] -= sl
            out[:, :, mi, 2] += 1j * sl
        if mi < nm - 1:
            sl = s[:, :, mi + 1] @ Dp[:, :, md]
            out[:, :, mi, 1] += sl
            out[:, :, mi, 2] += 1j * sl
    return out


@pytest.mark.parametrize("name,env", [("lpa_m2", False), ("lpa_m3_chunked", False),
                                      ("fel_env_k1", True)])
def test_fb_grad_vs_numpy(orc, golden, name, env):
    g = _ops(golden, name)
    nx, nk, nm = int(g["Nx"]), int(g["Nkr"]), int(g["Mtot"])
    s = _rand_fb((nx, nk, nm), 1)
    out = np.zeros((nx, nk, nm, 3), complex, order="F")
    f = orc.fb_grad_env if env else orc.fb_grad
    got = f(out, s, g["DpS2S"], g["DmS2S"], g["kx"])
    ref = _np_grad(s, g["DpS2S"], g["DmS2S"], g["kx"], env)
    assert rel_l2(got, ref) < 1e-13


def _np_rot(v, Dp, Dm, kx, env):
    """numpy restatement of fb_rot (fb_math.f90:18-94) and fb_rot_env
    (fb_math_env.f90:106-162, whose lower-neighbour term of the first
    component is computed and discarded, :146-151)."""
    nx, nk, nm, _ = v.shape
    nkl = Dp.shape[1]
    out = np.zeros((nx, nkl, nm, 3), complex)
    ext = -np.conj(v[(-np.arange(nx)) % nx, :, 1]) if nm > 1 else None
    for mi in range(nm):
        md = mi + 1 if env else mi
        out[:, :, mi, 1] -= 1j * kx[:, None] * v[:, :nkl, mi, 2]
        out[:, :, mi, 2] += 1j * kx[:, None] * v[:, :nkl, mi, 1]
        if mi < nm - 1:
            up = v[:, :, mi + 1]
            out[:, :, mi, 0] -= (1j * up[..., 1] - up[..., 2]) @ Dp[:, :, md]
            sl = up[..., 0] @ Dp[:, :, md]
            out[:, :, mi, 1] += 1j * sl
            out[:, :, mi, 2] -= sl
        lo = v[:, :, mi - 1] if mi > 0 else (None if env else ext)
        if lo is not None:
            if not env:
                out[:, :, mi, 0] -= (1j * lo[..., 1] + lo[..., 2]) @ Dm[:, :, md]
            sl = lo[..., 0] @ Dm[:, :, md]
            out[:, :, mi, 1] += 1j * sl
            out[:, :, mi, 2] += sl
    return out


@pytest.mark.parametrize("name,env", [("lpa_m2", False), ("lpa_m3_chunked", False),
                                      ("fel_env_k1", True)])
def test_fb_rot_vs_numpy(orc, golden, name, env):
    g = _ops(golden, name)
    nx, nk, nm = int(g["Nx"]), int(g["Nkr"]), int(g["Mtot"])
    v = _rand_fb((nx, nk, nm, 3), 3)
    out = np.zeros((nx, nk, nm, 3), complex, order="F")
    f = orc.fb_rot_env if env else orc.fb_rot
    got = f(out, v, g["DpS2S"], g["DmS2S"], g["kx"])
    assert rel_l2(got, _np_rot(v, g["DpS2S"], g["DmS2S"], g["kx"], env)) < 1e-13


def _np_div(v, Dp, Dm, kx, env):
    """numpy restatement of fb_div (fb_math.f90:150-199) and fb_div_env
    (fb_math_env.f90:62-104)."""
    nx, nk, nm, _ = v.shape
    nkl = Dp.shape[1]
    out = np.zeros((nx, nkl, nm), complex)
    ext = -np.conj(v[(-np.arange(nx)) % nx, :, 1]) if nm > 1 else None
    for mi in range(nm):
        md = mi + 1 if env else mi
        out[:, :, mi] += 1j * kx[:, None] * v[:, :nkl, mi, 0]
        lo = v[:, :, mi - 1] if mi > 0 else (None if env else ext)
        if lo is not None:
            out[:, :, mi] += (1j * lo[..., 2] - lo[..., 1]) @ Dm[:, :, md]
        if mi < nm - 1:
            up = v[:, :, mi + 1]
            out[:, :, mi] += (1j * up[..., 2] + up[..., 1]) @ Dp[:, :, md]
    return out


@pytest.mark.parametrize("name,env", [("lpa_m2", False), ("lpa_m3_chunked", False),
                                      ("fel_env_k1", True)])
def test_fb_div_vs_numpy(orc, golden, name, env):
    g = _ops(golden, name)
    nx, nk, nm = int(g["Nx"]), int(g["Nkr"]), int(g["Mtot"])
    v = _rand_fb((nx, nk, nm, 3), 4)
    out = np.zeros((nx, nk, nm), complex, order="F")
    f = orc.fb_div_env if env else orc.fb_div
    got = f(out, v, g["DpS2S"], g["DmS2S"], g["kx"])
    assert rel_l2(got, _np_div(v, g["DpS2S"], g["DmS2S"], g["kx"], env)) < 1e-13


def _np_graddiv(v, Dp, Dm, kx, env):
    """numpy restatement of fb_graddiv (fb_math.f90:201-293) and
    fb_graddiv_env (fb_math_env.f90:164-233): the divergence on one extra
    mode above (and, for the envelope, one below) the stored ones, then its
    gradient back on the stored modes."""
    nx, nk, nm, _ = v.shape
    lo0 = 1 if env else 0          # slot of the first stored mode in S
    ns = nm + 1 + lo0              # slots of the divergence
    S = np.zeros((nx, nk, ns), complex)
    refl = (-np.arange(nx)) % nx
    for j in range(ns):
        mi = j - lo0               # stored mode index (may be -1 or nm)
        if 0 <= mi < nm:
            S[:, :, j] += 1j * kx[:, None] * v[:, :, mi, 0]
        if mi >= 1:
            lo = v[:, :, mi - 1]
        elif not env and mi == 0 and nm > 1:
            lo = -np.conj(v[refl, :, 1])
        else:
            lo = None
        if lo is not None:
            S[:, :, j] += (1j * lo[..., 2] - lo[..., 1]) @ Dm[:, :, j]
        if mi < nm - 1:
            up = v[:, :, mi + 1]
            S[:, :, j] += (1j * up[..., 2] + up[..., 1]) @ Dp[:, :, j]
    out = np.zeros((nx, nk, nm, 3), complex)
    for mi in range(nm):
        j = mi + lo0
        out[:, :, mi, 0] = 1j * kx[:, None] * S[:, :, j]
        if j > 0:
            sl = S[:, :, j - 1] @ Dm[:, :, j]
        elif nm > 1:
            sl = -np.conj(S[refl, :, 1]) @ Dm[:, :, j]
        else:
            sl = 0
        out[:, :, mi, 1] -= sl
        out[:, :, mi, 2] += 1j * sl
        sl = S[:, :, j + 1] @ Dp[:, :, j]
        out[:, :, mi, 1] += sl
        out[:, :, mi, 2] += 1j * sl
    return out


@pytest.mark.parametrize("name,env", [("lpa_m2", False), ("lpa_m3_chunked", False),
                                      ("fel_env_k1", True)])
def test_fb_graddiv_vs_numpy(orc, golden, name, env):
    g = _ops(golden, name)
    nx, nk, nm = int(g["Nx"]), int(g["Nkr"]), int(g["Mtot"])
    v = _rand_fb((nx, nk, nm, 3), 5)
    f = orc.fb_graddiv_env if env else orc.fb_graddiv
    got = f(v.copy(order="F"), g["DpS2S"], g["DmS2S"], g["kx"])
    assert rel_l2(got, _np_graddiv(v, g["DpS2S"], g["DmS2S"], g["kx"], env)) < 1e-13


def test_graddiv_equals_grad_of_div_interior(orc, golden):
    """fb_graddiv builds the divergence on one extra mode; for the m=0..M-2
    outputs it equals grad(div v) formed with fb_div and fb_grad."""
    g = _ops(golden, "lpa_m3_chunked")
    nx, nk, nm = int(g["Nx"]), int(g["Nkr"]), int(g["Mtot"])
    v = _rand_fb((nx, nk, nm, 3), 2)
    gd = orc.fb_graddiv(v.copy(order="F"), g["DpS2S"], g["DmS2S"], g["kx"])
    d = orc.fb_div(np.zeros((nx, nk, nm), complex, order="F"), v, g["DpS2S"], g["DmS2S"], g["kx"])
    gg = orc.fb_grad(np.zeros((nx, nk, nm, 3), complex, order="F"), d, g["DpS2S"], g["DmS2S"], g["kx"])
    assert rel_l2(gd[:, :, : nm - 2], gg[:, :, : nm - 2]) < 1e-12


def test_boris_uniform_b_gyration(orc):
    """particle_tools.f90:18-56 in a uniform B: |p| is conserved and the
    rotation angle per step is 2 atan(dt B / (2 gamma))."""
    n = 64
    rng = np.random.default_rng(3)
    p = np.asfortranarray(rng.standard_normal((3, n)))
    p[2] = 0.0
    F = np.zeros((6, n), order="F")
    B = 0.7
    F[5] = B
    dt = 0.3
    p0 = p.copy()
    orc.push_velocs(p, F, dt)
    g = np.sqrt(1 + (p0 ** 2).sum(0))
    assert np.allclose(np.linalg.norm(p, axis=0), np.linalg.norm(p0, axis=0), rtol=1e-14)
    ang = np.arctan2(p0[0] * p[1] - p0[1] * p[0], (p0[:2] * p[:2]).sum(0))
    assert np.allclose(-ang, 2 * np.arctan(dt * B / (2 * g)), rtol=1e-12)


def test_boris_vs_numpy(orc):
    """particle_tools.f90:18-56 restated in numpy (half E kick, rotation by
    t = dt/2 B / gamma and s = 2 t / (1 + t^2), half E kick) on random
    momenta and fields, including strong fields."""
    rng = np.random.default_rng(18)
    n = 500
    p = np.asfortranarray(rng.standard_normal((3, n)) * 3)
    F = np.asfortranarray(rng.standard_normal((6, n)) * np.r_[[1.0] * 3, [5.0] * 3][:, None])
    dt = 0.3
    h = 0.5 * dt
    um = p + h * F[:3]
    g = np.sqrt(1.0 + (um * um).sum(0))
    t = h * F[3:] / g
    sv = 2 * t / (1 + (t * t).sum(0))
    u0 = um + np.cross(um, t, axis=0)
    up = um + np.cross(u0, sv, axis=0)
    want = up + h * F[:3]
    got = orc.push_velocs(p.copy(order="F"), F, dt)
    assert np.abs(got - want).max() < 1e-13 * np.abs(want).max()


def test_push_coords_half_step(orc):
    x = np.asfortranarray(np.random.default_rng(4).standard_normal((3, 10)))
    p = np.asfortranarray(np.random.default_rng(5).standard_normal((3, 10)))
    xc = np.zeros_like(x, order="F")
    x0 = x.copy()
    orc.push_coords(x, p, xc, 0.2)
    v = p / np.sqrt(1 + (p ** 2).sum(0))
    assert np.allclose(x, x0 + 0.2 * v, rtol=0, atol=1e-15)
    assert np.allclose(xc, 0.5 * (x0 + x), rtol=0, atol=1e-15)


def _particles(n, seed, x0=-2.0, x1=1.0, rmin=0.3, rmax=2.5):
    rng = np.random.default_rng(seed)
    x = rng.uniform(x0, x1, n)
    r = rng.uniform(rmin, rmax, n)
    th = rng.uniform(0, 2 * np.pi, n)
    c = np.asfortranarray(np.vstack([x, r * np.cos(th), r * np.sin(th)]))
    p = np.asfortranarray(rng.standard_normal((3, n)))
    w = rng.uniform(0.5, 1.5, n)
    return c, p, w


def test_dep_dens_conserves_charge(orc):
    """grid_deps.f90:89-147: linear weights sum to one, so with particles off
    the axis row the m=0 density sums to the total weight."""
    c, p, w = _particles(500, 6)
    rg = 0.25 * (np.arange(13) - 0.5)
    dens = np.zeros((64, 13, 2), complex, order="F")
    dens = orc.dep_dens(c, w, dens, -2.5, rg, 1 / 0.1, 1 / 0.25)
    assert abs(dens[:, :, 0].sum() - w.sum()) < 1e-12 * w.sum()


def test_envelope_deposits_single_particle(orc):
    """grid_deps_env.f90:18-162 for one particle: the current's J_z (the only
    component deposited) is w v_z / gamma S_x S_r e^{-i kx0 x} e^{-+i m theta}
    in modes +-m; the density takes the complex weight w e^{-i kx0 x} twice,
    w^2 e^{-2 i kx0 x}; a particle on the ghost row (r < dr / 2) is folded
    into row 1 with the sign flipped and row 0 cleared."""
    nx, nr, K = 16, 6, 2
    nm = 2 * K + 1
    dx, dr, leftX, kx0 = 0.1, 0.25, -0.8, 37.0
    rg = dr * (np.arange(nr) - 0.5)
    for r, th in ((0.61, 0.7), (0.07, 2.1)):
        x = leftX + 6.3 * dx
        c = np.asfortranarray([[x], [r * np.cos(th)], [r * np.sin(th)]])
        p = np.asfortranarray([[0.3], [-0.4], [1.7]])
        w = np.array([0.8])
        J = orc.dep_curr_env(c, p, w, np.zeros((nx, nr, nm, 3), complex, order="F"), leftX, rg,
                             1 / dx, 1 / dr, kx0)
        D = orc.dep_dens_env(c, w, np.zeros((nx, nr, nm), complex, order="F"), leftX, rg,
                             1 / dx, 1 / dr, kx0)
        ix = int(np.floor((x - leftX) / dx))
        ir = int(np.floor((r - rg[0]) / dr))
        sx = (x - leftX) / dx - ix
        sr = (r - rg[ir]) / dr
        S = np.outer([1 - sx, sx], [1 - sr, sr])
        car = np.exp(-1j * kx0 * x)
        vz = p[2, 0] / np.sqrt(1 + (p[:, 0] ** 2).sum())
        Jz = np.zeros((nx, nr, nm), complex)
        Dn = np.zeros((nx, nr, nm), complex)
        for m in range(-K, K + 1):
            ph = np.exp(-1j * m * th)
            Jz[ix:ix + 2, ir:ir + 2, m + K] = w[0] * vz * S * car * ph
            Dn[ix:ix + 2, ir:ir + 2, m + K] = (w[0] * car) ** 2 * S * ph
        for G in (Jz, Dn):
            G[:, 1] -= G[:, 0]
            G[:, 0] = 0
        assert (ir == 0) == (r < 0.5 * dr)
        assert np.abs(J[..., 2] - Jz).max() < 1e-14 and np.all(J[..., :2] == 0)
        assert np.abs(D - Dn).max() < 1e-14


def test_envelope_gather_and_correction_single_particle(orc):
    """grid_deps_env.f90:164-283: the gather of one particle is
    sum over m = -K..K and the 2 x 2 nodes of Re(S_x S_r e^{+i kx0 x}
    e^{+i m theta} F_m), with theta's phase 1 on the axis;
    eb_correction_env scales every mode by 1/pi and writes row 0 as -row 1
    (+row 1 with a single mode)."""
    rng = np.random.default_rng(13)
    nx, nr, K = 12, 5, 2
    nm = 2 * K + 1
    dx, dr, leftX, kx0 = 0.2, 0.3, -1.0, 21.0
    rg = dr * (np.arange(nr) - 0.5)
    F = np.asfortranarray(rng.standard_normal((nx, nr, nm, 6))
                          + 1j * rng.standard_normal((nx, nr, nm, 6)))
    for r, th in ((0.52, -1.1), (0.0, 0.0)):
        x = leftX + 4.7 * dx
        c = np.asfortranarray([[x], [r * np.cos(th)], [r * np.sin(th)]])
        got = orc.proj_fld_env(c, np.array([1.3]), F, np.zeros((6, 1), order="F"), leftX, rg,
                               1 / dx, 1 / dr, kx0)
        ix = int(np.floor((x - leftX) / dx))
        ir = int(np.floor((r - rg[0]) / dr))
        sx, sr = (x - leftX) / dx - ix, (r - rg[ir]) / dr
        S = np.outer([1 - sx, sx], [1 - sr, sr]) * np.exp(1j * kx0 * x)
        want = np.zeros(6)
        for m in range(-K, K + 1):
            ph = np.exp(1j * m * th)  # th = 0 on the axis: phase 1
            for l in range(6):
                want[l] += np.real(S * ph * F[ix:ix + 2, ir:ir + 2, m + K, l]).sum()
        assert np.abs(got[:, 0] - want).max() < 1e-13 * np.abs(F).max()
    for modes, sign in ((nm, -1.0), (1, 1.0)):
        G = np.asfortranarray(F[:, :, :modes].copy())
        out = orc.eb_correction_env(G.copy(order="F"))
        assert np.allclose(out[:, 1:], G[:, 1:] / np.pi, rtol=1e-15, atol=0)
        assert np.array_equal(out[:, 0], sign * out[:, 1])


def test_plain_deposit_gather_correction_single_particle(orc):
    """grid_deps.f90:18-266 for one particle: J_l = w v_l / gamma S_x S_r
    e^{-i m theta} on modes m = 0..M-1 and rho = w S_x S_r e^{-i m theta},
    both folded at the ghost row; the gather sums Re(S_x S_r e^{+i m theta}
    F_m) with theta's phase 0 on the axis (only m = 0 there); eb_correction
    scales m = 0 by 1/(2 pi) and m > 0 by 1/pi, row 0 = +row 1 for m = 0
    and -row 1 for m > 0.  A particle at rest deposits no current."""
    rng = np.random.default_rng(16)
    nx, nr, nm = 12, 6, 3
    dx, dr, leftX = 0.15, 0.2, -0.9
    rg = dr * (np.arange(nr) - 0.5)
    F = np.asfortranarray(rng.standard_normal((nx, nr, nm, 6))
                          + 1j * rng.standard_normal((nx, nr, nm, 6)))
    for r, th, p in ((0.47, 0.9, (0.2, -0.6, 1.1)), (0.05, -2.0, (1.0, 0.5, -0.3)),
                     (0.0, 0.0, (0.3, 0.0, 0.0)), (0.33, 1.3, (0.0, 0.0, 0.0))):
        x = leftX + 5.4 * dx
        c = np.asfortranarray([[x], [r * np.cos(th)], [r * np.sin(th)]])
        pp = np.asfortranarray(np.array(p, float)[:, None])
        w = np.array([0.7])
        J = orc.dep_curr(c, pp, w, np.zeros((nx, nr, nm, 3), complex, order="F"), leftX, rg,
                         1 / dx, 1 / dr)
        D = orc.dep_dens(c, w, np.zeros((nx, nr, nm), complex, order="F"), leftX, rg,
                         1 / dx, 1 / dr)
        E = orc.proj_fld(c, w, F, np.zeros((6, 1), order="F"), leftX, rg, 1 / dx, 1 / dr)
        ix = int(np.floor((x - leftX) / dx))
        ir = int(np.floor((r - rg[0]) / dr))
        sx, sr = (x - leftX) / dx - ix, (r - rg[ir]) / dr
        S = np.outer([1 - sx, sx], [1 - sr, sr])
        ph = np.array([np.exp(-1j * m * th) if (r > 0 or m == 0) else 0 for m in range(nm)])
        v = np.array(p) / np.sqrt(1 + np.sum(np.square(p)))
        Jw = np.zeros((nx, nr, nm, 3), complex)
        Dw = np.zeros((nx, nr, nm), complex)
        for m in range(nm):
            Dw[ix:ix + 2, ir:ir + 2, m] = w[0] * S * ph[m]
            if any(p):
                for l in range(3):
                    Jw[ix:ix + 2, ir:ir + 2, m, l] = w[0] * v[l] * S * ph[m]
        for G in (Jw, Dw):
            G[:, 1] -= G[:, 0]
            G[:, 0] = 0
        assert np.abs(J - Jw).max() < 1e-14 and np.abs(D - Dw).max() < 1e-14
        want = [sum(np.real(S * np.conj(ph[m]) * F[ix:ix + 2, ir:ir + 2, m, l]).sum()
                    for m in range(nm)) for l in range(6)]
        assert np.abs(E[:, 0] - want).max() < 1e-13
    out = orc.eb_correction(F.copy(order="F"))
    scale = np.array([0.5, 1.0, 1.0]) / np.pi
    assert np.allclose(out[:, 1:], F[:, 1:] * scale[None, None, :, None], rtol=1e-15, atol=0)
    assert np.array_equal(out[:, 0, 0], out[:, 1, 0])
    assert np.array_equal(out[:, 0, 1:], -out[:, 1, 1:])


def test_chunked_deposit_matches_serial(orc):
    """grid_deps_chnk.f90: same grid as the serial deposit when chunk 0 holds
    no particle next to x-node 0."""
    c, p, w = _particles(4000, 7, -2.3, 3.5)
    rg = 0.25 * (np.arange(13) - 0.5)
    leftX, nx, nch = -2.5, 64, 4
    xg = leftX + 0.1 * np.arange(nx)
    ids, ind, go = orc.chunk_coords_boundaries(c, np.array([leftX, xg[-1], 0, 100.0]), xg, nch)
    order = np.argsort(ids, kind="stable")[go:]
    c2, p2, w2 = (np.asfortranarray(a[..., order]) for a in (c, p, w))
    ser = orc.dep_curr(c2, p2, w2, np.zeros((nx, 13, 2, 3), complex, order="F"), leftX, rg, 10.0, 4.0)
    chk = orc.dep_curr_chnk(c2, p2, w2, np.zeros((nx, 13, 2, 3), complex, order="F"), ind, 3,
                            leftX, rg, 10.0, 4.0)
    assert rel_l2(chk, ser) < 1e-13


def test_bookkeeping_known_answers(orc):
    """particle_tools.f90:130-208, 270-324: sortpartsout keeps the 0-based
    indices of particles with lims(1) <= x <= lims(2) and lims(3) <= r^2 <=
    lims(4); chunk_coords_boundaries labels each kept particle with
    floor((x - Xgrid(0)) / L), L = Xgrid(len / nchnk) - Xgrid(0), the others
    with -2, returns the chunk offsets and the count outside (a kept
    particle past the last chunk is counted in none); align_data
    gathers the first len(idx) particles by index and keeps the rest."""
    rng = np.random.default_rng(14)
    n = 3000
    c = np.asfortranarray(np.vstack([rng.uniform(-3.0, 4.0, n), rng.uniform(-1.5, 1.5, n),
                                     rng.uniform(-1.5, 1.5, n)]))
    c[0, :5] = [-2.0, 3.0, 0.0, 1.0, -1.0]  # on the x limits and on chunk edges
    xg = -2.0 + 0.05 * np.arange(101)
    lims = np.array([-2.0, 3.0, 0.01, 1.44])
    x, r2 = c[0], c[1] ** 2 + c[2] ** 2
    keep = (x >= lims[0]) & (x <= lims[1]) & (r2 >= lims[2]) & (r2 <= lims[3])
    idx, num = orc.sortpartsout(c, lims)
    assert num == keep.sum() and np.array_equal(idx[:num], np.flatnonzero(keep))
    assert np.all(idx[num:] == 0)
    nch = 4
    ids, ind, go = orc.chunk_coords_boundaries(c, lims, xg, nch)
    L = xg[xg.size // nch] - xg[0]
    want = np.where(keep, np.floor((x - xg[0]) * (1.0 / L)), -2).astype(np.int8)
    assert np.array_equal(ids, want) and go == n - keep.sum()
    # x = lims(2) at the grid's right edge falls in chunk nchnk, one past the
    # last: labelled so, counted in no chunk (the Fortran's count array
    # would be written one past its end there)
    assert ids[1] == nch
    counts = np.bincount(want[keep & (want < nch)], minlength=nch)
    assert np.array_equal(ind, np.concatenate([[0], np.cumsum(counts)]))
    order = np.argsort(ids, kind="stable")[go:].astype(np.int64)
    d = np.asfortranarray(rng.standard_normal((3, n)))
    got = orc.align_data_vec(d.copy(order="F"), order)
    assert np.array_equal(got[:, :order.size], d[:, order])
    assert np.array_equal(got[:, order.size:], d[:, order.size:])
    s = rng.standard_normal(n)
    got = orc.align_data_scl(s.copy(), order)
    assert np.array_equal(got[:order.size], s[order]) and np.array_equal(got[order.size:],
                                                                          s[order.size:])


def test_chunked_envelope_deposits_match_serial(orc):
    """grid_deps_env_chnk.f90: the chunked envelope current and density equal
    the serial ones when chunk 0 holds no particle next to x-node 0."""
    c, p, w = _particles(3000, 17, -2.3, 3.5)
    rg = 0.25 * (np.arange(13) - 0.5)
    leftX, nx, nch, nm, kx0 = -2.5, 64, 4, 3, 11.0
    xg = leftX + 0.1 * np.arange(nx)
    ids, ind, go = orc.chunk_coords_boundaries(c, np.array([leftX, xg[-1], 0, 100.0]), xg, nch)
    order = np.argsort(ids, kind="stable")[go:]
    c2, p2, w2 = (np.asfortranarray(a[..., order]) for a in (c, p, w))
    zJ = np.zeros((nx, 13, nm, 3), complex, order="F")
    zD = np.zeros((nx, 13, nm), complex, order="F")
    ser = orc.dep_curr_env(c2, p2, w2, zJ.copy(order="F"), leftX, rg, 10.0, 4.0, kx0)
    chk = orc.dep_curr_env_chnk(c2, p2, w2, zJ.copy(order="F"), ind, 3, leftX, rg, 10.0, 4.0,
                                kx0)
    assert np.abs(ser).max() > 0 and rel_l2(chk, ser) < 1e-13
    ser = orc.dep_dens_env(c2, w2, zD.copy(order="F"), leftX, rg, 10.0, 4.0, kx0)
    chk = orc.dep_dens_env_chnk(c2, w2, zD.copy(order="F"), ind, 3, leftX, rg, 10.0, 4.0, kx0)
    assert rel_l2(chk, ser) < 1e-13


def test_undulator_closed_form(orc):
    """devices.f90:162-203 inside the flat part of the undulator."""
    n = 200
    rng = np.random.default_rng(8)
    c = np.asfortranarray(np.vstack([rng.uniform(2.0, 8.0, n), rng.uniform(-0.1, 0.1, n),
                                     np.zeros(n)]))
    F = np.zeros((6, n), order="F")
    a0, lam, X0, Lx = 1.3, 1.0, 0.5, 10.0
    orc.undul_analytic(c, F, 0.0, np.array([a0, lam, X0, Lx]))
    ku = 2 * np.pi / lam
    assert np.allclose(F[4], a0 * np.sin(ku * (c[0] - X0)) * np.cosh(ku * c[1]), atol=1e-14)
    assert np.allclose(F[3], a0 * np.cos(ku * (c[0] - X0)) * np.sinh(ku * c[1]), atol=1e-14)


def test_mapped_undulator_known_answers(orc):
    """devices.f90:18-115: the map column j (1-based) sits at Xleft + j dx
    (the spline at ix reads a0(:, ix-1:ix+1)); the quadratic weights sum to
    one, so a constant map returns the taper's amplitude exactly; particles
    outside [Xleft + dx, Xright - dx] get nothing."""
    rng = np.random.default_rng(11)
    lam, xleft, mdx, nmap = 1.0, 0.3, 0.01, 700
    xright = xleft + nmap * mdx
    n = 400
    x = rng.uniform(xleft + 2 * mdx, xright - 2 * mdx, n)
    y = rng.uniform(-0.05, 0.05, n)
    c = np.asfortranarray(np.vstack([x, y, np.zeros(n)]))
    ku = 2 * np.pi / lam
    xc = xleft + mdx * np.arange(1, nmap + 1)
    # a sampled wiggler: the spline smooths sin(ku x) by about (ku dx)^2 / 8
    a0 = np.asfortranarray(np.stack([np.sin(ku * xc), np.cos(ku * xc)]))
    F = orc.undul_mapped(c, np.zeros((6, n), order="F"), 0.0, a0, np.array([lam, xleft, mdx]))
    tol = (ku * mdx) ** 2 / 4
    assert np.abs(F[4] - np.sin(ku * x) * np.cosh(ku * y)).max() < tol
    assert np.abs(F[3] - np.cos(ku * x) * np.sinh(ku * y)).max() < tol
    # the same samples one column along miss by about ku dx
    a1 = np.asfortranarray(np.stack([np.sin(ku * (xc - mdx)), np.cos(ku * (xc - mdx))]))
    F1 = orc.undul_mapped(c, np.zeros((6, n), order="F"), 0.0, a1, np.array([lam, xleft, mdx]))
    assert np.abs(F1[4] - np.sin(ku * x) * np.cosh(ku * y)).max() > 10 * tol
    # a constant map under the taper: amp = 1 + taper (x - x_shift - Xleft - Lx/2) / (Lx/2)
    Lx, taper = 0.8 * nmap * mdx, 0.1
    x_shift = 0.5 * (nmap * mdx - Lx)
    ones = np.asfortranarray(np.stack([np.ones(nmap), np.zeros(nmap)]))
    xe = np.concatenate([x, [xleft + 0.5 * mdx, xright - 0.5 * mdx]])
    ce = np.asfortranarray(np.vstack([xe, np.zeros(n + 2), np.zeros(n + 2)]))
    Ft = orc.undul_mapped_tap(ce, np.zeros((6, n + 2), order="F"), 0.0, ones,
                              np.array([lam, xleft, mdx, Lx, taper]))
    amp = 1 + taper * (x - x_shift - xleft - 0.5 * Lx) / (0.5 * Lx)
    assert np.allclose(Ft[4, :n], amp, rtol=0, atol=1e-14)
    assert np.all(Ft[:, n:] == 0) and np.all(Ft[3] == 0)


def test_planewave_and_gaussbeam_known_answers(orc):
    """devices.f90:205-297: the plane wave's field (E_z, B_x, B_y) =
    (1, sin theta, -cos theta) a0 ramp sin(k0 (x cos theta + y sin theta - t)
    + phi0) with linear ramps of length `ramp` inside [X0, X0 + Lx]; the
    Gaussian beam's E_z = a0 exp(-sum (x_i / L_i)^2) sin(2 pi x' / lambda)
    with x' = x - x0 - axis t, and B_y = -axis E_z; nothing else is written."""
    rng = np.random.default_rng(12)
    n = 300
    c = np.asfortranarray(rng.uniform(-1.0, 1.0, (3, n)) * np.array([[6.0], [1.0], [1.0]]))
    x, y, z = c
    a0, lam, X0, Lx, ramp, th, phi0, t = 0.7, 0.9, -4.0, 8.0, 1.5, 0.3, 0.2, 0.4
    F = orc.planewave(c, np.zeros((6, n), order="F"), t,
                      np.array([a0, lam, X0, Lx, ramp, th, phi0]))
    env = np.clip(np.minimum(x - X0, X0 + Lx - x) / ramp, 0.0, 1.0)
    e = a0 * env * np.sin(2 * np.pi / lam * (x * np.cos(th) + y * np.sin(th) - t) + phi0)
    assert np.abs(F[2] - e).max() < 1e-14
    assert np.abs(F[3] - e * np.sin(th)).max() < 1e-14
    assert np.abs(F[4] + e * np.cos(th)).max() < 1e-14
    assert np.all(F[[0, 1, 5]] == 0)
    prm = np.array([0.8, 1.0, 0.5, 0.1, -0.2, 2.0, 0.7, 0.9])
    G = orc.gaussbeam(c, np.zeros((6, n), order="F"), t, a0, prm)
    xp = x - prm[2] - prm[1] * t
    e = a0 * np.exp(-(xp / prm[5]) ** 2 - ((y - prm[3]) / prm[6]) ** 2
                    - ((z - prm[4]) / prm[7]) ** 2) * np.sin(2 * np.pi / prm[0] * xp)
    assert np.abs(G[2] - e).max() < 1e-14
    assert np.abs(G[4] + prm[1] * e).max() < 1e-14
    assert np.all(G[[0, 1, 3, 5]] == 0)


def test_spectral_elementwise_known_answers(orc):
    """maxwell_solvers.f90:18-60, 131-164, 228-318 restated in numpy:
    PSATD with space charge (E' = C1 . [E, G, J, grad rho_n, grad rho_n+1],
    G' = C2 . [the same, from the old E and G]), the Poisson correction
    J += (grad div J + (grad rho_n+1 - grad rho_n) / dt) / w^2, and the
    real multiply / complex add of the vector and scalar helpers."""
    rng = np.random.default_rng(15)
    sh = (10, 7, 2)
    eg = _rand_fb(sh + (6,), 1)
    j, gn, gp, gd = (_rand_fb(sh + (3,), s) for s in (2, 3, 4, 5))
    C1 = np.asfortranarray(rng.standard_normal(sh + (5,)))
    C2 = np.asfortranarray(rng.standard_normal(sh + (5,)))
    terms = [eg[..., :3], eg[..., 3:], j, gn, gp]
    e_new = sum(C1[..., i, None] * t for i, t in enumerate(terms))
    g_new = sum(C2[..., i, None] * t for i, t in enumerate(terms))
    out = orc.maxwell_push_with_spchrg(eg.copy(order="F"), j, gn, gp, C1, C2)
    assert np.abs(out[..., :3] - e_new).max() < 1e-13
    assert np.abs(out[..., 3:] - g_new).max() < 1e-13
    w2_inv = np.asfortranarray(rng.uniform(0.1, 2.0, sh))
    dt_inv = 7.0
    out = orc.poiss_corr(j.copy(order="F"), gd, gn, gp, dt_inv, w2_inv)
    assert np.abs(out - (j + (gd + (gp - gn) * dt_inv) * w2_inv[..., None])).max() < 1e-13
    A = np.asfortranarray(rng.standard_normal(sh))
    assert np.array_equal(orc.omp_mult_vec(j.copy(order="F"), A), j * A[..., None])
    assert np.array_equal(orc.omp_mult_scl(gd[..., 0].copy(order="F"), A), gd[..., 0] * A)
    assert np.array_equal(orc.omp_add_vec(j.copy(order="F"), gd), j + gd)
    assert np.array_equal(orc.omp_add_scl(gn[..., 1].copy(order="F"), gp[..., 2].copy(order="F")),
                          gn[..., 1] + gp[..., 2])


def test_static_field_routines_known_answers(orc):
    """maxwell_solvers.f90:98-129, 166-226 restated in numpy:
    maxwell_init_push adds C1 . [J, grad rho] to E and C2 . [J, grad rho]
    to G (complex coefficients), poiss_corr_stat adds (grad div J + DT(kx)
    grad rho) / w^2 to J, and field_drift multiplies every component by
    exp(-i dt beta0 kx / 2)."""
    rng = np.random.default_rng(17)
    sh = (9, 5, 2)
    eg = _rand_fb(sh + (6,), 11)
    j, gr, gd = (_rand_fb(sh + (3,), s) for s in (12, 13, 14))
    C1, C2 = _rand_fb(sh + (2,), 15), _rand_fb(sh + (2,), 16)
    out = orc.maxwell_init_push(eg.copy(order="F"), j, gr, C1, C2)
    assert np.abs(out[..., :3] - (eg[..., :3] + C1[..., :1] * j + C1[..., 1:] * gr)).max() < 1e-13
    assert np.abs(out[..., 3:] - (eg[..., 3:] + C2[..., :1] * j + C2[..., 1:] * gr)).max() < 1e-13
    DT = rng.standard_normal(sh[0]) + 1j * rng.standard_normal(sh[0])
    w2_inv = np.asfortranarray(rng.uniform(0.1, 2.0, sh))
    out = orc.poiss_corr_stat(j.copy(order="F"), gd, gr, DT, w2_inv)
    want = j + (gd + DT[:, None, None, None] * gr) * w2_inv[..., None]
    assert np.abs(out - want).max() < 1e-13
    kx = rng.uniform(-30.0, 30.0, sh[0])
    out = orc.field_drift(eg.copy(order="F"), kx, 0.99, 0.4)
    want = eg * np.exp(-0.5j * 0.4 * 0.99 * kx)[:, None, None, None]
    assert np.abs(out - want).max() < 1e-13


def test_psatd_vacuum_matches_analytic(orc, golden):
    """maxwell_solvers.f90:62-96 with J = 0 rotates (E, G) by exp(i w dt):
    N steps equal one step of N dt."""
    g = _ops(golden, "plain_m1_vacuum")
    nx, nk, nm = int(g["Nx"]), int(g["Nkr"]), int(g["Mtot"])
    w = g["w"]
    dt = 0.1
    def coeffs(t):
        C1 = np.zeros(w.shape + (3,), order="F")
        C2 = np.zeros(w.shape + (3,), order="F")
        C1[..., 0], C1[..., 1], C1[..., 2] = np.cos(t * w), np.sin(t * w) / w, -np.sin(t * w) / w
        C2[..., 0], C2[..., 1], C2[..., 2] = -w * np.sin(t * w), np.cos(t * w), 1 - np.cos(t * w)
        return C1, C2
    eg = _rand_fb((nx, nk, nm, 6), 9)
    j = np.zeros((nx, nk, nm, 3), complex, order="F")
    a = eg.copy(order="F")
    C1, C2 = coeffs(dt)
    for _ in range(5):
        a = orc.maxwell_push_wo_spchrg(a, j, C1, C2)
    C1, C2 = coeffs(5 * dt)
    b = orc.maxwell_push_wo_spchrg(eg.copy(order="F"), j, C1, C2)
    assert rel_l2(a, b) < 1e-12


def test_oracle_intens_profo_is_the_angular_sum(orc):
    """utils.f90:18-57 restated: |sum_k e^{i k phi} F_k|^2 summed over x and
    components, per angle phi_iO = 2 pi iO / (NO - 1) and row ir >= 1."""
    rng = np.random.default_rng(5)
    F = rng.standard_normal((9, 6, 5, 3)) + 1j * rng.standard_normal((9, 6, 5, 3))
    NO, K = 8, 2
    got = orc.intens_profo(F, NO)
    ref = np.zeros((NO, 5))
    for io in range(NO):
        ph = np.exp(1j * 2 * np.pi * io / (NO - 1) * np.arange(-K, K + 1))
        s = (F[:, 1:] * ph[None, None, :, None]).sum(2)
        ref[io] = (np.abs(s) ** 2).sum(-1).sum(0)
    assert np.abs(got - ref).max() <= 1e-13 * np.abs(ref).max()
    with pytest.raises(ValueError):
        orc.intens_profo(F[:, :, :4], NO)
