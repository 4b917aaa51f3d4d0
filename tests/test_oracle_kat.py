"""Known-answer tests that pin the CPU oracle (the reference ships no tests or
golden vectors and cannot be compiled here).  CPU only."""
import numpy as np
import pytest

import les_gb300.config as C


@pytest.fixture(scope="module")
def O(oracle_lib):
    return oracle_lib.Oracle


def rel(a, b):
    nb = np.linalg.norm(b)
    return np.linalg.norm(a - b) / (nb if nb > 0 else 1.0)


@pytest.mark.parametrize("n", [8, 12, 16, 24, 32, 48, 64, 96, 128])
def test_fft_matches_numpy(O, n):
    """rfftwnd semantics (fft.f90:40-47): unnormalised r2c along x then y,
    complex (lh,ny) over (ld,ny); c2r of an r2c returns nx*ny times the input."""
    cfg = C.make_config(n, n, 4)
    d = C.dims(cfg)
    o = O(cfg)
    rng = np.random.default_rng(n)
    for big in (0, 1):
        nn = 3 * n // 2 if big else n
        ld = d["ld_big"] if big else d["ld"]
        x = rng.standard_normal((2, nn, ld))
        p = x.copy()
        o.call("fft_r2c", p, ints=(2, big))
        ref = np.fft.fft2(x[:, :, :nn])[:, :, :nn // 2 + 1]
        assert rel(p.view(np.complex128), ref) < 1e-15 * 20
        o.call("fft_c2r", p, ints=(2, big))
        assert rel(p[:, :, :nn], nn * nn * x[:, :, :nn]) < 1e-15 * 20


def test_c2r_ignores_imag_of_self_conjugate_columns(O):
    """FFTW's halfcomplex pass drops Im of the kx = 0 and kx = nx/2 entries
    after the y pass: a non-Hermitian kx=0 column gives Re(ifft) there."""
    cfg = C.make_config(16, 16, 4)
    o = O(cfg)
    rng = np.random.default_rng(1)
    spec = (rng.standard_normal((1, 16, 9)) + 1j * rng.standard_normal((1, 16, 9)))
    p = np.ascontiguousarray(spec).view(np.float64).copy()
    o.call("fft_c2r", p, ints=(1, 0))
    # expected: y-inverse per column, then real inverse along x keeping Re of columns 0 and nx/2
    t = np.fft.ifft(spec, axis=1) * 16
    t[:, :, 0] = t[:, :, 0].real
    t[:, :, 8] = t[:, :, 8].real
    expect = np.fft.irfft(t, n=16, axis=2) * 16
    assert rel(p[:, :, :16], expect) < 1e-14


@pytest.mark.parametrize("kx,ky", [(1, 0), (3, 2), (5, -7), (0, 4)])
def test_spectral_derivatives_of_modes(O, kx, ky):
    """ddx/ddy (ddx.f90, ddy.f90) are exact for resolved trigonometric modes."""
    n = 32
    cfg = C.make_config(n, n, 4)
    d = C.dims(cfg)
    o = O(cfg)
    x = np.arange(n) * 2 * np.pi / n
    X, Y = np.meshgrid(x, x, indexing="xy")
    f = np.zeros((cfg.nz, n, d["ld"]))
    f[:, :, :n] = np.sin(kx * X + ky * Y + 0.3)
    dx = np.zeros_like(f); dy = np.zeros_like(f)
    o.call("ddx", dx, f, ints=(cfg.nz,))
    o.call("ddy", dy, f, ints=(cfg.nz,))
    ex = kx * np.cos(kx * X + ky * Y + 0.3)
    ey = ky * np.cos(kx * X + ky * Y + 0.3)
    assert np.abs(dx[0, :, :n] - ex).max() < 1e-12
    assert np.abs(dy[0, :, :n] - ey).max() < 1e-12


def test_filt_da_kills_nyquist(O):
    """filt_da (filt_da.f90:26-38) overwrites f with its Nyquist-filtered self."""
    n = 16
    cfg = C.make_config(n, n, 4)
    d = C.dims(cfg)
    o = O(cfg)
    x = np.arange(n) * 2 * np.pi / n
    X, Y = np.meshgrid(x, x, indexing="xy")
    base = np.sin(2 * X + Y)
    f = np.zeros((cfg.nz, n, d["ld"]))
    f[:, :, :n] = base + np.cos(8 * X) + np.cos(8 * Y)  # Nyquist in x and y
    dx = np.zeros_like(f); dy = np.zeros_like(f)
    o.call("filt_da", f, dx, dy, ints=(cfg.nz,))
    assert np.abs(f[1, :, :n] - base).max() < 1e-13
    assert np.abs(dx[1, :, :n] - 2 * np.cos(2 * X + Y)).max() < 1e-12


def test_three_halves_rule_product_is_exact(O):
    """dealias1 -> pointwise product on the 3/2 grid -> dealias2 equals the
    exact product truncated to the resolved band (convec.f90, dealias1/2)."""
    n = 16
    cfg = C.make_config(n, n, 4)
    d = C.dims(cfg)
    o = O(cfg)
    rng = np.random.default_rng(4)

    def bandlimited():
        s = np.zeros((n, n // 2 + 1), complex)
        for ky in list(range(0, n // 2)) + list(range(n // 2 + 1, n)):
            for kx in range(n // 2):
                s[ky, kx] = rng.standard_normal() + 1j * rng.standard_normal()
        s[0, 0] = s[0, 0].real
        return np.fft.irfft2(s, s=(n, n))
    a, b = bandlimited(), bandlimited()
    fa = np.zeros((1, n, d["ld"])); fb = np.zeros_like(fa)
    fa[0, :, :n] = a; fb[0, :, :n] = b
    ba = np.zeros((1, d["ny2"], d["ld_big"])); bb = np.zeros_like(ba)
    o.call("dealias1", fa, ba, ints=(1,))
    o.call("dealias1", fb, bb, ints=(1,))
    prod = np.zeros_like(ba)
    prod[:, :, :d["nx2"]] = ba[:, :, :d["nx2"]] * bb[:, :, :d["nx2"]]
    out = np.zeros_like(fa)
    o.call("dealias2", out, prod, ints=(1,))
    # exact: evaluate a, b on a 4n grid (exact for band-limited fields),
    # multiply, and keep the modes padd/unpadd keep (|kx| < n/2, ky != n/2)
    m = 4 * n

    def up(f):
        S = np.fft.rfft2(f)
        Sb = np.zeros((m, m // 2 + 1), complex)
        for ky in range(n):
            kb = ky if ky < n // 2 else ky + (m - n)
            Sb[kb, :n // 2] = S[ky, :n // 2]
        return np.fft.irfft2(Sb * (m * m) / (n * n), s=(m, m))
    Pb = np.fft.rfft2(up(a) * up(b)) * (n * n) / (m * m)
    P = np.zeros((n, n // 2 + 1), complex)
    for ky in range(n):
        if ky == n // 2:
            continue
        kb = ky if ky < n // 2 else ky + (m - n)
        P[ky, :n // 2] = Pb[kb, :n // 2]
    exact = np.fft.irfft2(P, s=(n, n))
    assert np.abs(out[0, :, :n] - exact).max() < 1e-12 * max(1.0, np.abs(exact).max())


def test_tridag_array_vs_dense(O):
    """tridag_array (tridag_array.f90) solves each (kx,ky) system; compare one
    non-skipped mode with a dense solve."""
    cfg = C.make_config(8, 8, 10)
    d = C.dims(cfg)
    o = O(cfg)
    rng = np.random.default_rng(2)
    n = cfg.nz + 1
    shp = (n, cfg.ny, d["lh"])
    a = rng.uniform(0.5, 1, shp); c = rng.uniform(0.5, 1, shp)
    b = -(a + c + rng.uniform(0.2, 1, shp))
    r = rng.standard_normal(shp + (2,))
    u = np.zeros_like(r)
    assert o.call("tridag_array", a, b, c, r, u) == 0
    for jy, jx in [(1, 1), (2, 3), (7, 0)]:
        M = np.diag(b[:, jy, jx]) + np.diag(a[1:, jy, jx], -1) + np.diag(c[:-1, jy, jx], 1)
        rhs = r[:, jy, jx, 0] + 1j * r[:, jy, jx, 1]
        sol = np.linalg.solve(M, rhs)
        got = u[:, jy, jx, 0] + 1j * u[:, jy, jx, 1]
        assert rel(got, sol) < 1e-13


def test_test_filter_transfer(O):
    """test_filter_init (test_filtermodule.f90:32-63): sharp cutoff at
    k2 >= (pi/(alpha*delta))^2 with 1/(nx*ny) folded in; modes below the
    cutoff pass unchanged, above vanish."""
    n = 32
    cfg = C.make_config(n, n, 4)
    d = C.dims(cfg)
    o = O(cfg)
    G = np.zeros((cfg.ny, d["lh"]))
    o.call("filter_G", G, ints=(0,))
    kxs = np.zeros_like(G); kys = np.zeros_like(G)
    o.call("wavenumbers", kxs, kys)
    k2 = kxs ** 2 + kys ** 2
    dx = 2 * np.pi / n
    kc2 = (np.pi / (2 * dx)) ** 2
    inside = (k2 < kc2)
    inside[:, -1] = False
    inside[n // 2, :] = False
    assert np.all(G[inside] == 1.0 / (n * n))
    assert np.all(G[~inside] == 0.0)
    x = np.arange(n) * 2 * np.pi / n
    X, Y = np.meshgrid(x, x, indexing="xy")
    for (kx, ky), keep in [((3, 4), True), ((9, 9), False)]:
        f = np.zeros((n, d["ld"]))
        f[:, :n] = np.cos(kx * X + ky * Y)
        o.call("test_filter", f, ints=(0,))
        expect = np.cos(kx * X + ky * Y) if keep else 0.0 * X
        assert np.abs(f[:, :n] - expect).max() < 1e-13


def test_interpolag_reproduces_linear_fields(O):
    """interpolag_Sdep (interpolag_Sdep.f90:302-372): trilinear
    interpolation is exact for F linear in (x,y,z) at interior points."""
    n, nzl = 16, 12
    cfg = C.make_config(n, n, nzl, dt=2e-4)
    o = O(cfg)
    nz = cfg.nz
    jz, jy, jx = np.meshgrid(np.arange(nz), np.arange(n), np.arange(n + 2), indexing="ij")
    F = 1.0 + 0.3 * jx + 0.2 * jy + 0.1 * jz
    for nm in ["F_LM", "F_MM", "F_QN", "F_NN"]:
        o.set(nm, F)
    rng = np.random.default_rng(8)
    dx = 2 * np.pi / n
    dzz = 1.0 / (nz - 1)
    # accumulated velocities over cs_count = 5 steps giving displacements < 1 cell
    ul = rng.uniform(-0.4, 0.4, (nz, n, n + 2)) * dx / (2e-4)
    vl = rng.uniform(-0.4, 0.4, (nz, n, n + 2)) * dx / (2e-4)
    wl = rng.uniform(-0.4, 0.4, (nz, n, n + 2)) * dzz / (2e-4)
    o.set("u_lag", ul); o.set("v_lag", vl); o.set("w_lag", wl)
    o.call("interpolag_sdep")
    got = o.get("F_LM")
    # displacement as the reference forms it (u_lag/cs then level average)
    ua = ul / 5.0
    ua[1:] = 0.5 * (ua[1:] + ua[:-1])
    va = vl / 5.0
    va[1:] = 0.5 * (va[1:] + va[:-1])
    xp = -ua * 2e-4 * 5 / dx
    yp = -va * 2e-4 * 5 / dx
    zp = -(wl / 5.0) * 2e-4 * 5 / dzz
    expect = 1.0 + 0.3 * (jx + xp) + 0.2 * (jy + yp) + 0.1 * (jz + zp)
    sl = (slice(2, nz - 2), slice(1, n - 1), slice(1, n - 1))
    assert np.abs(got[sl] - expect[sl]).max() < 1e-12


def _run(O, cfg, surf, steps, seed=5):
    o = O(cfg, surf)
    for k, v in C.initial_state(cfg, surf, seed=seed).items():
        o.set(k, v)
    assert o.step(steps) == 0
    return o


def test_projection_is_divergence_free(O):
    """After press_stag_array + project the start-of-step divergence used by
    rmsdiv (rmsdiv.f90:93-100) is at FP64 roundoff."""
    cfg = C.make_config(16, 16, 16, rmsdiv_every=1)
    o = _run(O, cfg, C.uniform_surface(cfg), 3)
    assert o.rmsdiv() < 1e-12


def test_pressure_zero_mode_closed_form(O):
    """kx = ky = 0 mode by direct integration (press_stag_array.f90:238-247):
    the plane-mean pressure increments by dz * mean(w*)/(1.5 dt)."""
    cfg = C.make_config(16, 16, 8, rmsdiv_every=0)
    d = C.dims(cfg)
    o = O(cfg, C.uniform_surface(cfg))
    rng = np.random.default_rng(6)
    for nm in ["u", "v", "w"]:
        a = np.zeros((cfg.nz, cfg.ny, d["ld"]))
        a[:, :, :16] = rng.standard_normal((cfg.nz, cfg.ny, 16))
        o.set(nm, a)
    o.set("divtz", np.zeros((cfg.nz, cfg.ny, d["ld"])))
    p = np.zeros((cfg.nz + 1, cfg.ny, d["ld"]))
    dpx = np.zeros((cfg.nz, cfg.ny, d["ld"])); dpy = np.zeros_like(dpx)
    assert o.call("press_stag_array", p, dpx, dpy) == 0
    w = o.get("w")
    dz = 1.0 / (cfg.nz - 1)
    pm = p[:, :, :16].mean(axis=(1, 2))
    wm = w[:, :, :16].mean(axis=(1, 2)) / (1.5 * cfg.dt)
    for k in range(2, cfg.nz):
        assert abs((pm[k] - pm[k - 1]) - wm[k - 1] * dz) < 1e-9 * max(1.0, abs(wm[k - 1] * dz))


def _std_dynamic(O, u, v, w, S, nz):
    """Oracle std_dynamic (model 2) on given velocities and S_ij."""
    cfg = C.make_config(16, 16, nz - 1, model=2)
    o = O(cfg)
    o.set("u", u); o.set("v", v); o.set("w", w)
    cs = np.zeros(nz)
    o.call("std_dynamic", cs, *S)
    return cs


def _smooth_state(seed, nz):
    """Band-limited velocities and strain-like fields on a 16 x 16 x nz grid."""
    rng = np.random.default_rng(seed)
    ld, n = 18, 16
    x = np.arange(n) * 2 * np.pi / n
    X, Y = np.meshgrid(x, x)  # (ny, nx)
    out = []
    for q in range(9):
        a = np.zeros((nz, n, ld))
        for k in range(nz):
            f = sum(rng.standard_normal() * np.cos(kx * X + ky * Y + rng.uniform(0, 6.3))
                    for kx in range(0, 6) for ky in range(-5, 6))
            a[k, :, :n] = f / 30.0
        out.append(a)
    return out[:3], out[3:]


def test_std_dynamic_scale_invariance(O):
    """std_dynamic.f90: Cs^2 = <L M>/<M M> with L quadratic in the velocity
    and M quadratic in S_ij, so scaling u, v, w and S_ij by a common factor
    leaves Cs^2 unchanged; Cs^2 >= 0 (the clip of :133)."""
    nz = 6
    (u, v, w), S = _smooth_state(3, nz)
    a = _std_dynamic(O, u, v, w, S, nz)
    b = _std_dynamic(O, 2.5 * u, 2.5 * v, 2.5 * w, [2.5 * s for s in S], nz)
    assert np.all(a >= 0) and np.any(a > 0)
    assert rel(b, a) < 1e-12, (a, b)


def test_std_dynamic_galilean_invariance(O):
    """A uniform velocity passes the spectral test filter unchanged (G_test's
    (0,0) entry is 1/(nx ny)), so L_ij = (u_i u_j)~ - u_i~ u_j~ and Cs^2 do not
    change when a constant is added to u and v."""
    nz = 6
    (u, v, w), S = _smooth_state(4, nz)
    a = _std_dynamic(O, u, v, w, S, nz)
    u2, v2 = u.copy(), v.copy()
    u2[:, :, :16] += 0.7
    v2[:, :, :16] -= 0.3
    b = _std_dynamic(O, u2, v2, w, S, nz)
    assert rel(b, a) < 1e-10, (a, b)


@pytest.mark.parametrize("routine,fields", [("interpolag_ssim", ("F_LM", "F_MM")),
                                            ("interpolag_sdep", ("F_LM", "F_MM", "F_QN", "F_NN")),
                                            ("interpolag_scalar_sdep", ("G_LM", "G_MM", "G_QN", "G_NN"))])
@pytest.mark.parametrize("axis,shift", [(2, 0), (2, 1), (2, -1), (1, 1), (1, -1)])
def test_interpolag_shifts_by_whole_cells(O, routine, fields, axis, shift):
    """interpolag_Ssim.f90 / interpolag_Sdep.f90: a uniform accumulated lag
    velocity of shift * dx / dt (x) or shift * dy / dt (y) gives a
    displacement of exactly -shift cells, so every F_* comes back shifted by
    `shift` cells (periodic) with frac = 0, comp = 1; the lag arrays are
    reset afterwards.  interpolag_scalar_Sdep.f90 moves G_* along u_lag_s,
    v_lag_s, w_lag_s the same way."""
    model = {"interpolag_ssim": 4, "interpolag_sdep": 5, "interpolag_scalar_sdep": 7}[routine]
    sfx = "_s" if model == 7 else ""
    cfg = C.make_config(16, 16, 8, model=model, s_flag=1 if model == 7 else 0)
    d = C.dims(cfg)
    o = O(cfg)
    rng = np.random.default_rng(2)
    shp = (cfg.nz, cfg.ny, d["ld"])
    F = {f: rng.uniform(0.1, 1.0, shp) for f in fields}
    for f, v in F.items():
        o.set(f, v)
    h = 2 * np.pi / cfg.nx  # dx = dy on the 2pi x 2pi box with nx = ny
    lag = np.zeros(shp)
    lag[:, :, :cfg.nx] = shift * h / cfg.dt  # sum over cs_count steps: displacement -lag dt / dx
    o.set("u_lag" + sfx, lag if axis == 2 else np.zeros(shp))
    o.set("v_lag" + sfx, lag if axis == 1 else np.zeros(shp))
    o.set("w_lag" + sfx, np.zeros(shp))
    o.call(routine)
    n = cfg.nx
    for f, v in F.items():
        want = np.roll(v[:, :, :n], shift, axis=axis)
        assert np.allclose(o.get(f)[:, :, :n], want, rtol=0, atol=1e-15), f
    assert not o.get("u_lag" + sfx).any() and not o.get("v_lag" + sfx).any()


# ---- SGS model 7: the scalars' Lagrangian dynamic Prandtl number -----------

def _m7(O, jt0=500, model=7, seed=9, **kw):
    cfg = C.make_config(16, 16, 8, s_flag=1, model=model, jt_total0=jt0, **kw)
    surf = C.striped_surface(cfg)
    o = O(cfg, surf)
    for k, v in C.initial_state(cfg, surf, seed=seed, theta_levels=cfg.nz).items():
        o.set(k, v)
    return cfg, surf, o


def test_model7_below_500_is_model5(O):
    """sgs_stag.f90:166-173: while jt_total < 500 model 7 holds Cs_opt2 at
    0.16^2 and Pr_t at Pr, so its run is model 5's; the only trace of
    lagrange_scalar_Sdep is its in-place Nyquist filter of theta (filt_da,
    lagrange_scalar_Sdep.f90:83), which changes theta by rounding only."""
    _, _, a = _m7(O, jt0=0, model=5)
    cfg, _, b = _m7(O, jt0=0)
    assert a.step(10) == 0 and b.step(10) == 0
    n = cfg.nx
    for nm in ("u", "v", "w", "theta"):
        assert rel(b.get(nm)[:-1, :, :n], a.get(nm)[:-1, :, :n]) < 1e-13, nm
    assert np.all(b.get("Pr_t") == cfg.pr)
    # the scalar averages were updated at jt = 5 and 10 all the same
    assert np.abs(b.get("G_MM")[:-1, :, :n]).min() > 0.0


def test_lagrange_scalar_scale_covariance(O):
    """theta -> 2 theta with the surface heat flux and the lid gradient
    doubled: every filtered product and gradient doubles exactly (powers of
    two scale IEEE arithmetic exactly), L_i and M_i double, L.M and M.M
    quadruple, so with G_* quadrupled the relaxed G_* quadruple bit for bit
    and Cs2_Pr and Pr_t are unchanged wherever the 1e-24 floor on G_LM,
    G_QN (lagrange_scalar_Sdep.f90:331, :359) does not bind."""
    cfg, surf, a = _m7(O, dtdz_top=0.003)
    assert a.step(7) == 0  # past the update at jt = 5; lag sums of two steps
    cfg2 = C.make_config(16, 16, 8, s_flag=1, model=7, jt_total0=500, dtdz_top=0.006)
    b = O(cfg2, surf)
    names = ["u", "v", "w", "theta", "G_LM", "G_MM", "G_QN", "G_NN", "u_lag_s", "v_lag_s", "w_lag_s",
             "TnLMMM", "TnQNNN", "Cs_opt2", "psi_m", "phi_h", "wt_s", "S11", "S12", "S13", "S22", "S23", "S33"]
    scale = {"theta": 2.0, "wt_s": 2.0, "G_LM": 4.0, "G_MM": 4.0, "G_QN": 4.0, "G_NN": 4.0}
    for nm in names:
        b.set(nm, scale.get(nm, 1.0) * a.get(nm))
    shp = C.field_shape(cfg, "u")
    ca, cb = np.zeros(shp), np.zeros(shp)
    a.call("lagrange_scalar_sdep", ca)
    b.call("lagrange_scalar_sdep", cb)
    n = cfg.nx
    free = (a.get("G_LM") > 1e-23) & (a.get("G_QN") > 1e-23)
    free[:, :, n:] = False
    assert free.sum() > 0.2 * free[:, :, :n].size
    for nm in ("G_LM", "G_MM", "G_QN", "G_NN"):
        assert np.array_equal(b.get(nm)[free], 4.0 * a.get(nm)[free]), nm
    assert np.array_equal(cb[free], ca[free])
    assert np.array_equal(b.get("Pr_t")[free], a.get("Pr_t")[free])
    assert np.array_equal(b.get("theta")[:, :, :n], 2.0 * a.get("theta")[:, :, :n])
    # Pr_t = Cs_opt2 / Cs2_Pr everywhere, the padding columns at 1
    pr = a.get("Pr_t")
    assert np.array_equal(pr[:, :, :n], a.get("Cs_opt2")[:, :, :n] / ca[:, :, :n])
    assert np.all(pr[:, :, n:] == 1.0)


def test_model7_step_is_finite_and_diffuses_with_pr_t(O):
    """From jt_total = 500 model 7 runs its scalar SGS fluxes with the
    dynamic Pr_t (scalars_module.f90:77-82): the state stays finite and the
    scalar differs from model 5's, the velocities only through buoyancy."""
    _, _, a = _m7(O, model=5)
    cfg, _, b = _m7(O)
    assert a.step(10) == 0 and b.step(10) == 0
    n = cfg.nx
    for nm in ("u", "v", "w", "theta", "Pr_t", "G_LM", "G_MM"):
        assert np.all(np.isfinite(b.get(nm)[:-1, :, :n])), nm
    assert rel(b.get("theta")[:-1, :, :n], a.get("theta")[:-1, :, :n]) > 1e-9
    assert not np.all(b.get("Pr_t") == cfg.pr)


# ---- humidity (scalars_module_q.f90, atm_thermodynamics.f90) ----------------

def _q_pair(O, n=16, levels=8, **kw):
    cfg = C.make_config(n, n, levels, s_flag=1, **kw)
    surf = C.striped_surface(cfg)
    o = O(cfg, surf)
    for k, v in C.initial_state(cfg, surf, seed=5).items():
        o.set(k, v)
    return cfg, o


def test_zero_humidity_leaves_the_step_unchanged(O):
    """qmix = 0, wq_s = 0 and dqdz_top = 0: theta (1 + 0.61 0.001 qmix q_scale)
    is theta and the moisture buoyancy flux is zero, so a q_flag = 1 run
    gives the q_flag = 0 run's state bit for bit and qmix stays zero."""
    cfg0, a = _q_pair(O)
    cfg1, b = _q_pair(O, q_flag=1, dqdz_top=0.0)
    b.set("q", np.zeros(C.field_shape(cfg1, "q")))
    b.set("wq_s", np.zeros((cfg1.ny, cfg1.nx)))
    assert a.step(4) == 0 and b.step(4) == 0
    for nm in ("u", "v", "w", "theta", "p", "Cs_opt2"):
        assert np.array_equal(a.get(nm), b.get(nm)), nm
    assert not b.get("q").any()


def test_surface_moisture_flux_first_step(O):
    """Uniform wind, uniform qmix = 0.1, uniform surface moisture flux wq_s:
    nothing advects or diffuses qmix in the first (Euler) step, whose
    right-hand side is the surface flux divergence surf_flux / dz at level 1
    (scalars_module_q.f90:174-178, 298-347, surf_flux = wq_s / q_scale / u_star)
    and zero above (dqdz_top = 0)."""
    n, lev = 16, 8
    cfg = C.make_config(n, n, lev, s_flag=1, q_flag=1, dqdz_top=0.0)
    surf = C.uniform_surface(cfg, 1e-4, 0.0)
    o = O(cfg, surf)
    shp = C.field_shape(cfg, "u")
    u = np.zeros(shp)
    u[:, :, :n] = 5.0
    th = np.zeros(shp)
    th[:, :, :n] = 300.0 / cfg.t_scale
    q = np.zeros(shp)
    q[:, :, :n] = 0.1
    for nm, v in (("u", u), ("theta", th), ("q", q)):
        o.set(nm, v)
    wq = 0.05
    o.set("wq_s", np.full((n, n), wq))
    assert o.step(1) == 0
    dz = cfg.lz_over_zi / (cfg.nz - 1)
    inc = cfg.dt * (wq / cfg.q_scale / cfg.u_star) / dz
    got = o.get("q")
    assert np.allclose(got[0, :, :n], 0.1 + inc, rtol=0, atol=1e-13)
    assert np.allclose(got[1:cfg.nz - 1, :, :n], 0.1, rtol=0, atol=1e-13)
    assert np.allclose(o.get("sgs_q3"), wq / cfg.q_scale / cfg.u_star, rtol=1e-15)


def test_humid_step_moistens_and_stays_finite(O):
    """Striped surface with a striped moisture flux: 6 steps of the coupled
    theta / qmix step stay finite, the first level moistens, and qmix enters
    the buoyancy (beta_scal differs from the dry run's)."""
    cfg, o = _q_pair(O, q_flag=1)
    o.set("wq_s", C.moisture_flux(cfg))
    q0 = o.get("q")[0, :, :cfg.nx].mean()
    _, dry = _q_pair(O)
    assert o.step(6) == 0 and dry.step(6) == 0
    q = o.get("q")
    assert np.isfinite(q).all()
    assert q[0, :, :cfg.nx].mean() > q0
    assert not np.array_equal(o.get("beta_scal"), dry.get("beta_scal"))


def test_thermo_restatement(O):
    """The oracle's thermo against a numpy writing of
    atm_thermodynamics.f90:37-52 on a seeded theta / qmix state."""
    cfg, o = _q_pair(O, q_flag=1)
    shp = C.field_shape(cfg, "u")
    out = [np.zeros(shp) for _ in range(9)]
    o.call("atm_thermodynamics", *out)
    th, q = o.get("theta"), o.get("q")
    n, nz = cfg.nx, cfg.nz
    dz = cfg.lz_over_zi / (nz - 1)
    cp, Rd, prs, g = 1005.0, 287.04, 100000.0, cfg.g
    k = np.arange(1, nz)[:, None, None]
    zg = k * dz * cfg.z_i
    T = th[:nz - 1, :, :n] - (g / cp) * zg / cfg.t_scale
    qq = 0.001 * cfg.q_scale * q[:nz - 1, :, :n]
    Tv = T * (1 + 0.61 * qq)
    es = 611.2 * np.exp(17.62 * (T * cfg.t_scale - 273.2) / (243.12 + (T * cfg.t_scale - 273.2)))
    p = prs * np.exp(-zg / (Rd * Tv * cfg.t_scale / g))
    e = qq / (qq + 0.622) * p
    qs = 0.622 * es / (p - es)
    rq = qq / qs
    zl = zg + (cp / g) * (T * cfg.t_scale - 55 - 1.0 / (1 / (T * cfg.t_scale - 55) - np.log(rq) / 2840))
    for a, b in zip(out, (T, Tv, es, p, e, qs, e / es, rq, zl)):
        assert rel(a[:nz - 1, :, :n], b) < 1e-13
        assert not a[nz - 1].any() and not a[:, :, n:].any()
    assert 0.0 < rq.min() and rq.max() < 1.5


# ---- running statistics (io.f90:403-1218 MM_XYZ_Out) ------------------------

def test_running_statistics_bookkeeping(O):
    """A fixed state accumulated three times gives 3 fr x (the w-node value):
    u at level 1, (u(k) + u(k-1))/2 above, 0.25 w(2) at level 1; groups 1 and 2
    are zeroed separately and atxy by neither (io.f90:457-502, 997-1006,
    1189-1216); with jt_total <= c_count every accumulation starts from zero."""
    cfg, o = _q_pair(O, q_flag=1, jt_total0=100)
    assert o.step(1) == 0  # nonzero stresses and gradients
    o.stats_enable(2, 10)
    fr = 2 / 10
    for _ in range(3):
        o.stats_accumulate()
    n = cfg.nx
    u, w, txy = o.get("u")[:, :, :n], o.get("w")[:, :, :n], o.get("txy")[:, :, :n]
    au = o.stats_get("au")
    assert np.allclose(au[0], 3 * fr * u[0], rtol=1e-14, atol=0)
    assert np.allclose(au[1:], 3 * fr * (u[1:cfg.nz - 1] + u[:cfg.nz - 2]) / 2, rtol=1e-14, atol=0)
    assert np.allclose(o.stats_get("aw")[0], 3 * fr * 0.25 * w[1], rtol=1e-14, atol=1e-300)
    assert np.allclose(o.stats_get("u2")[0], 3 * fr * u[0] ** 2, rtol=1e-14, atol=0)
    assert np.allclose(o.stats_get("atxy"), 3 * fr * txy[:cfg.nz - 1], rtol=1e-14, atol=1e-300)
    o.stats_reset(1)
    assert not o.stats_get("au").any() and o.stats_get("ap").any() and o.stats_get("atxy").any()
    o.stats_reset(2)
    assert not o.stats_get("ap").any() and not o.stats_get("aactual_T").any() and o.stats_get("atxy").any()
    # a run whose jt_total <= c_count starts every accumulation from zero
    cfg2, o2 = _q_pair(O, q_flag=1)
    o2.stats_enable(2, 10)
    o2.stats_accumulate()
    o2.stats_accumulate()
    assert np.allclose(o2.stats_get("au")[0], fr * o2.get("u")[0, :, :n], rtol=1e-14, atol=0)
    # thermodynamic statistics follow thermo (T_scale-scaled temperatures)
    out = [np.zeros(C.field_shape(cfg, "u")) for _ in range(9)]
    o.call("atm_thermodynamics", *out)
    o.stats_enable(2, 10)
    o.stats_accumulate()
    assert np.allclose(o.stats_get("aactual_T"), fr * out[0][:cfg.nz - 1, :, :n] * cfg.t_scale, rtol=1e-14)
    assert np.allclose(o.stats_get("azlcl_all"), fr * out[8][:cfg.nz - 1, :, :n], rtol=1e-14)
