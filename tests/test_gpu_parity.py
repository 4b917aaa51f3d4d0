"""GPU (sm_103a library, through the C ABI) vs the CPU oracle on identical
seeded inputs.  FP64 form: relative error <= 1e-12 on u, v, w, theta, Cs^2
and rmsdiv (the FP64 parity tolerance of the step); routine-level checks at
rounding level.
"""
import numpy as np
import pytest

import les_gb300 as lg

pytestmark = pytest.mark.gpu

TOL = 1e-12


def rel(a, b):
    nb = np.linalg.norm(b)
    return np.linalg.norm(a - b) / (nb if nb > 0 else 1.0)


def interior(cfg, a, lev=slice(0, -1)):
    return a[lev, :, :cfg.nx]


def pair(cfg, surf, seed=11):
    from oracle.oracle import Oracle
    st = lg.initial_state(cfg, surf, seed=seed)
    g = lg.Context(cfg, surf)
    o = Oracle(cfg, surf)
    for k, v in st.items():
        g.set(k, v)
        o.set(k, v)
    return g, o


@pytest.fixture(scope="module")
def libs(gpu_lib, oracle_lib):
    return gpu_lib, oracle_lib


@pytest.mark.parametrize("n", [32, 48])
def test_fft_roundtrip_and_spectra(libs, n):
    from oracle.oracle import Oracle
    cfg = lg.make_config(n, n, 4)
    d = lg.dims(cfg)
    g = lg.Context(cfg)
    o = Oracle(cfg)
    rng = np.random.default_rng(3)
    for big, nn, ld in [(0, n, d["ld"]), (1, 3 * n // 2, d["ld_big"])]:
        x = rng.standard_normal((3, nn, ld))
        a = x.copy(); b = x.copy()
        g.call("fft_r2c", a, ints=(3, big))
        o.call("fft_r2c", b, ints=(3, big))
        assert rel(a, b) < 1e-14
        g.call("fft_c2r", a, ints=(3, big))
        o.call("fft_c2r", b, ints=(3, big))
        assert rel(a[:, :, :nn], b[:, :, :nn]) < 1e-14
        assert rel(a[:, :, :nn] / (nn * nn), x[:, :, :nn]) < 1e-14


def test_derivatives_filters_dealias(libs):
    from oracle.oracle import Oracle
    cfg = lg.make_config(32, 32, 16)
    d = lg.dims(cfg)
    g = lg.Context(cfg)
    o = Oracle(cfg)
    rng = np.random.default_rng(5)
    nz = cfg.nz
    f = rng.standard_normal((nz, cfg.ny, d["ld"]))
    for name in ["ddx", "ddy"]:
        a = np.zeros_like(f); b = np.zeros_like(f)
        g.call(name, a, f, ints=(nz,))
        o.call(name, b, f, ints=(nz,))
        assert rel(a[:, :, :32], b[:, :, :32]) < 1e-13, name
    fa, fb = f.copy(), f.copy()
    ax, ay = np.zeros_like(f), np.zeros_like(f)
    bx, by = np.zeros_like(f), np.zeros_like(f)
    g.call("filt_da", fa, ax, ay, ints=(nz,))
    o.call("filt_da", fb, bx, by, ints=(nz,))
    for p, q in [(fa, fb), (ax, bx), (ay, by)]:
        assert rel(p[:, :, :32], q[:, :, :32]) < 1e-13
    big_a = np.zeros((nz, d["ny2"], d["ld_big"]))
    big_b = np.zeros_like(big_a)
    g.call("dealias1", f, big_a, ints=(nz,))
    o.call("dealias1", f.copy(), big_b, ints=(nz,))
    assert rel(big_a[:, :, :d["nx2"]], big_b[:, :, :d["nx2"]]) < 1e-13
    sa, sb = np.zeros_like(f), np.zeros_like(f)
    g.call("dealias2", sa, big_a.copy(), ints=(nz,))
    o.call("dealias2", sb, big_b.copy(), ints=(nz,))
    assert rel(sa[:, :, :32], sb[:, :, :32]) < 1e-13


def test_tridag_array(libs):
    from oracle.oracle import Oracle
    cfg = lg.make_config(16, 16, 12)
    d = lg.dims(cfg)
    g = lg.Context(cfg)
    o = Oracle(cfg)
    rng = np.random.default_rng(9)
    n = cfg.nz + 1
    shp = (n, cfg.ny, d["lh"])
    a = rng.uniform(0.5, 1.0, shp); c = rng.uniform(0.5, 1.0, shp)
    b = -(a + c + rng.uniform(0.1, 1.0, shp))
    r = rng.standard_normal(shp + (2,))
    ug = np.zeros_like(r); uo = np.zeros_like(r)
    g.call("tridag_array", a, b, c, r, ug)
    o.call("tridag_array", a, b, c, r, uo)
    assert rel(ug, uo) < 1e-13


def _fp32_flips(a, b):
    """Points where Cs^2 differs by more than rounding: the reference truncates
    Cs^2 and F_LM/F_QN to FP32 (lagrange_Sdep.f90:321-421), so a 1-ulp FP64
    difference upstream can flip one FP32 rounding (about 6e-8 relative)."""
    d = np.abs(a - b) / np.maximum(np.abs(b), 1e-300)
    return int(np.count_nonzero(d > 1e-12)), float(d.max())


@pytest.mark.parametrize("s_flag,jt0", [(0, 0), (1, 0), (1, 500)])
def test_step_parity_32(libs, s_flag, jt0):
    """32^3 FP64, 10 steps (Euler first step, AB2 after), Lagrangian
    scale-dependent SGS; jt_total0 = 500 switches the Cs^2 override off
    (sgs_stag.f90:166-173) so the dynamic Cs^2 feeds back from step 5."""
    cfg = lg.make_config(32, s_flag=s_flag, jt_total0=jt0, model=5, rmsdiv_every=1)
    surf = lg.striped_surface(cfg) if s_flag else lg.uniform_surface(cfg)
    g, o = pair(cfg, surf)
    g.step(1)
    assert o.step(1) == 0
    # first-step rmsdiv is the divergence of the seeded initial state (order 1)
    rg, ro = g.rmsdiv(), o.rmsdiv()
    assert abs(rg - ro) <= TOL * abs(ro), (rg, ro)
    for it in range(9):
        g.step(1)
        assert o.step(1) == 0
    names = ["u", "v", "theta"] if s_flag else ["u", "v"]
    for nm in names:
        e = rel(interior(cfg, g.get(nm)), interior(cfg, o.get(nm)))
        assert e < TOL, (nm, e)
    e = rel(interior(cfg, g.get("w"), slice(None)), interior(cfg, o.get("w"), slice(None)))
    assert e < TOL, ("w", e)
    cg, co = interior(cfg, g.get("Cs_opt2")), interior(cfg, o.get("Cs_opt2"))
    nflip, dmax = _fp32_flips(cg, co)
    assert nflip <= max(2, cg.size // 10000) and dmax < 1e-6, (nflip, dmax)
    # after the projection rmsdiv is FP64 roundoff: both at rounding level
    rg, ro = g.rmsdiv(), o.rmsdiv()
    assert rg < 1e-12 and ro < 1e-12 and abs(rg - ro) < 1e-13, (rg, ro)


# The oracle's own rounding sensitivity for model 3 (32^3, theta, striped
# surface, jt_total0 = 500, 10 steps): the oracle built with FMA contraction
# (-ffp-contract=fast) against the oracle without it (-ffp-contract=off)
# differs by u 1.7e-9, v 1.7e-7, w 9.8e-8 (relative L2), Cs^2 5.1e-2 and
# rmsdiv 1.6 %.  The GPU is held to three times that measured spread.
M3_SPREAD = {"u": 1.7e-9, "v": 1.7e-7, "w": 9.8e-8, "theta": 4.2e-16, "Cs_opt2": 5.1e-2, "rmsdiv": 1.6e-2}


def test_step_parity_32_plane_scaledep(libs):
    """model = 3 (scaledep_dynamic): the plane-averaged quintic for beta
    (sgsmodule.f90:37-59 rtnewt) is ill-conditioned in the reference
    algorithm itself, so the GPU (plane sums in a fixed tree order, FMA
    contraction) is held to three times the oracle's own FMA / no-FMA spread
    (M3_SPREAD) per field, Cs^2 and rmsdiv included."""
    cfg = lg.make_config(32, s_flag=1, jt_total0=500, model=3, rmsdiv_every=1)
    surf = lg.striped_surface(cfg)
    g, o = pair(cfg, surf)
    g.step(10)
    assert o.step(10) == 0
    errs = {}
    for nm in ["u", "v", "theta"]:
        errs[nm] = rel(interior(cfg, g.get(nm)), interior(cfg, o.get(nm)))
    errs["w"] = rel(interior(cfg, g.get("w"), slice(None)), interior(cfg, o.get("w"), slice(None)))
    errs["Cs_opt2"] = rel(interior(cfg, g.get("Cs_opt2"), slice(None)), interior(cfg, o.get("Cs_opt2"), slice(None)))
    rg, ro = g.rmsdiv(), o.rmsdiv()
    errs["rmsdiv"] = abs(rg - ro) / ro
    print("model 3 GPU vs oracle", errs)
    for nm, e in errs.items():
        bound = 3.0 * M3_SPREAD[nm]
        if nm == "theta":
            bound = TOL
        assert e < bound, (nm, e, bound)


def test_std_dynamic_routine(libs):
    """std_dynamic.f90:1-136 (model 2) on the same u, v, w and S_ij: the
    per-level Cs^2 of the GPU (plane sums in a fixed tree order) against the
    oracle (sequential sums)."""
    cfg = lg.make_config(32, 32, 20, model=2, s_flag=0)
    surf = lg.uniform_surface(cfg)
    g, o = pair(cfg, surf, seed=5)
    rng = np.random.default_rng(6)
    shp = lg.field_shape(cfg, "u")
    S = []
    for q in range(6):  # smooth strain-like fields (a few low modes per level)
        a = np.zeros(shp)
        x = np.arange(cfg.nx) * 2 * np.pi / cfg.nx
        X, Y = np.meshgrid(x, x)
        for k in range(shp[0]):
            a[k, :, :cfg.nx] = sum(rng.standard_normal() * np.cos(i * X + j * Y + rng.uniform(0, 6.3))
                                   for i in range(4) for j in range(-3, 4)) / 10.0
        S.append(a)
    cg, co = np.zeros(cfg.nz), np.zeros(cfg.nz)
    g.call("std_dynamic", cg, *S)
    o.call("std_dynamic", co, *S)
    assert np.all(co >= 0) and np.any(co > 0)
    assert rel(cg, co) < TOL, (cg, co)


def test_step_parity_32_std_dynamic(libs):
    """model = 2 (standard dynamic, plane-averaged Cs^2 from the 2 delta test
    filter, std_dynamic.f90): 10 steps with active theta; the dynamic Cs^2 is
    computed at steps 5 and 10 and feeds back.  Velocities and theta are held
    to 1e-12.  Cs^2(z) is a ratio of plane sums whose numerator cancels: the
    oracle built with and without FMA contraction differs by up to 2.8e-11
    per level after these 10 steps (u, v, w by 6e-14 at most), so Cs^2 is
    held to that rounding sensitivity (1e-9), not 1e-12."""
    cfg = lg.make_config(32, s_flag=1, jt_total0=500, model=2, rmsdiv_every=1)
    surf = lg.striped_surface(cfg)
    g, o = pair(cfg, surf)
    g.step(10)
    assert o.step(10) == 0
    for nm in ["u", "v", "theta"]:
        e = rel(interior(cfg, g.get(nm)), interior(cfg, o.get(nm)))
        assert e < TOL, (nm, e)
    e = rel(interior(cfg, g.get("w"), slice(None)), interior(cfg, o.get("w"), slice(None)))
    assert e < TOL, ("w", e)
    cg, co = interior(cfg, g.get("Cs_opt2"), slice(None)), interior(cfg, o.get("Cs_opt2"), slice(None))
    assert np.any(co > 0) and rel(cg, co) < 1e-9, rel(cg, co)


def test_interpolag_ssim_routine(libs):
    """interpolag_Ssim.f90:3-316 on the same F_LM, F_MM and lag velocities,
    with near-wall vertical displacements beyond one cell (interpolag_Sdep
    would clip them; interpolag_Ssim does not)."""
    cfg = lg.make_config(32, 32, 12, model=4)
    surf = lg.uniform_surface(cfg)
    g, o = pair(cfg, surf, seed=8)
    rng = np.random.default_rng(8)
    shp = lg.field_shape(cfg, "u")
    f = {"F_LM": rng.uniform(0.1, 1.0, shp), "F_MM": rng.uniform(0.1, 1.0, shp),
         "u_lag": rng.uniform(-2.0, 2.0, shp), "v_lag": rng.uniform(-2.0, 2.0, shp),
         "w_lag": rng.uniform(-2.0, 2.0, shp)}
    f["w_lag"][1] *= 4000.0  # level 2: |displacement| above 1 near the wall
    for k, v in f.items():
        g.set(k, v)
        o.set(k, v)
    g.call("interpolag_ssim")
    o.call("interpolag_ssim")
    for k in ("F_LM", "F_MM"):
        e = rel(interior(cfg, g.get(k), slice(None)), interior(cfg, o.get(k), slice(None)))
        assert e < 1e-14, (k, e)


def test_step_parity_32_lagrange_ssim(libs):
    """model = 4 (Lagrangian scale-invariant, lagrange_Ssim.f90): 10 steps
    with active theta; F_LM, F_MM are relaxed along trajectories at steps 5
    and 10 and Cs^2 = F_LM / F_MM feeds back."""
    cfg = lg.make_config(32, s_flag=1, jt_total0=500, model=4, rmsdiv_every=1)
    surf = lg.striped_surface(cfg)
    g, o = pair(cfg, surf)
    g.step(10)
    assert o.step(10) == 0
    for nm in ["u", "v", "theta"]:
        e = rel(interior(cfg, g.get(nm)), interior(cfg, o.get(nm)))
        assert e < TOL, (nm, e)
    e = rel(interior(cfg, g.get("w"), slice(None)), interior(cfg, o.get("w"), slice(None)))
    assert e < TOL, ("w", e)
    for nm in ["Cs_opt2", "F_LM", "F_MM"]:
        a, b = interior(cfg, g.get(nm), slice(None)), interior(cfg, o.get(nm), slice(None))
        assert np.any(b > 1e-20) and rel(a, b) < 1e-10, (nm, rel(a, b))
    assert np.all(g.get("Beta") == 1.0)


C2_SEED = 21
# The oracle's own rounding sensitivity on the 128^3 workload (theta, striped
# surface, jt_total from 0), from `python -m oracle.rounding_spread c2`: the
# oracle built with FMA contraction against the oracle without it.  The
# builds agree to 5e-13 up to step 50; from about step 55 the first level's
# explicit SGS diffusion (Nu_t dt / dz^2 above the AB2 limit there) grows
# every rounding difference until it saturates, and at step 200 they differ
# by these relative L2 amounts (and the plane-mean u, theta profiles by
# 5.4e-7, 2.1e-9 of max |mean|).
C2_SPREAD_200 = {"u": 3.5e-5, "v": 4.5e-3, "w": 6.0e-3, "theta": 8.2e-8}
C2_MEAN_SPREAD_200 = {"u": 5.4e-7, "theta": 2.1e-9}


def _c2_pair():
    from oracle.oracle import Oracle
    cfg = lg.make_config(128, s_flag=1, rmsdiv_every=10)
    surf = lg.striped_surface(cfg)
    g, o = pair(cfg, surf, seed=C2_SEED)
    Oracle.set_threads(max(1, Oracle.max_threads()))
    return cfg, g, o


def test_step_parity_128_theta(libs):
    """128^3 FP64, active theta, x-striped z0 (1e-4 / 1e-2) and surface heat
    flux (0.05 / 0.15 K m/s), dt = 2e-4, from the reference's spin-up
    (jt_total from 0: Cs^2 = 0.16^2 while the Lagrangian averages F_LM..F_NN
    build up every cs_count steps), rmsdiv and the CFL check every 10 steps
    (main.f90:451-458).  First 50 steps, before the first-level
    amplification of rounding differences sets in (see C2_SPREAD_200):
    u, v, w, theta to 1e-12; the Lagrangian averages F_LM..F_NN, which the
    reference rounds through FP32 (lagrange_Sdep.f90:321-421), to 1e-6;
    rmsdiv at FP64 roundoff in both.  Then on to 200 steps: every field
    within twice the oracle's own FMA / no-FMA spread at step 200."""
    cfg, g, o = _c2_pair()
    g.step(50)
    assert o.step(50) == 0
    assert g.counters() == o.counters() == (50, 50)
    for nm in ["u", "v", "theta"]:
        e = rel(interior(cfg, g.get(nm)), interior(cfg, o.get(nm)))
        assert e < TOL, (nm, e)
    e = rel(interior(cfg, g.get("w"), slice(None)), interior(cfg, o.get("w"), slice(None)))
    assert e < TOL, ("w", e)
    cg, co = interior(cfg, g.get("Cs_opt2"), slice(None)), interior(cfg, o.get("Cs_opt2"), slice(None))
    assert np.array_equal(cg, co)  # the spin-up value 0.16**2 (in FP32) everywhere
    # F_LM and F_QN are rounded through FP32 at every update; a 1-ulp FP64
    # difference upstream flips a rounding, and the flip is then carried along
    # the trajectories by ten interpolated updates, so these are held to a
    # few FP32 roundings of their norm
    for nm in ["F_LM", "F_QN", "F_MM", "F_NN"]:
        a, b = interior(cfg, g.get(nm), slice(None)), interior(cfg, o.get(nm), slice(None))
        assert rel(a, b) < 1e-6, (nm, rel(a, b))
    rg, ro = g.rmsdiv(), o.rmsdiv()
    assert rg < 1e-12 and ro < 1e-12 and abs(rg - ro) < 1e-13, (rg, ro)
    # steps 51..200
    g.step(150)
    assert o.step(150) == 0
    for nm in ["u", "v", "w", "theta"]:
        lev = slice(None) if nm == "w" else slice(0, -1)
        a, b = interior(cfg, g.get(nm), lev), interior(cfg, o.get(nm), lev)
        e = rel(a, b)
        assert e < 2.0 * C2_SPREAD_200[nm], (nm, e)
        if nm in C2_MEAN_SPREAD_200:
            ma, mb = a.mean(axis=(1, 2)), b.mean(axis=(1, 2))
            em = np.abs(ma - mb).max() / np.abs(mb).max()
            # one realisation of the amplified difference: an order of magnitude
            assert em < 10.0 * C2_MEAN_SPREAD_200[nm], (nm, "mean profile", em)
    rg, ro = g.rmsdiv(), o.rmsdiv()
    assert rg < 1e-12 and ro < 1e-12 and abs(rg - ro) < 1e-13, (rg, ro)
