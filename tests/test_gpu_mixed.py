"""FP32-mixed form vs the FP64 form on the GPU (same seeded inputs).

The mixed form runs the scalar, convective, stress-divergence and SGS
transforms in FP32 with FP32 3/2-grid and filter temporaries; the convective
term is split about the plane-mean wind, whose linear terms come from
float-float transforms; u, v, w, theta, the AB2 update, filt_da of the
velocity, the pressure solve and the plane (wall-stress, mean-profile)
quantities stay FP64 or float-float.  Bound: relative L2 error <= 1e-5 on
each of u, v, w and theta separately (v and w are two orders of magnitude
smaller than u, so a combined velocity norm would hide their error), and
rmsdiv <= 1e-10."""
import ctypes

import numpy as np
import pytest

import les_gb300 as lg

pytestmark = pytest.mark.gpu


def rel(a, b):
    return np.linalg.norm(a - b) / np.linalg.norm(b)


def run(n, steps, prec, seed=3, levels=None, rmsdiv_every=10):
    cfg = lg.make_config(n, nz_levels=levels, s_flag=1, jt_total0=500, precision=prec,
                         rmsdiv_every=rmsdiv_every)
    surf = lg.striped_surface(cfg)
    ctx = lg.Context(cfg, surf)
    for k, v in lg.initial_state(cfg, surf, seed=seed).items():
        ctx.set(k, v)
    ctx.step(steps)
    out = {nm: ctx.get(nm)[:-1, :, :n] for nm in ["u", "v", "w", "theta", "Cs_opt2"]}
    out["Nu_t"] = ctx.get("Nu_t")[:-1, :, :n]  # FP32-held in the mixed form, read back widened
    out["rmsdiv"] = ctx.rmsdiv()
    ctx.close()
    return out


@pytest.mark.parametrize("n,steps", [(32, 20), (64, 50)])
def test_mixed_vs_fp64(gpu_lib, n, steps):
    a, b = run(n, steps, 1), run(n, steps, 0)
    vel_a = np.concatenate([a[k].ravel() for k in ("u", "v", "w")])
    vel_b = np.concatenate([b[k].ravel() for k in ("u", "v", "w")])
    errs = {k: rel(a[k], b[k]) for k in ("u", "v", "w", "theta", "Cs_opt2")}
    th_a = a["theta"] - a["theta"].mean(axis=(1, 2), keepdims=True)
    th_b = b["theta"] - b["theta"].mean(axis=(1, 2), keepdims=True)
    errs["theta_fluct"] = rel(th_a, th_b)
    errs["velocity"] = rel(vel_a, vel_b)
    print("mixed vs fp64", n, steps, errs, "rmsdiv", a["rmsdiv"], b["rmsdiv"])
    for nm in ("u", "v", "w", "theta"):
        assert errs[nm] <= 1e-5, (nm, errs)
    assert a["rmsdiv"] <= 1e-10, a["rmsdiv"]


@pytest.mark.parametrize("n", [256, 128])
def test_mixed_vs_fp64_256_lengths(gpu_lib, n):
    """n x n x 32 for n = 256 and 128, 40 steps: the register-resident FP32
    transforms of the 256^3 workload (y pass 256 = 16 x 16, x passes of half
    lengths 128 and 192, the 3/2 padding and truncation y passes 256 <-> 384
    = 16 x 24) and of the 128^3 ensemble members (padding 128 <-> 192 =
    16 x 12), the float-float mean-wind terms and pressure transforms, the
    chunked float-float tridiagonal solve, and eight Lagrangian updates of the
    dynamic Cs^2 (steps 5, 10, .., 40; jt_total0 = 500, so Cs^2 feeds back),
    with the Lagrangian filters restricted to the nonzero kx columns, against
    the FP64 form, field by field."""
    # the seeded 256-wide state runs at CFL 0.109, above the in-step check's
    # 0.1, so the in-step diagnostic is off; rmsdiv is read after the steps
    a, b = run(n, 40, 1, levels=32, rmsdiv_every=0), run(n, 40, 0, levels=32, rmsdiv_every=0)
    errs = {nm: rel(a[nm], b[nm]) for nm in ("u", "v", "w", "theta")}
    ecs = rel(a["Cs_opt2"], b["Cs_opt2"])
    enu = rel(a["Nu_t"], b["Nu_t"])
    print("mixed vs fp64 %dx%dx32" % (n, n), errs, ecs, enu, "rmsdiv", a["rmsdiv"], b["rmsdiv"])
    for nm, e in errs.items():
        assert e <= 1e-5, (nm, errs)
    assert ecs <= 1e-3, ecs  # dynamic coefficient from FP32 filters (the reference truncates it to FP32)
    assert enu <= 1e-3, enu  # FP32-held eddy viscosity, read back widened
    assert a["rmsdiv"] <= 1e-10, a["rmsdiv"]


def test_mixed_context_refuses_fp64_module_routines(gpu_lib):
    """The per-routine entries that read S_ij, Nu_t or tau_ij in FP64 need a
    precision-0 context; on a mixed context they return LES_ERR_ARG."""
    cfg = lg.make_config(32, s_flag=1, precision=1)
    surf = lg.striped_surface(cfg)
    ctx = lg.Context(cfg, surf)
    L = lg.lib()
    for name in ("les_sgs_stag", "les_wallstress", "les_theta_all_in_one"):
        f = getattr(L, name)
        f.restype = ctypes.c_int
        f.argtypes = [ctypes.c_void_p]
        assert f(ctx.h) == -1, name
    ctx.close()
