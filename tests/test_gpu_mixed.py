"""FP32-mixed form vs the FP64 form on the GPU (same seeded inputs).

The mixed form runs the scalar, convective, stress-divergence and SGS
transforms in FP32 with FP32 3/2-grid and filter temporaries; u, v, w, theta,
the AB2 update, filt_da of the velocity, the pressure solve and the plane
(wall-stress, mean-profile) quantities stay FP64.  Targets: relative error
<= 1e-5 on the velocity field, rmsdiv <= 1e-10."""
import numpy as np
import pytest

import les_gb300 as lg

pytestmark = pytest.mark.gpu


def rel(a, b):
    return np.linalg.norm(a - b) / np.linalg.norm(b)


def run(n, steps, prec, seed=3):
    cfg = lg.make_config(n, s_flag=1, jt_total0=500, precision=prec, rmsdiv_every=10)
    surf = lg.striped_surface(cfg)
    ctx = lg.Context(cfg, surf)
    for k, v in lg.initial_state(cfg, surf, seed=seed).items():
        ctx.set(k, v)
    ctx.step(steps)
    out = {nm: ctx.get(nm)[:-1, :, :n] for nm in ["u", "v", "w", "theta", "Cs_opt2"]}
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
    assert errs["velocity"] <= 1e-5, errs
    assert errs["theta"] <= 1e-5, errs
    assert a["rmsdiv"] <= 1e-10, a["rmsdiv"]
