"""FP32-mixed form vs the FP64 form on the GPU (same seeded inputs).

The mixed form runs the scalar, convective, stress-divergence and SGS
transforms in FP32 with FP32 3/2-grid and filter temporaries; u, v, w, theta,
the AB2 update, filt_da of the velocity, the pressure solve and the plane
(wall-stress, mean-profile) quantities stay FP64.  Targets: relative error
<= 1e-5 on velocity and theta, rmsdiv <= 1e-10."""
import numpy as np
import pytest

import les_gb300 as lg

pytestmark = pytest.mark.gpu


def rel(a, b):
    return np.linalg.norm(a - b) / np.linalg.norm(b)


@pytest.mark.parametrize("n,steps", [(32, 20), (64, 50)])
def test_mixed_vs_fp64(gpu_lib, n, steps):
    out = {}
    for prec in (0, 1):
        cfg = lg.make_config(n, s_flag=1, jt_total0=500, precision=prec, rmsdiv_every=10)
        surf = lg.striped_surface(cfg)
        ctx = lg.Context(cfg, surf)
        for k, v in lg.initial_state(cfg, surf, seed=3).items():
            ctx.set(k, v)
        ctx.step(steps)
        out[prec] = {nm: ctx.get(nm)[:-1, :, :n] for nm in ["u", "v", "w", "theta", "Cs_opt2"]}
        out[prec]["rmsdiv"] = ctx.rmsdiv()
        ctx.close()
    for nm in ["u", "v", "w", "theta"]:
        e = rel(out[1][nm], out[0][nm])
        assert e <= 1e-5, (nm, e)
    assert out[1]["rmsdiv"] <= 1e-10, out[1]["rmsdiv"]
    assert rel(out[1]["Cs_opt2"], out[0]["Cs_opt2"]) < 1e-2
