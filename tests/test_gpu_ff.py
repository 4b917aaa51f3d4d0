"""Precision 2: the FP64 form's state, pointwise arithmetic, dynamic models
and projection (pressure transforms and solve) with every other spectral
transform in float-float (about 48 significant bits on the FP32 pipe),
against the CPU oracle through the C ABI, at the FP64 form's tolerance.

Those transforms see each field's plane mean taken out (u, v, w, theta, the
wall shear stresses, the Lagrangian products) and put back in FP64, so a
float-float rounding is relative to the fluctuations.  Measured against the
oracle: u, theta, qmix at the FP64 form's level (<= 2e-15), v and w <= 3.3e-13
(32^3 to 128^3), rmsdiv after the projection at the FP64 form's level.
"""
import numpy as np
import pytest

import les_gb300 as lg
from les_gb300.config import moisture_flux

pytestmark = pytest.mark.gpu

TOL = 1e-12   # FP64 parity tolerance of the step (relative L2), every field
RMSDIV_ABS = 1e-12  # after the projection (FP64 form: 1e-14 .. 1e-13)


def rel(a, b):
    nb = np.linalg.norm(b)
    return np.linalg.norm(a - b) / (nb if nb > 0 else 1.0)


@pytest.fixture(scope="module")
def libs(gpu_lib, oracle_lib):
    return gpu_lib, oracle_lib


def ff_pair(n, s_flag=1, jt0=0, q=0, model=5, seed=11):
    from oracle.oracle import Oracle
    cfg = lg.make_config(n, s_flag=s_flag, q_flag=q, jt_total0=jt0, model=model, rmsdiv_every=1, precision=2)
    surf = lg.striped_surface(cfg) if s_flag else lg.uniform_surface(cfg)
    g = lg.Context(cfg, surf)
    o = Oracle(cfg, surf)
    if q:
        wq = moisture_flux(cfg)
        g.set("wq_s", wq)
        o.set("wq_s", wq)
    levels = cfg.nz if model == 7 else 10
    for k, v in lg.initial_state(cfg, surf, seed=seed, theta_levels=levels).items():
        g.set(k, v)
        o.set(k, v)
    return cfg, g, o


def check(cfg, g, o, tight):
    n = cfg.nx
    for nm in tight:
        e = rel(g.get(nm)[:-1, :, :n], o.get(nm)[:-1, :, :n])
        assert e < TOL, (nm, e)
    e = rel(g.get("v")[:-1, :, :n], o.get("v")[:-1, :, :n])
    assert e < TOL, ("v", e)
    e = rel(g.get("w")[:, :, :n], o.get("w")[:, :, :n])
    assert e < TOL, ("w", e)
    assert g.rmsdiv() < RMSDIV_ABS


@pytest.mark.parametrize("s_flag,jt0", [(0, 0), (1, 0), (1, 500)])
def test_ff_step_parity_32(libs, s_flag, jt0):
    cfg, g, o = ff_pair(32, s_flag=s_flag, jt0=jt0)
    g.step(1)
    assert o.step(1) == 0
    # first-step rmsdiv: the divergence of the seeded state (order 1)
    rg, ro = g.rmsdiv(), o.rmsdiv()
    assert abs(rg - ro) <= TOL * abs(ro), (rg, ro)
    g.step(9)
    assert o.step(9) == 0
    check(cfg, g, o, ["u", "theta"] if s_flag else ["u"])


def test_ff_step_parity_humidity_and_model7(libs):
    """qmix with the striped moisture flux, and SGS model 7 from
    jt_total = 500 (the dynamic Pr_t feeding back), 10 steps at 32^3."""
    cfg, g, o = ff_pair(32, q=1)
    g.step(10)
    assert o.step(10) == 0
    check(cfg, g, o, ["u", "theta", "q"])
    cfg, g, o = ff_pair(32, jt0=500, model=7)
    g.step(10)
    assert o.step(10) == 0
    check(cfg, g, o, ["u", "theta"])


def test_ff_step_parity_128_theta(libs):
    """128^3 with theta and the striped surface, 20 steps."""
    cfg, g, o = ff_pair(128)
    g.step(20)
    assert o.step(20) == 0
    check(cfg, g, o, ["u", "theta"])


def test_ff_against_fp64_form(gpu_lib):
    """The float-float transform form against the FP64 form on the GPU,
    64^3 with theta over 30 steps."""
    out = {}
    for prec in (2, 0):
        cfg = lg.make_config(64, s_flag=1, rmsdiv_every=1, precision=prec)
        surf = lg.striped_surface(cfg)
        g = lg.Context(cfg, surf)
        for k, v in lg.initial_state(cfg, surf, seed=13).items():
            g.set(k, v)
        g.step(30)
        out[prec] = {nm: g.get(nm)[:-1, :, :64] for nm in ("u", "v", "w", "theta")}
        g.close()
    for nm in ("u", "v", "w", "theta"):
        assert rel(out[2][nm], out[0][nm]) < TOL, nm
