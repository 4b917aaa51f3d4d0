"""Running statistics (io.f90:403-1218 MM_XYZ_Out) on the GPU against the
oracle's restatement: all 133 accumulators after a run that accumulates
every c_count steps and zeroes the two output groups every p_count and
2 p_count steps, as output_loop does (io.f90:211-213)."""
import numpy as np
import pytest

import les_gb300 as lg
from les_gb300.config import moisture_flux

pytestmark = pytest.mark.gpu


def rel(a, b):
    nb = np.linalg.norm(b)
    return np.linalg.norm(a - b) / (nb if nb > 0 else 1.0)


def pair(n=32, q=1, precision=0, oracle=True):
    from oracle.oracle import Oracle
    cfg = lg.make_config(n, s_flag=1, q_flag=q, rmsdiv_every=1, precision=precision)
    surf = lg.striped_surface(cfg)
    g = lg.Context(cfg, surf)
    o = Oracle(cfg, surf) if oracle else None
    if q:
        wq = moisture_flux(cfg)
        g.set("wq_s", wq)
        if o is not None:
            o.set("wq_s", wq)
    for k, v in lg.initial_state(cfg, surf, seed=51).items():
        g.set(k, v)
        if o is not None:
            o.set(k, v)
    return cfg, g, o


@pytest.mark.parametrize("q", [1, 0])
def test_stats_match_oracle(gpu_lib, oracle_lib, q):
    cfg, g, o = pair(q=q)
    c_count, p_count = 2, 4
    g.stats_enable(c_count, p_count)
    o.stats_enable(c_count, p_count)
    names = lg.stats_names()
    groups = lg.stats_groups()
    assert len(names) == 133
    worst = {}
    for jt in range(1, 9):
        g.step(1)
        assert o.step(1) == 0
        if jt % c_count:
            continue
        g.stats_accumulate()
        o.stats_accumulate()
        for nm in names:
            e = rel(g.stats_get(nm), o.stats_get(nm))
            worst[nm] = max(worst.get(nm, 0.0), e)
        for grp, every in ((1, p_count), (2, 2 * p_count)):
            if jt % every == 0:
                g.stats_reset(grp)
                o.stats_reset(grp)
    bad = {nm: e for nm, e in worst.items() if e > 1e-10}
    assert not bad, bad
    assert sum(1 for v in groups.values() if v == 1) == 19 and groups["atxy"] == 0
    # the group-1 statistics were zeroed at the last output step, group 2 not
    assert not g.stats_get("au").any() and not g.stats_get("ap").any()
    assert g.stats_get("atxy").any()


def test_stats_auto_accumulate_matches_manual(gpu_lib):
    """With auto accumulation les_step adds the statistics after every
    c_count-th step; the result is bit-identical to accumulating by hand."""
    cfg, a, _ = pair(oracle=False)
    _, b, _ = pair(oracle=False)
    a.stats_enable(3, 6, auto=True)
    b.stats_enable(3, 6)
    a.step_graph(9)
    for jt in range(1, 10):
        b.step(1)
        if jt % 3 == 0:
            b.stats_accumulate()
    for nm in ("au", "u2", "awt", "at13s13", "asgsq3", "azlcl_all", "adpdz"):
        assert np.array_equal(a.stats_get(nm), b.stats_get(nm)), nm


def test_stats_mixed_form(gpu_lib):
    """The FP32-mixed form's statistics (FP32-held gradients and stresses
    widened in the accumulation) against the FP64 form's after 6 steps."""
    out = {}
    for prec in (1, 0):
        cfg, g, _ = pair(n=64, precision=prec, oracle=False)
        g.stats_enable(2, 4, auto=True)
        g.step(6)
        out[prec] = {nm: g.stats_get(nm) for nm in ("au", "u2", "atheta", "aq", "awt", "atxz", "adudz", "asgst3")}
        g.close()
    for nm in out[0]:
        e = rel(out[1][nm], out[0][nm])
        assert e < 1e-4, (nm, e)
