"""CUDA-graph replay and ensembles: a step replayed from a captured graph runs
the same kernels on the same buffers as an eager step, so results are
bit-identical; an ensemble member's result is bit-identical to the same
member advanced alone (members share nothing on the device)."""
import numpy as np
import pytest

import les_gb300 as lg

pytestmark = pytest.mark.gpu


def member(n, nzl, seed, precision=1, jt0=500, ny=None):
    cfg = lg.make_config(n, ny, nzl, s_flag=1, jt_total0=jt0, precision=precision, rmsdiv_every=0)
    surf = lg.patch_surface(cfg, seed)
    surf.wt_s[:] = 0.05
    ctx = lg.Context(cfg, surf)
    for k, v in lg.initial_state(cfg, surf, seed=seed).items():
        ctx.set(k, v)
    return ctx


def state(ctx):
    return {k: ctx.get(k) for k in ("u", "v", "w", "theta", "F_LM", "Cs_opt2")}


@pytest.mark.parametrize("precision", [0, 1])
def test_graph_replay_is_bit_identical(gpu_lib, precision):
    a = member(32, 32, 5, precision)
    b = member(32, 32, 5, precision)
    a.step(12)
    b.step_graph(12)
    sa, sb = state(a), state(b)
    for k in sa:
        assert np.array_equal(sa[k], sb[k]), k


@pytest.mark.parametrize("precision", [1, 2])
def test_graph_prepare_changes_nothing(gpu_lib, precision):
    """les_step_graph_prepare captures the replayed step graphs ahead of time
    without stepping: counters and state are unchanged, and the prepared
    member then replays bit-identically to one capturing on first use and to
    eager steps."""
    a = member(32, 32, 7, precision)
    b = member(32, 32, 7, precision)
    c = member(32, 32, 7, precision)
    a.step(1)
    b.step(1)
    c.step(1)
    before = state(b)
    b.graph_prepare()
    assert b.counters() == a.counters()
    after = state(b)
    for k in before:
        assert np.array_equal(before[k], after[k]), k
    a.step_graph(11)
    b.step_graph(11)
    c.step(11)
    sa, sb, sc = state(a), state(b), state(c)
    for k in sa:
        assert np.array_equal(sa[k], sb[k]), k
        assert np.array_equal(sa[k], sc[k]), k


def test_autotune_keeps_results(gpu_lib):
    a = member(32, 32, 6)
    b = member(32, 32, 6)
    tuned = b.autotune()
    assert tuned["tx64"] in (2, 4, 8) and tuned["tx32"] in (4, 8, 16)
    a.step(6)
    b.step(6)
    sa, sb = state(a), state(b)
    for k in ("u", "v", "w", "theta"):
        e = np.linalg.norm(sa[k] - sb[k]) / np.linalg.norm(sa[k])
        assert e < 1e-12, (k, e, tuned)


def test_ensemble_member_equals_alone(gpu_lib):
    shapes = [(32, 32, None), (32, 24, None), (48, 32, None), (64, 16, 48)]
    ens_members = [member(n, z, 100 + i, ny=ny) for i, (n, z, ny) in enumerate(shapes)]
    alone = [member(n, z, 100 + i, ny=ny) for i, (n, z, ny) in enumerate(shapes)]
    for m in alone:
        m.step(11)
    ens = lg.Ensemble(ens_members)
    ens.step(11)
    # read right after the ensemble step: a member's field read (on its own
    # stream) must be ordered after the graph launched on the ensemble stream
    for m, a in zip(ens_members, alone):
        sm, sa = state(m), state(a)
        for k in sm:
            assert np.array_equal(sm[k], sa[k]), k
    ens.close()
