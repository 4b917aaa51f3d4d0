"""Checkpoint record on the GPU (les_checkpoint_write / _read through the C
ABI): the file holds the io.f90:1314-1338 list, checked array by array with
the numpy restatement in oracle/fortran_record.py; reading it into a fresh
context restores the state bit for bit; a velocity-only restart continues
exactly as the uninterrupted run does."""
import numpy as np
import pytest

import les_gb300 as lg
from oracle import fortran_record as fr

pytestmark = pytest.mark.gpu

CARRIED = {1: ["u", "v", "w", "theta", "RHSx", "RHSy", "RHSz", "RHS_T", "psi_m", "psi_m0", "psi_h", "psi_h0",
               "Cs_opt2", "F_LM", "F_MM", "F_QN", "F_NN", "sgs_t3"],
           0: ["u", "v", "w", "RHSx", "RHSy", "RHSz", "Cs_opt2", "F_LM", "F_MM", "F_QN", "F_NN"]}


def member(n, s_flag, precision=0, jt_total0=500, restart=False):
    cfg = lg.make_config(n, s_flag=s_flag, jt_total0=jt_total0, precision=precision,
                         initu=int(restart), initsc=int(restart and s_flag), rmsdiv_every=0)
    surf = lg.striped_surface(cfg)
    ctx = lg.Context(cfg, surf)
    if not restart:
        for k, v in lg.initial_state(cfg, surf, seed=11).items():
            ctx.set(k, v)
    return cfg, ctx


@pytest.mark.parametrize("s_flag,precision", [(1, 0), (0, 0), (1, 1)])
def test_checkpoint_file_and_round_trip(gpu_lib, tmp_path, s_flag, precision):
    n = 32
    cfg, a = member(n, s_flag, precision)
    a.step(10)
    p = str(tmp_path / "vel_sc.out")
    a.checkpoint_write(p)
    data, end = fr.read_record(open(p, "rb").read())
    assert end == len(open(p, "rb").read())  # one record, nothing after it
    arr = fr.split_checkpoint(data, n, n, cfg.nz, s_flag)
    for name in CARRIED[s_flag]:
        want = a.get(name)
        got = arr[name].T
        if name == "sgs_t3":  # (ld,ny) plane in the record, (nx,ny) in the context
            assert np.all(got[:, n:] == 0)
            got = got[:, :n]
        assert np.array_equal(got, want), name
    if s_flag:
        for name in ("qmix", "RHS_q", "sgs_q3", "G_LM", "G_MM", "G_QN", "G_NN"):
            assert not arr[name].any(), name
        assert np.all(arr["Pr_t"] == cfg.pr)
    # read into a fresh restart context: the same state bit for bit
    _, b = member(n, s_flag, precision, jt_total0=cfg.jt_total0 + 10, restart=True)
    b.checkpoint_read(p)
    for name in CARRIED[s_flag]:
        assert np.array_equal(b.get(name), a.get(name)), name
    b.step(5)
    assert np.isfinite(b.get("u")).all() and b.rmsdiv() < 1e-10
    a.close(); b.close()


def test_velocity_restart_continues_exactly(gpu_lib, tmp_path):
    """Without scalars nothing outside the record survives a step once the
    Lagrangian accumulators are reset (a step count that is a multiple of
    cs_count): 10 steps, checkpoint, restart, 5 steps equals 15 steps."""
    n = 32
    cfg, a = member(n, 0)
    a.step(10)
    p1, p2, p3 = (str(tmp_path / s) for s in ("c10.out", "a15.out", "b15.out"))
    a.checkpoint_write(p1)
    _, b = member(n, 0, jt_total0=cfg.jt_total0 + 10, restart=True)
    b.checkpoint_read(p1)
    a.step(5)
    b.step(5)
    for name in ("u", "v", "w", "Cs_opt2", "F_LM", "F_MM"):
        assert np.array_equal(a.get(name), b.get(name)), name
    a.checkpoint_write(p2)
    b.checkpoint_write(p3)
    assert open(p2, "rb").read() == open(p3, "rb").read()
    a.close(); b.close()


def test_checkpoint_read_rejects_a_short_record(gpu_lib, tmp_path):
    cfg, a = member(32, 1)
    p = str(tmp_path / "short.out")
    lg.fortran_record_write(p, [np.zeros(100)])
    with pytest.raises(lg.LesError) as e:
        a.checkpoint_read(p)
    assert e.value.code == -10
    a.close()


def test_checkpoint_read_refuses_the_other_layout(gpu_lib, tmp_path):
    """A record written without scalars does not read into a context with
    them (the lists differ in length); nothing in the context changes."""
    _, a = member(32, 0)
    p = str(tmp_path / "vel.out")
    a.checkpoint_write(p)
    _, b = member(32, 1)
    u0, th0 = b.get("u"), b.get("theta")
    with pytest.raises(lg.LesError) as e:
        b.checkpoint_read(p)
    assert e.value.code == -10
    assert np.array_equal(b.get("u"), u0) and np.array_equal(b.get("theta"), th0)
    a.close(); b.close()
