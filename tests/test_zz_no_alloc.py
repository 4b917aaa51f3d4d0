"""les_tridag_array_noalloc: the tridiagonal solve for callers that cannot
allocate device memory (applications whose device memory all comes from
their own pool or arena, or code that must not allocate mid-run).  It takes
device pointers and draws its scratch from a fixed array inside the library.

Checked through the C ABI against les_tridag_array on two calls in a row on
the same buffers (the scratch keeps the previous call's contents): the same
kernel on the same inputs, so the results must be bit-identical; the first
call is also held to the CPU oracle's tridag_array.  A second case runs on a
non-default stream with u pre-filled with a sentinel, so the modes the solve
skips keep the caller's values exactly as tridag_array.f90 leaves them.
Then the size limit, the pointer checks, a row-1 zero pivot (u left
unchanged) and the clearing of the pivot flag between calls.  The file is
named to run last in the suite.
"""
import ctypes

import numpy as np
import pytest

import les_gb300 as lg

pytestmark = pytest.mark.gpu

ORACLE_TOL = 1e-13   # the tolerance of the les_tridag_array parity test
LES_ERR_ARG, LES_ERR_PIVOT = -1, -4
MAX_ELEMS = 1 << 21  # LES_NOALLOC_TRIDAG_MAX_ELEMS
SENTINEL = -12345.0


def rel(a, b):
    nb = np.linalg.norm(b)
    return np.linalg.norm(a - b) / (nb if nb > 0 else 1.0)


def _fn():
    f = lg.lib().les_tridag_array_noalloc
    vp = ctypes.c_void_p
    f.restype = ctypes.c_int
    f.argtypes = [vp, vp, vp, vp, vp, ctypes.c_int, ctypes.c_int, ctypes.c_int, vp]
    return f


def _system(shp, seed):
    rng = np.random.default_rng(seed)
    a = rng.uniform(0.5, 1.0, shp)
    c = rng.uniform(0.5, 1.0, shp)
    b = -(a + c + rng.uniform(0.1, 1.0, shp))
    r = rng.standard_normal(shp + (2,))
    return a, b, c, r


def test_noalloc_matches_tridag_array_two_calls(gpu_lib):
    import torch
    from oracle.oracle import Oracle
    cfg = lg.make_config(64, 64, 48)
    d = lg.dims(cfg)
    lh, ny, n = d["lh"], cfg.ny, cfg.nz + 1
    shp = (n, ny, lh)
    ctx = lg.Context(cfg)
    f = _fn()
    dev = torch.device("cuda", 0)
    A = torch.empty(shp, dtype=torch.float64, device=dev)
    B, C = torch.empty_like(A), torch.empty_like(A)
    R = torch.empty(shp + (2,), dtype=torch.float64, device=dev)
    U = torch.zeros_like(R)
    stream = torch.cuda.current_stream(dev).cuda_stream
    for seed in (21, 22):
        a, b, c, r = _system(shp, seed)
        u_ref = np.zeros_like(r)
        ctx.call("tridag_array", a, b, c, r, u_ref)
        for T, x in ((A, a), (B, b), (C, c), (R, r)):
            T.copy_(torch.from_numpy(x))
        torch.cuda.synchronize()
        st = f(A.data_ptr(), B.data_ptr(), C.data_ptr(), R.data_ptr(), U.data_ptr(), lh, ny, n, stream)
        assert st == 0, lg.lib().les_last_error()
        got = U.cpu().numpy()
        assert np.array_equal(got, u_ref), (seed, rel(got, u_ref))
        if seed == 21:
            u_orc = np.zeros_like(r)
            Oracle(cfg).call("tridag_array", a, b, c, r, u_orc)
            assert rel(got, u_orc) < ORACLE_TOL
    ctx.close()


def test_noalloc_side_stream_keeps_skipped_modes(gpu_lib):
    import torch
    cfg = lg.make_config(32, 32, 20)
    d = lg.dims(cfg)
    lh, ny, n = d["lh"], cfg.ny, cfg.nz + 1
    shp = (n, ny, lh)
    a, b, c, r = _system(shp, 31)
    ctx = lg.Context(cfg)
    u_ref = np.full(shp + (2,), SENTINEL)
    ctx.call("tridag_array", a, b, c, r, u_ref)
    ctx.close()
    f = _fn()
    dev = torch.device("cuda", 0)
    side = torch.cuda.Stream(device=dev)
    with torch.cuda.stream(side):
        A, B, C = (torch.from_numpy(x).to(dev, non_blocking=False) for x in (a, b, c))
        R = torch.from_numpy(r).to(dev)
        U = torch.full(shp + (2,), SENTINEL, dtype=torch.float64, device=dev)
    side.synchronize()
    for _ in range(2):
        st = f(A.data_ptr(), B.data_ptr(), C.data_ptr(), R.data_ptr(), U.data_ptr(), lh, ny, n,
               side.cuda_stream)
        assert st == 0, lg.lib().les_last_error()
        got = U.cpu().numpy()
        assert np.array_equal(got, u_ref)
    # the skipped modes beyond row 1 still hold the sentinel
    assert (got[1:, ny // 2, :, :] == SENTINEL).all()
    assert (got[1:, :, lh - 1, :] == SENTINEL).all()
    assert (got[1:, 0, 0, :] == SENTINEL).all()


def test_noalloc_limits_and_pivot_flag(gpu_lib):
    import torch
    f = _fn()
    dev = torch.device("cuda", 0)
    lh, ny, n = 9, 16, 13
    shp = (n, ny, lh)
    a, b, c, r = _system(shp, 5)
    A, B, C = (torch.from_numpy(x).to(dev) for x in (a, b, c))
    R = torch.from_numpy(r).to(dev)
    U = torch.zeros_like(R)
    stream = torch.cuda.current_stream(dev).cuda_stream
    ptrs = [A.data_ptr(), B.data_ptr(), C.data_ptr(), R.data_ptr(), U.data_ptr()]
    # beyond the fixed scratch: rejected before any GPU work
    assert f(*ptrs, 129, 256, 257, stream) == LES_ERR_ARG
    assert b"exceeds" in lg.lib().les_last_error()
    assert MAX_ELEMS // (129 * 256) < 257
    # a host pointer is rejected, not dereferenced on the device
    host = np.zeros(shp)
    assert f(host.ctypes.data, *ptrs[1:], lh, ny, n, stream) == LES_ERR_ARG
    # a zero b in row 1 reports a pivot error before the solve: u unchanged
    b0 = b.copy()
    b0[0, 3, 2] = 0.0
    B.copy_(torch.from_numpy(b0))
    U.fill_(SENTINEL)
    torch.cuda.synchronize()
    assert f(*ptrs, lh, ny, n, stream) == LES_ERR_PIVOT
    assert (U.cpu().numpy() == SENTINEL).all()
    # the next call starts clean
    B.copy_(torch.from_numpy(b))
    U.zero_()
    torch.cuda.synchronize()
    assert f(*ptrs, lh, ny, n, stream) == 0, lg.lib().les_last_error()
    assert np.isfinite(U.cpu().numpy()).all()
