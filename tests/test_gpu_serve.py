"""Serving on the GPU: every member's state after the served trace is
bit-identical to the same member advanced alone by the same number of steps
(members share nothing on the device; steps of different members overlap)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_result_same_alone_and_in_the_mix(gpu_lib):
    import les_gb300 as lg
    from les_gb300.serve import GpuExecutor, Request, Scheduler
    sizes = {0: (32, 32, 32), 1: (32, 32, 24), 2: (48, 48, 32), 3: (64, 64, 16)}
    trace = []
    t = 0.0
    rng = np.random.default_rng(4)
    for rid in range(14):
        m = int(rng.integers(4))
        t += float(rng.exponential(0.004))
        trace.append(Request(rid=rid, member=m, size=sizes[m], nsteps=int(rng.integers(1, 8)), arrival=t))
    ex = GpuExecutor(precision=1, autotune=False)
    s = Scheduler(ex, budget_bytes=64 << 30)
    summary, wall = s.run(trace)
    assert all(r.status == "done" for r in s.done), [(r.rid, r.status, r.error) for r in s.done]
    served = {m: sum(r.nsteps for r in trace if r.member == m) for m in sizes}
    assert summary["steps"] == sum(served.values())
    solo = GpuExecutor(precision=1, autotune=False)
    for m, n in served.items():
        if n == 0:
            continue
        solo.load(m, sizes[m])
        solo.ctx[m].step(n)
        a, b = ex.state(m), solo.state(m)
        for k in a:
            assert np.array_equal(a[k], b[k]), (m, k)
        solo.evict(m)


def test_evicted_members_resume_exactly(gpu_lib):
    """A memory budget that holds about two of the four members forces
    evictions: an evicted member is spilled to host memory with its whole
    state and resumed from it when it is admitted again, so every member's
    final state is still bit-identical to the same member advanced alone.
    Step latencies are device times (CUDA events around each step)."""
    import les_gb300 as lg
    from les_gb300.serve import GpuExecutor, Request, Scheduler
    sizes = {0: (32, 32, 32), 1: (32, 32, 24), 2: (48, 48, 32), 3: (64, 64, 16)}
    ex = GpuExecutor(precision=1, autotune=False)
    fp = {m: ex.footprint(sz) for m, sz in sizes.items()}
    budget = max(fp.values()) + sorted(fp.values())[-2] + 1
    trace = []
    t = 0.0
    rng = np.random.default_rng(9)
    for rid in range(24):
        m = rid % 4 if rid < 8 else int(rng.integers(4))
        t += float(rng.exponential(0.003))
        trace.append(Request(rid=rid, member=m, size=sizes[m], nsteps=int(rng.integers(1, 7)), arrival=t))
    s = Scheduler(ex, budget_bytes=budget)
    summary, wall = s.run(trace)
    assert all(r.status == "done" for r in s.done), [(r.rid, r.status, r.error) for r in s.done]
    assert summary["evicted"] > 0 and ex.restores > 0, (summary["evicted"], ex.restores)
    assert all(0.0 < x < 5.0 for x in s.metrics.step_lat)
    served = {m: sum(r.nsteps for r in trace if r.member == m) for m in sizes}
    solo = GpuExecutor(precision=1, autotune=False)
    for m, n in served.items():
        if n == 0:
            continue
        if m not in ex.ctx:  # spilled at the end of the trace: bring it back to read it
            ex.load(m, sizes[m])
        solo.load(m, sizes[m])
        solo.ctx[m].step(n)
        a, b = ex.state(m), solo.state(m)
        for k in a:
            assert np.array_equal(a[k], b[k]), (m, k)
        assert ex.ctx[m].counters() == solo.ctx[m].counters()
        solo.evict(m)
