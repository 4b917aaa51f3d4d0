"""Host-side tests of the continuous-batching scheduler against a fake
executor (no GPU): admission by footprint, eviction, rejection, injected
allocation failure, cancellation, a failing member, continuous batching."""
from les_gb300.serve import FakeExecutor, Request, Scheduler, poisson_trace


def R(rid, member, n=3, size=(32, 32, 32), t=0.0):
    return Request(rid=rid, member=member, size=size, nsteps=n, arrival=t)


def drain(s, limit=1000):
    for _ in range(limit):
        if s.idle():
            return
        s.tick(0.0)
        s.poll()
    raise AssertionError("scheduler did not drain")


def test_concurrent_requests_share_ticks():
    ex = FakeExecutor()
    s = Scheduler(ex, budget_bytes=10 ** 12)
    for i in range(4):
        s.submit(R(i, member=i, n=5))
    s.tick(0.0)
    assert len(s.active) == 4                      # all four run in the same tick
    assert sum(r.inflight for r in s.active) == 4
    s.poll()
    s.submit(R(9, member=9, n=2))                  # arrives while others run
    s.tick(0.0)
    assert any(r.rid == 9 and r.status == "active" for r in s.active)
    drain(s)
    assert all(r.status == "done" for r in s.done)
    assert ex.steps[0] == 5 and ex.steps[9] == 2


def test_admission_waits_for_memory_and_evicts_idle():
    ex = FakeExecutor()
    fp = ex.footprint((32, 32, 32))
    s = Scheduler(ex, budget_bytes=2 * fp + 1)
    s.submit(R(0, 0, n=3)); s.submit(R(1, 1, n=3)); s.submit(R(2, 2, n=3))
    s.tick(0.0)
    assert {r.member for r in s.active} == {0, 1}
    assert len(s.pending) == 1                     # member 2 waits for room
    drain(s)
    assert [r.status for r in sorted(s.done, key=lambda r: r.rid)] == ["done"] * 3
    assert s.metrics.evicted >= 1 and s.used <= s.budget


def test_oversized_member_rejected():
    ex = FakeExecutor()
    s = Scheduler(ex, budget_bytes=ex.footprint((32, 32, 32)))
    s.submit(R(0, 0, size=(128, 128, 128)))
    s.submit(R(1, 1))
    drain(s)
    st = {r.rid: r.status for r in s.done}
    assert st == {0: "rejected", 1: "done"}


def test_injected_allocation_failure_is_rejected_not_fatal():
    ex = FakeExecutor(fail_alloc={3})
    s = Scheduler(ex, budget_bytes=10 ** 12)
    s.submit(R(0, 3)); s.submit(R(1, 4))
    drain(s)
    st = {r.rid: (r.status, r.error) for r in s.done}
    assert st[0][0] == "rejected" and "allocation" in st[0][1]
    assert st[1][0] == "done"


def test_cancel_pending_and_active():
    ex = FakeExecutor()
    s = Scheduler(ex, budget_bytes=ex.footprint((32, 32, 32)) + 1)
    s.submit(R(0, 0, n=50)); s.submit(R(1, 1, n=5))
    s.tick(0.0)
    assert s.cancel(1)                              # still pending (no room)
    assert s.cancel(0)                              # active
    drain(s)
    st = {r.rid: r.status for r in s.done}
    assert st == {0: "cancelled", 1: "cancelled"}
    assert ex.steps[0] < 50


def test_failing_member_does_not_stop_others():
    ex = FakeExecutor(fail_step={7})
    s = Scheduler(ex, budget_bytes=10 ** 12)
    s.submit(R(0, 7)); s.submit(R(1, 8))
    drain(s)
    st = {r.rid: r.status for r in s.done}
    assert st == {0: "failed", 1: "done"}


def test_requests_on_one_member_run_in_order():
    ex = FakeExecutor()
    s = Scheduler(ex, budget_bytes=10 ** 12)
    s.submit(R(0, 5, n=4)); s.submit(R(1, 5, n=2))
    s.tick(0.0)
    assert sum(r.inflight for r in s.active) == 1   # only the older request steps
    drain(s)
    order = [r.rid for r in s.done]
    assert order == [0, 1]


def test_poisson_trace_shape():
    tr = poisson_trace(200, rate=200.0, seed=1)
    assert len(tr) == 200 and all(1 <= r.nsteps <= 50 for r in tr)
    gaps = [b.arrival - a.arrival for a, b in zip(tr, tr[1:])]
    assert 0.002 < sum(gaps) / len(gaps) < 0.01


def test_inflight_work_budget_bounds_concurrency():
    """With max_inflight_points the scheduler launches steps only while the
    points of the steps in flight fit the budget (one step always runs), the
    least recently served request first, and still completes every request."""
    ex = FakeExecutor()
    pts = 32 * 32 * 32
    s = Scheduler(ex, budget_bytes=10 ** 12, max_inflight_points=2 * pts)
    for i in range(5):
        s.submit(R(i, member=i, n=3))
    seen = []
    for _ in range(200):
        if s.idle():
            break
        s.tick(0.0)
        seen.append(sum(r.inflight for r in s.active))
        s.poll()
    assert s.idle() and max(seen) == 2
    assert all(r.status == "done" for r in s.done) and all(ex.steps[m] == 3 for m in range(5))
    # a member larger than the budget still runs, alone
    s2 = Scheduler(FakeExecutor(), budget_bytes=10 ** 12, max_inflight_points=pts)
    s2.submit(R(0, 0, size=(64, 64, 64)))
    drain(s2)
    assert s2.done[0].status == "done"


def test_step_latency_counts_the_wait_between_steps():
    """The step latency of a request's later steps runs from its previous
    step's completion; the device time of the step alone is kept beside it."""
    ex = FakeExecutor(ns_per_pt=1.0)
    s = Scheduler(ex, budget_bytes=10 ** 12)
    s.submit(R(0, 0, n=3))
    drain(s)
    assert len(s.metrics.step_lat) == 3 and len(s.metrics.step_dev) == 3
    assert all(g >= d - 1e-15 for g, d in zip(s.metrics.step_lat, s.metrics.step_dev))


def test_two_steps_in_flight_per_request():
    """With two steps of a request queued on its member's stream at once the
    host's poll-and-relaunch no longer sits between them; the steps still
    run in order, one stream per member, and every step is counted once."""
    ex = FakeExecutor(ns_per_pt=1.0)
    s = Scheduler(ex, budget_bytes=10 ** 12, max_inflight_per_member=2)
    s.submit(R(0, 0, n=5))
    s.submit(R(1, 1, n=1))
    s.tick(0.0)
    s.tick(0.0)
    reqs = {r.rid: r for r in s.active}
    assert reqs[0].inflight == 2 and reqs[1].inflight == 1
    ends = [b for (r, a, b, p, f) in ex.inflight if r.rid == 0]
    starts = [a for (r, a, b, p, f) in ex.inflight if r.rid == 0]
    assert starts[1] >= ends[0]                     # queued behind the first on the stream
    drain(s)
    assert ex.steps[0] == 5 and ex.steps[1] == 1
    assert len(s.metrics.step_lat) == 6
    assert all(r.status == "done" for r in s.done)


def test_active_slots_queue_requests_in_arrival_order():
    """With an active-points cap, pending requests start only as slots free
    up, in arrival order; the first one always starts; all complete."""
    ex = FakeExecutor()
    pts = 32 * 32 * 32
    s = Scheduler(ex, budget_bytes=10 ** 12, max_active_points=2 * pts)
    for i in range(5):
        s.submit(R(i, member=i, n=2))
    s.tick(0.0)
    assert sorted(r.rid for r in s.active) == [0, 1]
    assert [r.rid for r in s.pending] == [2, 3, 4]
    assert s.active_points == 2 * pts
    drain(s)
    assert all(r.status == "done" for r in s.done) and len(s.done) == 5
    assert s.active_points == 0
    big = Scheduler(FakeExecutor(), budget_bytes=10 ** 12, max_active_points=1)
    big.submit(R(0, 0, n=1, size=(64, 64, 64)))   # larger than the cap: starts when nothing runs
    big.tick(0.0)
    assert len(big.active) == 1


def test_active_slots_by_step_time():
    """max_active_ms caps the summed step-time estimates of the active
    requests (FakeExecutor: ns_per_pt per grid point)."""
    ex = FakeExecutor(ns_per_pt=1.0)              # a 32^3 step: 0.0328 ms
    s = Scheduler(ex, budget_bytes=10 ** 12, max_active_ms=0.07)
    for i in range(4):
        s.submit(R(i, member=i, n=2))
    s.tick(0.0)
    assert len(s.active) == 2 and len(s.pending) == 2
    drain(s)
    assert len(s.done) == 4 and abs(s.active_ms) < 1e-12


def test_lock_step_rounds():
    """With rounds, no step launches while any step of the previous round is
    in flight; every request still completes."""
    ex = FakeExecutor()
    s = Scheduler(ex, budget_bytes=10 ** 12, rounds=True)
    s.submit(R(0, 0, n=3))
    s.submit(R(1, 1, n=3, size=(64, 64, 64)))
    s.tick(0.0)
    assert len(ex.inflight) == 2
    s.tick(0.0)                       # round 1 still in flight: nothing new
    assert len(ex.inflight) == 2
    s.poll()
    s.tick(0.0)
    assert len(ex.inflight) == 2
    drain(s)
    assert ex.steps[0] == 3 and ex.steps[1] == 3
