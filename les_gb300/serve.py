"""Continuous-batching server for ensemble members.

Requests are "advance member M by N steps".  Member state stays resident on
the device between requests.  A new member is admitted only when its
estimated footprint (les_estimate_device_bytes) fits in the memory budget;
members that are idle are evicted least-recently-used when room is needed.
Every tick the scheduler launches one step of every active request, each on
its member's own stream, so steps of different members overlap on the GPU;
requests that arrive while others run join at the next tick (continuous
batching, not a queue).  A request's step latency runs from the completion
of its previous step to the completion of this one (its first step: from
the step's start), on the device's clock: CUDA events recorded on the
member's stream, so it includes host scheduling, any wait for an in-flight
work budget and the time the step shares the device with other members;
the device time of each step alone is reported beside it.  Request latency
runs from arrival to completion on the host clock.  An evicted member is spilled to host memory with its whole state
(les_state_save) and resumed from it when it is admitted again
(les_state_restore), so it continues exactly where it stopped.

The scheduler is pure host logic and runs against an executor: GpuExecutor
(les_gb300 contexts, graph-replayed steps) or FakeExecutor (deterministic
timings, for CPU tests of admission, cancellation and failure handling).
"""
import collections
import heapq
import math
import time
from dataclasses import dataclass, field

import numpy as np

SIZES = [(32, 32, 32), (64, 64, 64), (96, 96, 64), (128, 128, 128), (192, 192, 128)]
WEIGHTS = [0.3, 0.3, 0.2, 0.15, 0.05]


@dataclass
class Request:
    rid: int
    member: int           # member id (seeded state + surface)
    size: tuple           # (nx, ny, nz_levels)
    nsteps: int
    arrival: float        # seconds, trace time
    arrival_wall: float = None
    done_steps: int = 0
    inflight: int = 0
    started: float = None
    finished: float = None
    status: str = "pending"   # pending | active | done | cancelled | rejected | failed
    error: str = None
    last_tick: int = 0
    prev_done: object = None  # executor's completion marker of the previous step


@dataclass
class Metrics:
    step_lat: list = field(default_factory=list)            # seconds, inter-step (see Scheduler)
    step_lat_by_size: dict = field(default_factory=lambda: collections.defaultdict(list))
    step_dev: list = field(default_factory=list)            # seconds, device time of the step alone
    req_lat: list = field(default_factory=list)
    pt_steps: float = 0.0
    admitted: int = 0
    rejected: int = 0
    evicted: int = 0

    def summary(self, wall):
        def pct(a, q):
            return float(np.percentile(a, q)) if len(a) else None
        out = {"steps": len(self.step_lat),
               "step_p50_ms": None if not self.step_lat else 1e3 * pct(self.step_lat, 50),
               "step_p99_ms": None if not self.step_lat else 1e3 * pct(self.step_lat, 99),
               "step_device_p50_ms": None if not self.step_dev else 1e3 * pct(self.step_dev, 50),
               "step_device_p99_ms": None if not self.step_dev else 1e3 * pct(self.step_dev, 99),
               "req_p50_ms": None if not self.req_lat else 1e3 * pct(self.req_lat, 50),
               "req_p99_ms": None if not self.req_lat else 1e3 * pct(self.req_lat, 99),
               "pt_steps_per_s": self.pt_steps / wall if wall > 0 else None,
               "admitted": self.admitted, "rejected": self.rejected, "evicted": self.evicted,
               "by_size": {}}
        for sz, lat in sorted(self.step_lat_by_size.items()):
            out["by_size"]["%dx%dx%d" % sz] = {"n": len(lat), "p50_ms": 1e3 * pct(lat, 50),
                                              "p99_ms": 1e3 * pct(lat, 99)}
        return out


def poisson_trace(n_requests, rate, seed, n_members=64, sizes=SIZES, weights=WEIGHTS, nmax=50):
    """Poisson arrivals of 'advance N' requests (N ~ U{1..nmax}) over a pool
    of members whose sizes are drawn with the given weights."""
    rng = np.random.default_rng(seed)
    msize = [sizes[i] for i in rng.choice(len(sizes), size=n_members, p=weights)]
    t = 0.0
    reqs = []
    for r in range(n_requests):
        t += rng.exponential(1.0 / rate)
        m = int(rng.integers(n_members))
        reqs.append(Request(rid=r, member=m, size=msize[m], nsteps=int(rng.integers(1, nmax + 1)), arrival=t))
    return reqs


class Scheduler:
    """Admission by footprint, one step per active request per tick.

    A request's step latency is the time from the completion of its previous
    step (or, for its first step, from the step's start on the device) to
    the completion of this one, on the device's clock (CUDA events on the
    member's stream): what the request waits per step, host scheduling and
    queueing included.  The device time of the step alone is kept beside it.
    With max_inflight_points set, a tick launches steps only while the grid
    points of all steps in flight stay within it (at least one step always
    runs), oldest-served request first: every step then shares the device
    with a bounded amount of other work, which bounds the spread of its
    latency at some cost in overlap.

    With max_active_points set, a pending request becomes active (a slot)
    only while the grid points of the active requests stay within it (one is
    always admitted when none is active), in arrival order: under overload
    the requests queue before they start instead of all stretching each
    other's steps, so the work of one round of steps, and with it the step
    latency, stays near the cap.  max_active_ms caps instead the sum of the
    active requests' step times as the executor estimates them
    (executor.step_ms(size)); small members' steps are launch-bound, so
    equal points are not equal time.

    With rounds set, the active requests step in lock-step rounds: a tick
    launches only when every step of the previous round has completed, so
    every request of a round sees the same latency whatever its member's
    size (small members do not run ahead of large ones)."""

    def __init__(self, executor, budget_bytes, max_inflight_per_member=1, clock=time.perf_counter,
                 max_inflight_points=None, max_active_points=None, max_active_ms=None, rounds=False):
        self.ex = executor
        self.budget = budget_bytes
        self.used = 0
        self.resident = collections.OrderedDict()   # member -> bytes (LRU order)
        self.busy = collections.Counter()          # member -> active requests
        self.pending = collections.deque()
        self.active = []
        self.metrics = Metrics()
        self.clock = clock
        self.max_inflight = max_inflight_per_member
        self.max_points = max_inflight_points
        self.inflight_points = 0
        self.max_active = max_active_points
        self.active_points = 0
        self.max_active_ms = max_active_ms
        self.active_ms = 0.0
        self.rounds = rounds
        self.tick_no = 0
        self.done = []

    # ---- admission ----------------------------------------------------------
    def _admit_member(self, req):
        if req.member in self.resident:
            self.resident.move_to_end(req.member)
            return True
        need = self.ex.footprint(req.size)
        if need > self.budget:
            req.status = "rejected"
            req.error = "footprint %d B exceeds the memory budget %d B" % (need, self.budget)
            self.metrics.rejected += 1
            return False
        # evict idle members, least recently used first
        while self.used + need > self.budget:
            victim = next((m for m in self.resident if self.busy[m] == 0), None)
            if victim is None:
                return False  # wait for memory to free up
            self.used -= self.resident.pop(victim)
            self.ex.evict(victim)
            self.metrics.evicted += 1
        try:
            self.ex.load(req.member, req.size)
        except MemoryError as e:  # allocation failure: reject, keep serving
            req.status = "rejected"
            req.error = str(e)
            self.metrics.rejected += 1
            return False
        self.resident[req.member] = need
        self.used += need
        self.metrics.admitted += 1
        return True

    def submit(self, req):
        self.pending.append(req)

    def cancel(self, rid):
        for q in list(self.pending):
            if q.rid == rid:
                self.pending.remove(q)
                q.status = "cancelled"
                self.done.append(q)
                return True
        for q in self.active:
            if q.rid == rid:
                q.status = "cancelled"  # retired once its in-flight steps complete
                return True
        return False

    # ---- one tick -----------------------------------------------------------
    def tick(self, now):
        # admit in arrival order; a request whose member does not fit waits
        waiting = collections.deque()
        while self.pending:
            req = self.pending.popleft()
            if req.status == "rejected":
                continue
            pts = req.size[0] * req.size[1] * req.size[2]
            cost = self.ex.step_ms(req.size) if self.max_active_ms is not None else 0.0
            if self.active and ((self.max_active is not None and
                                 (waiting or self.active_points + pts > self.max_active)) or
                                (self.max_active_ms is not None and
                                 (waiting or self.active_ms + cost > self.max_active_ms))):
                waiting.append(req)  # no slot: wait, in arrival order
                continue
            if self._admit_member(req):
                self.active_points += pts
                self.active_ms += cost
                req.status = "active"
                req.started = now
                self.busy[req.member] += 1
                self.active.append(req)
            elif req.status == "rejected":
                self.done.append(req)
            else:
                waiting.append(req)
        self.pending = waiting
        # one step per active request per tick; requests on one member run in
        # arrival order (the oldest owns the member until it completes)
        self.tick_no += 1
        if self.rounds and any(r.inflight for r in self.active):
            return  # the previous round is still on the device
        owned = set()
        ready = []
        for req in self.active:
            if req.status != "active" or req.member in owned:
                continue
            owned.add(req.member)
            if req.done_steps + req.inflight >= req.nsteps or req.inflight >= self.max_inflight:
                continue
            ready.append(req)
        if self.max_points is not None:  # least recently served first
            ready.sort(key=lambda q: q.last_tick)
        for req in ready:
            pts = req.size[0] * req.size[1] * req.size[2]
            if (self.max_points is not None and self.inflight_points > 0 and
                    self.inflight_points + pts > self.max_points):
                continue
            self.ex.launch(req, self.clock())
            if req.status == "active":
                req.inflight += 1
                req.last_tick = self.tick_no
                self.inflight_points += pts

    def poll(self):
        for req, t_launch, t_done, pts, lat, dev in self.ex.completed():
            req.inflight -= 1
            req.done_steps += 1
            self.inflight_points -= pts
            if req.status == "cancelled":
                continue
            self.metrics.step_lat.append(lat)
            self.metrics.step_lat_by_size[req.size].append(lat)
            self.metrics.step_dev.append(dev)
            self.metrics.pt_steps += pts
        still = []
        for req in self.active:
            if req.status == "failed":
                self.busy[req.member] -= 1
                self._release(req)
                self.done.append(req)
            elif req.inflight == 0 and (req.done_steps >= req.nsteps or req.status == "cancelled"):
                req.finished = self.clock()
                if req.status != "cancelled":
                    req.status = "done"
                    t_arr = req.arrival_wall if req.arrival_wall is not None else req.started
                    self.metrics.req_lat.append(req.finished - t_arr)
                self.busy[req.member] -= 1
                self._release(req)
                self.done.append(req)
            else:
                still.append(req)
        self.active = still

    def _release(self, req):
        self.active_points -= req.size[0] * req.size[1] * req.size[2]
        if self.max_active_ms is not None:
            self.active_ms = max(0.0, self.active_ms - self.ex.step_ms(req.size))

    def idle(self):
        return not self.pending and not self.active

    def run(self, trace, time_scale=1.0, max_wall=600.0):
        """Replay a trace in real time (arrival times x time_scale)."""
        t0 = self.clock()
        arrivals = sorted(trace, key=lambda r: r.arrival)
        i = 0
        while i < len(arrivals) or not self.idle():
            now = self.clock() - t0
            while i < len(arrivals) and arrivals[i].arrival * time_scale <= now:
                arrivals[i].arrival_wall = t0 + arrivals[i].arrival * time_scale
                self.submit(arrivals[i])
                i += 1
            self.tick(now)
            self.poll()
            if now > max_wall:
                break
            if not self.active and i < len(arrivals):
                dtw = arrivals[i].arrival * time_scale - (self.clock() - t0)
                if dtw > 0:
                    time.sleep(min(dtw, 0.01))
            else:
                self.ex.wait_any(0.0005)
        wall = self.clock() - t0
        return self.metrics.summary(wall), wall


def priority_of(size, lo=32 ** 3, hi=192 * 192 * 128, levels=5):
    """CUDA stream priority of a member: 0 (least urgent) for the smallest
    size, -levels for the largest, by log of the grid points."""
    nx, ny, nz = size
    f = (math.log(nx * ny * nz) - math.log(lo)) / (math.log(hi) - math.log(lo))
    return -int(round(levels * min(1.0, max(0.0, f))))


class FakeExecutor:
    """Deterministic executor for host-side tests: a step of an nx*ny*nz
    member takes `ns_per_pt` ns per grid point; allocation can be made to
    fail; a member can be marked to fail (NaN detected) on its next step."""

    def __init__(self, ns_per_pt=0.1, fail_alloc=(), fail_step=(), clock=None):
        self.ns = ns_per_pt
        self.fail_alloc = set(fail_alloc)
        self.fail_step = set(fail_step)
        self.t = 0.0
        self.inflight = []
        self.loaded = {}
        self.steps = collections.Counter()
        self.stream_end = {}  # member -> end time of its last queued step (one stream per member)

    def footprint(self, size):
        nx, ny, nz = size
        return int(1200 * nx * ny * (nz + 1))

    def step_ms(self, size):
        nx, ny, nz = size
        return self.ns * 1e-6 * nx * ny * nz

    def load(self, member, size):
        if member in self.fail_alloc:
            raise MemoryError("injected allocation failure for member %d" % member)
        self.loaded[member] = size

    def evict(self, member):
        self.loaded.pop(member, None)

    def launch(self, req, t):
        nx, ny, nz = req.size
        if req.member in self.fail_step:
            req.status = "failed"
            req.error = "non-finite state detected"
            return
        dur = self.ns * 1e-9 * nx * ny * nz
        start = max(t, self.stream_end.get(req.member, t))  # behind the member's queued steps
        self.stream_end[req.member] = start + dur
        self.inflight.append((req, start, start + dur, nx * ny * nz, False))
        self.steps[req.member] += 1

    def completed(self):
        out = []
        for (r, a, b, p, f) in self.inflight:
            gap = b - r.prev_done if r.prev_done is not None else b - a
            r.prev_done = b
            out.append((r, a, b, p, gap, b - a))
        self.inflight = []
        return out

    def wait_any(self, dt):
        pass


class GpuExecutor:
    """les_gb300 contexts on the GPU; two CUDA events per launched step (its
    device time); evicted members spilled to pinned host memory."""

    def __init__(self, precision=1, seed0=1000, use_graphs=True, autotune=True, priorities=False):
        import torch  # events on the members' streams, pinned host buffers
        import les_gb300 as lg
        self.torch = torch
        self.lg = lg
        self.precision = precision
        self.seed0 = seed0
        self.use_graphs = use_graphs
        self.autotune = autotune
        # larger members get more urgent streams, so their steps are not
        # starved behind many small members' short kernels
        self.priorities = priorities
        self.ctx = {}
        self.streams = {}
        self.inflight = collections.deque()
        self.spilled = {}      # member -> pinned host image of its whole state
        self.spills = 0
        self.restores = 0
        self.prepared = {}     # member -> (surface, initial state), made before serving
        self.ms = {}           # grid size -> device time of one step (ms), measured at start-up

    def prepare(self, trace, preload_bytes=0):
        """Work that is not the server's, done before the trace starts: each
        member's seeded surface and initial state (what a client would send
        with its first request), and one tuning of the launch shapes per grid
        size (the server's start-up; every later context of that size reuses
        the process-wide table), with one step time measured per size.  With
        preload_bytes > 0 the pool's members are made resident up front, in
        order of first request while their footprints fit, with their step
        graphs captured (les_step_graph_prepare): admitting them later costs
        no allocation or capture on the serving path."""
        lg = self.lg
        for req in trace:
            if req.member in self.prepared:
                continue
            cfg = self.config(req.size)
            surf = lg.patch_surface(cfg, self.seed0 + req.member)
            surf.wt_s[:] = 0.05
            self.prepared[req.member] = (surf, lg.initial_state(cfg, surf, seed=self.seed0 + req.member))
        for size in sorted({r.size for r in trace}):
            cfg = self.config(size)
            surf = lg.patch_surface(cfg, 0)
            surf.wt_s[:] = 0.05
            ctx = lg.Context(cfg, surf)
            if self.autotune:
                ctx.autotune()
            for k, v in lg.initial_state(cfg, surf, seed=1).items():
                ctx.set(k, v)
            st = self.torch.cuda.ExternalStream(ctx.stream())
            step = ctx.step_graph if self.use_graphs else ctx.step
            step(3)
            e0 = self.torch.cuda.Event(enable_timing=True)
            e1 = self.torch.cuda.Event(enable_timing=True)
            e0.record(st)
            step(5)
            e1.record(st)
            e1.synchronize()
            self.ms[size] = e0.elapsed_time(e1) / 5.0
            ctx.close()
        used = 0
        for req in trace:
            if req.member in self.ctx or preload_bytes <= 0:
                continue
            need = self.footprint(req.size)
            if used + need > preload_bytes:
                continue
            self.load(req.member, req.size)
            if self.use_graphs:
                self.ctx[req.member].graph_prepare()
            used += need

    def step_ms(self, size):
        """Device time of one step of a member of this size (measured by
        prepare(); a points-proportional guess before it)."""
        if size in self.ms:
            return self.ms[size]
        nx, ny, nz = size
        return 0.5 + 1e-6 * nx * ny * nz

    def config(self, size):
        nx, ny, nz = size
        return self.lg.make_config(nx, ny, nz, s_flag=1, jt_total0=500, precision=self.precision,
                                   rmsdiv_every=0)

    def footprint(self, size):
        return int(self.lg.estimate_device_bytes(self.config(size)))

    def load(self, member, size):
        if member in self.ctx:  # made resident by prepare()
            return
        lg = self.lg
        cfg = self.config(size)
        prep = self.prepared.get(member)
        if prep is None:
            surf = lg.patch_surface(cfg, self.seed0 + member)
            surf.wt_s[:] = 0.05
            state = None
        else:
            surf, state = prep
        try:
            ctx = lg.Context(cfg, surf)
        except lg.LesError as e:
            if e.code == -3:
                raise MemoryError(str(e))
            raise
        img = self.spilled.pop(member, None)
        if img is not None:  # resume where the member stopped
            ctx.state_restore(img)
            self.restores += 1
        else:
            if state is None:
                state = lg.initial_state(cfg, surf, seed=self.seed0 + member)
            for k, v in state.items():
                ctx.set(k, v)
        if self.autotune:
            ctx.autotune()
        if self.priorities:
            ctx.set_priority(priority_of(size))
        self.ctx[member] = ctx
        self.streams[member] = self.torch.cuda.ExternalStream(ctx.stream())

    def evict(self, member):
        ctx = self.ctx.pop(member, None)
        self.streams.pop(member, None)
        if ctx is not None:
            nb = ctx.state_bytes()
            buf = self.torch.empty(nb, dtype=self.torch.uint8, pin_memory=True).numpy()
            ctx.state_save(buf)
            self.spilled[member] = buf
            self.spills += 1
            ctx.close()

    def launch(self, req, t):
        ctx = self.ctx[req.member]
        st = self.streams[req.member]
        e0 = self.torch.cuda.Event(enable_timing=True)
        e1 = self.torch.cuda.Event(enable_timing=True)
        e0.record(st)
        if self.use_graphs:
            ctx.step_graph(1)
        else:
            ctx.step(1)
        e1.record(st)
        nx, ny, nz = req.size
        self.inflight.append((req, t, e0, e1, nx * ny * nz))

    def completed(self):
        out = []
        now = time.perf_counter()
        keep = collections.deque()
        while self.inflight:
            req, t, e0, e1, pts = self.inflight.popleft()
            if e1.query():
                dev = e0.elapsed_time(e1) / 1e3
                gap = req.prev_done.elapsed_time(e1) / 1e3 if req.prev_done is not None else dev
                req.prev_done = e1
                out.append((req, t, now, pts, gap, dev))
            else:
                keep.append((req, t, e0, e1, pts))
        self.inflight = keep
        return out

    def wait_any(self, dt):
        time.sleep(dt)

    def state(self, member, names=("u", "v", "w", "theta")):
        ctx = self.ctx[member]
        return {k: ctx.get(k) for k in names}
