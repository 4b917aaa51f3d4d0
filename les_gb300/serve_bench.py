"""Serving measurement: Poisson arrivals (mean 200/s) of 'advance N steps'
requests (N ~ U{1..50}) over a pool of 64 members with sizes drawn from
{32^3, 64^3, 96^2x64, 128^3, 192^2x128} (weights 0.3/0.3/0.2/0.15/0.05),
FP32-mixed steps replayed from CUDA graphs, admission by estimated footprint
against free device memory, then to a slot while the active requests' summed
step times stay within 24 ms; the active requests step in lock-step rounds.  Before the trace starts the members' seeded
surfaces and initial states are generated (the client's side of a request)
and the launch shapes are tuned once per grid size (the server's start-up);
admitting a member is then its allocation, upload and graph capture.  Reports p50/p99 step and request latency and
aggregate pt-steps/s, beside an unbatched FP64 baseline (the same requests
served one at a time, eager FP64 steps).

  python -m les_gb300.serve_bench [--requests 200] [--rate 200]
"""
import argparse
import json
import time


def serve(requests=200, rate=200.0, seed=11, budget_gb=0.0, baseline_requests=60, priorities=False,
          max_inflight_points=None, steps_in_flight=1, max_active_points=None, max_active_ms=24.0,
          preload=True, rounds=True):
    """Serve one Poisson trace; returns the summary (and, when
    baseline_requests > 0, the unbatched FP64 baseline on its prefix)."""
    import torch
    from les_gb300.serve import GpuExecutor, Scheduler, poisson_trace
    free, total = torch.cuda.mem_get_info()
    budget = int(budget_gb * 2 ** 30) if budget_gb > 0 else int(0.9 * free)
    trace = poisson_trace(requests, rate, seed)
    ex = GpuExecutor(precision=1, autotune=True, priorities=priorities)
    # members' seeded states, the per-size tuning and, within the budget, the
    # resident pool with its captured step graphs: before the clock starts
    ex.prepare(trace, preload_bytes=budget if preload else 0)
    sched = Scheduler(ex, budget_bytes=budget, max_inflight_per_member=steps_in_flight,
                      max_inflight_points=max_inflight_points, max_active_points=max_active_points,
                      max_active_ms=max_active_ms, rounds=rounds)
    summary, wall = sched.run(trace)
    status = {}
    for r in sched.done:
        status[r.status] = status.get(r.status, 0) + 1
    for m in list(ex.ctx):
        ex.evict(m)
    out = {"requests": len(trace), "rate_per_s": rate, "priorities": priorities,
           "max_inflight_points": max_inflight_points, "steps_in_flight": steps_in_flight,
           "max_active_points": max_active_points, "max_active_ms": max_active_ms, "preload": preload, "rounds": rounds,
           "step_ms_by_size": {"%dx%dx%d" % k: v for k, v in sorted(ex.ms.items())},
           "wall_s": wall, "status": status,
           "budget_gb": budget / 2 ** 30, "serving": summary}
    if summary.get("step_p50_ms"):
        out["step_p99_over_p50"] = summary["step_p99_ms"] / summary["step_p50_ms"]
    if baseline_requests > 0:
        # unbatched FP64 baseline on a prefix of the same trace
        base = GpuExecutor(precision=0, autotune=False, use_graphs=False)
        nb = min(baseline_requests, len(trace))
        pts = 0
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for r in trace[:nb]:
            if r.member not in base.ctx:
                base.load(r.member, r.size)
            base.ctx[r.member].step(r.nsteps)
            base.ctx[r.member].synchronize()
            nx, ny, nz = r.size
            pts += nx * ny * nz * r.nsteps
        tb = time.perf_counter() - t0
        for m in list(base.ctx):
            base.evict(m)
        out["fp64_unbatched_pt_steps_per_s"] = pts / tb
        out["fp64_unbatched_requests"] = nb
        out["speedup_vs_fp64_unbatched"] = summary["pt_steps_per_s"] / out["fp64_unbatched_pt_steps_per_s"]
    return out


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--requests", type=int, default=200)
    ap.add_argument("--rate", type=float, default=200.0)
    ap.add_argument("--seed", type=int, default=11)
    ap.add_argument("--budget-gb", type=float, default=0.0, help="0: 90%% of free device memory")
    ap.add_argument("--baseline-requests", type=int, default=60)
    ap.add_argument("--priorities", action="store_true", help="more urgent streams for larger members")
    ap.add_argument("--max-inflight-points", type=float, default=0.0,
                    help="grid points of all steps in flight at once (0: no limit)")
    ap.add_argument("--steps-in-flight", type=int, default=1,
                    help="steps of one request queued on its member's stream at once")
    ap.add_argument("--max-active-points", type=float, default=0.0,
                    help="grid points of the active requests (slots; 0: no limit)")
    ap.add_argument("--max-active-ms", type=float, default=24.0,
                    help="summed step times of the active requests, ms (slots; 0: no limit)")
    ap.add_argument("--no-rounds", action="store_true",
                    help="relaunch each request as its step completes instead of lock-step rounds")
    ap.add_argument("--no-preload", action="store_true",
                    help="admit members on their first request (allocation and graph capture on the path)")
    args = ap.parse_args()
    mip = int(args.max_inflight_points) if args.max_inflight_points > 0 else None
    map_ = int(args.max_active_points) if args.max_active_points > 0 else None
    print(json.dumps(serve(args.requests, args.rate, args.seed, args.budget_gb, args.baseline_requests,
                           priorities=args.priorities, max_inflight_points=mip,
                           steps_in_flight=args.steps_in_flight, max_active_points=map_,
                           max_active_ms=args.max_active_ms if args.max_active_ms > 0 else None,
                           preload=not args.no_preload, rounds=not args.no_rounds)))


if __name__ == "__main__":
    main()
