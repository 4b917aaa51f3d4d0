"""Benchmark of the per-timestep spectral core (pt-steps/s = Nx*Ny*Nz*steps / s).

  python bench.py [--gpus N] [--steps K] [--warmup W] [--form mixed|fp64|ff]
                  [--impl ours|reference] [--grid 256] [--no-fp64] [--no-e2e] [--no-cpu]
                  [--no-serve]

Workload: 256^3 LES member (box 2pi x 2pi x 1, active theta, x-striped
z0 = 1e-4/1e-2 and surface heat flux 0.05/0.15 K m/s in stripes of width
Nx/8, Lagrangian scale-dependent SGS, dt = 2e-4), seeded synthetic initial
state.  A step is one call of the fused time step (main.f90:202-478) on the
device-resident member; the headline is the FP32-mixed step, with the FP64
step of the same member timed beside it (and the velocity error and rmsdiv
of the mixed state after the same steps).  The line also carries the
served ensemble's p50/p99 step latency (Poisson arrivals over 64 members of
uneven sizes, les_gb300.serve_bench), each transform family's share of the
step and HBM fraction, and the whole-step ledger.  With N > 1 (torchrun) every rank
advances its own independent member: replicas only, no collective.

`--impl reference` times the CPU restatement of the reference step (the
oracle; the Fortran reference has no compiler here) on all host cores on the
same configuration.
"""
import argparse
import ctypes
import json
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "pt-steps/s at 256³: FP32-mixed vs FP64 (≤1e-5 err); p99 ensemble step latency"
PEAKS = os.path.join(ROOT, "MEASURED_PEAKS.json")

# Transform families the profiling hook (les_profile_begin) can bracket; the
# roofline object reports the one with the largest share of the step, found
# by a short untimed pre-pass over all four.
FAMILIES = {1: "k_cols/k_colsf<double|dfloat> (FP64 / float-float y pass)",
            2: "k_colsr/k_colsr_sum/k_colsr_pad/k_colsf<float> (FP32 y pass)",
            3: "k_rows_r2c/k_rows_c2r<double|dfloat> (FP64 / float-float x pass)",
            4: "k_r2c_reg*/k_c2r_reg*/k_rows_*<float> (FP32 x pass)"}
# DRAM bytes (dram__bytes_read.sum + dram__bytes_write.sum) per algorithmic
# byte of a family, from one ncu capture of one step's launches of that
# family on a 256 x 256 x 96 member (bench.py --capture-step;
# profiles/transforms_fp32_traffic.md); scales the live algorithmic bytes
# per launch to the traffic per launch.  Only where a capture exists.
TRAFFIC_RATIO = {("mixed", 4): 0.741, ("mixed", 2): 0.797}


def parse():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=10)  # multiple of cs_count (5)
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--form", default="mixed", choices=["fp64", "mixed", "ff"],
                   help="mixed: FP32-mixed step; fp64: FP64 step; ff: FP64 state with float-float transforms")
    p.add_argument("--model", type=int, default=5, choices=[5, 4, 3, 2],
                   help="SGS model of the FP64 step (5 Lagrangian scale-dependent, 4 scale-invariant, "
                        "3 plane-averaged scale-dependent, 2 standard dynamic)")
    p.add_argument("--impl", default="ours", choices=["ours", "reference"])
    p.add_argument("--grid", type=int, default=256)
    p.add_argument("--levels", type=int, default=None,
                   help="uvp levels (default: the grid size); fewer make small ncu captures")
    p.add_argument("--no-fp64", action="store_true", help="skip the FP64 step timed beside the mixed one")
    p.add_argument("--no-e2e", action="store_true")
    p.add_argument("--no-cpu", action="store_true")
    p.add_argument("--no-serve", action="store_true", help="skip the served-ensemble latency run")
    p.add_argument("--threads", type=int, default=0,
                   help="--impl reference: host threads of the CPU step (0: all)")
    p.add_argument("--serve-requests", type=int, default=200)
    p.add_argument("--capture-step", action="store_true",
                   help="after the warm-up, run one step of --prof-family's transforms bracketed by "
                        "cudaProfilerStart/Stop (for ncu --profile-from-start off) and print its "
                        "launches and algorithmic bytes, then exit")
    p.add_argument("--prof-family", type=int, default=0,
                   help="transform family for the roofline object: 1 FP64/float-float y pass, 2 FP32 y pass, "
                        "3 FP64/float-float x pass, 4 FP32 x pass (default: the largest share of the step)")
    return p.parse_args()


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


def measured_peaks():
    try:
        with open(PEAKS) as f:
            d = json.load(f)
        return d.get("hbm_gbs"), "measured"
    except Exception:
        return 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi clocks and throttle reasons during the timed region."""

    def __init__(self, index=0):
        self.index = index
        self.samples = []
        self.proc = None
        self.thread = None

    def start(self):
        q = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
             "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
             "clocks_event_reasons.sw_power_cap")
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), "--query-gpu=" + q,
                                          "--format=csv,noheader,nounits", "-lms", "100"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except Exception:
            self.proc = None
            return

        def rd():
            for line in self.proc.stdout:
                self.samples.append([x.strip() for x in line.split(",")])
        self.thread = threading.Thread(target=rd, daemon=True)
        self.thread.start()

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        if self.thread:
            self.thread.join(timeout=2)
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for s in self.samples:
            try:
                sm.append(float(s[0]))
                mx.append(float(s[1]))
                for k, nm in enumerate(names):
                    if s[3 + k].lower().startswith("active"):
                        reasons.add(nm)
            except Exception:
                continue
        return {"sm_mhz": float(np.median(sm)) if sm else None,
                "sm_max_mhz": float(max(mx)) if mx else None,
                "reasons": sorted(reasons), "samples": len(sm)}


LEVELS = None  # --levels: uvp levels when not the grid size (small profiling captures)
MODEL = 5  # --model: SGS model of the FP64 step (the mixed form runs model 5)
MODEL_NAME = {5: "lagrangian-sdep", 4: "lagrangian-ssim", 3: "plane-sdep", 2: "std-dynamic"}


PRECISION = {"fp64": 0, "mixed": 1, "ff": 2}


def workload_config(lg, grid, form):
    cfg = lg.make_config(grid, nz_levels=LEVELS, s_flag=1, precision=PRECISION[form],
                         rmsdiv_every=0, model=5 if form == "mixed" else MODEL)
    surf = lg.striped_surface(cfg)
    return cfg, surf


def workload_name(cfg):
    return "les %dx%dx%d theta striped-surface %s" % (cfg.nx, cfg.ny, cfg.nz - 1, MODEL_NAME[cfg.model])


def oracle_build():
    from oracle import oracle as o
    o.build()


def cpu_baseline(lg, grid):
    """Oracle (CPU restatement) timed on the host cores on one step of the
    same workload (bounded sample)."""
    from oracle.oracle import Oracle
    oracle_build()
    cfg, surf = workload_config(lg, grid, "fp64")
    o = Oracle(cfg, surf)
    cores = Oracle.max_threads()
    for k, v in lg.initial_state(cfg, surf, seed=1234).items():
        o.set(k, v)
    o.step(1)  # first (Euler) step, untimed
    t0 = time.perf_counter()
    o.step(1)
    dt = time.perf_counter() - t0
    pts = cfg.nx * cfg.ny * (cfg.nz - 1)
    return {"value": pts / dt, "unit": "pt-steps/s", "cores": cores, "kind": "port",
            "sample": "1 FP64 step of the %dx%dx%d workload after one untimed step (%.2f s), %d threads"
                      % (cfg.nx, cfg.ny, cfg.nz - 1, dt, cores)}


def run_reference(args):
    import les_gb300.config as lg
    rank, world, _ = dist_env()
    if rank != 0:
        return
    from oracle.oracle import Oracle
    oracle_build()
    cfg, surf = workload_config(lg, args.grid, "fp64")
    o = Oracle(cfg, surf)
    cores = args.threads if args.threads > 0 else Oracle.max_threads()
    Oracle.set_threads(cores)
    for k, v in lg.initial_state(cfg, surf, seed=1234).items():
        o.set(k, v)
    for _ in range(max(args.warmup, 0)):
        o.step(1)
    ts = []
    for _ in range(args.steps):
        t0 = time.perf_counter()
        o.step(1)
        ts.append(time.perf_counter() - t0)
    tot = sum(ts)
    pts = cfg.nx * cfg.ny * (cfg.nz - 1)
    val = pts * args.steps / tot
    line = {"metric": METRIC, "value": val, "unit": "pt-steps/s", "n_gpus": args.gpus, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": 1e3 * tot / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded)",
            "impl": "reference",
            "config": {"workload": workload_name(cfg), "grid": [cfg.nx, cfg.ny, cfg.nz - 1], "form": "fp64",
                       "parallelism": "replicas x1"},
            "cpu_baseline": {"value": val, "unit": "pt-steps/s", "cores": cores, "kind": "port",
                             "sample": "%d FP64 steps of the workload on %d host threads (CPU restatement "
                                       "of the reference; no Fortran compiler available)" % (args.steps, cores)},
            "e2e": {"value": val, "unit": "pt-steps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def new_member(lg, grid, form, seed):
    cfg, surf = workload_config(lg, grid, form)
    ctx = lg.Context(cfg, surf)
    for k, v in lg.initial_state(cfg, surf, seed=seed).items():
        ctx.set(k, v)
    return cfg, ctx


def timed_steps(torch, lg, ctx, steps, prof_family=None):
    """Advance `steps` steps; returns (total ms, per-step ms list, profile)."""
    stream = torch.cuda.ExternalStream(ctx.stream())
    ev = [torch.cuda.Event(enable_timing=True) for _ in range(steps + 1)]
    L = lg.lib()
    if prof_family is not None:
        lg.check(L.les_profile_begin(ctx.h, prof_family, 64 * steps))
    ev[0].record(stream)
    for i in range(steps):
        ctx.step(1)
        ev[i + 1].record(stream)
    ev[-1].synchronize()
    prof = None
    if prof_family is not None:
        n, ms, by = ctypes.c_int(), ctypes.c_double(), ctypes.c_double()
        lg.check(L.les_profile_end(ctx.h, ctypes.byref(n), ctypes.byref(ms), ctypes.byref(by)))
        prof = (n.value, ms.value, by.value)
    per = [ev[i].elapsed_time(ev[i + 1]) for i in range(steps)]
    return ev[0].elapsed_time(ev[-1]), per, prof


def e2e_run(torch, lg, ctx, cfg, world, ke=5):
    """End to end through the public API in the resident mode a Fortran
    caller uses (les_register_field once, then per step les_sync_from_host,
    les_step, les_sync_to_host): H2D of the prognostic fields from pinned
    host buffers, one step, D2H of the prognostic fields, ke times."""
    L = lg.lib()
    names = ["u", "v", "w", "theta"]
    host = {}
    for nm in names:
        a = torch.empty(lg.field_shape(cfg, nm), dtype=torch.float64, pin_memory=True).numpy()
        a[...] = ctx.get(nm)
        host[nm] = a
        lg.check(L.les_register_field(ctx.h, lg.FIELD_ID[nm], lg._ptr(a)))
    nbytes = sum(a.nbytes for a in host.values())
    pts = cfg.nx * cfg.ny * (cfg.nz - 1)
    # one untimed round trip: the first transfers from freshly allocated
    # pinned buffers pay their first-use setup
    lg.check(L.les_sync_from_host(ctx.h))
    ctx.step(1)
    lg.check(L.les_sync_to_host(ctx.h))
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(ke):
        lg.check(L.les_sync_from_host(ctx.h))
        ctx.step(1)
        lg.check(L.les_sync_to_host(ctx.h))
    dt = time.perf_counter() - t0
    for nm in names:  # unbind the host arrays
        lg.check(L.les_register_field(ctx.h, lg.FIELD_ID[nm], None))
    return {"value": pts * ke * world / dt, "unit": "pt-steps/s", "h2d_bytes_per_step": nbytes,
            "d2h_bytes_per_step": nbytes, "api": "les_register_field + les_sync_from_host / les_step / "
                                                 "les_sync_to_host"}


def main():
    global LEVELS, MODEL
    args = parse()
    LEVELS = args.levels
    MODEL = args.model
    if args.form == "mixed" and MODEL != 5:
        raise SystemExit("--model: the FP32-mixed form runs model 5; use --form fp64")
    if args.impl == "reference":
        run_reference(args)
        return
    rank, world, local = dist_env()
    import torch
    import les_gb300 as lg
    from les_gb300 import build as b
    from les_gb300.dist import aggregate
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl" if torch.cuda.is_available() else "gloo")
    torch.cuda.set_device(local)
    b.build()
    L = lg.lib()
    L.les_kernel_launch_count.restype = ctypes.c_ulonglong
    cfg, ctx = new_member(lg, args.grid, args.form, 1234 + rank)
    pts = cfg.nx * cfg.ny * (cfg.nz - 1)
    warm = max(args.warmup, 3)
    for _ in range(warm):
        ctx.step(1)
    torch.cuda.synchronize()

    def barrier():
        if world > 1:
            import torch.distributed as dist
            dist.barrier()
    if args.capture_step:
        fam = args.prof_family or 4
        torch.cuda.profiler.start()
        ms_c, _, pr = timed_steps(torch, lg, ctx, 1, prof_family=fam)
        torch.cuda.profiler.stop()
        print(json.dumps({"capture_step": FAMILIES[fam], "family": fam, "launches": pr[0],
                          "algorithmic_bytes": pr[2], "family_ms": pr[1], "step_ms": ms_c,
                          "grid": [cfg.nx, cfg.ny, cfg.nz - 1], "form": args.form}), flush=True)
        ctx.close()
        return
    cflu, visc = ctx.timestep_conditions()
    # share of the step of each transform family (short untimed pre-pass)
    fam_share = {}
    for f in FAMILIES:
        ms_f, _, pr = timed_steps(torch, lg, ctx, 5, prof_family=f)
        if pr[0]:
            fam_share[f] = (pr[1] / ms_f, pr[0] / 5.0, pr[2] / pr[1] / 1e6)
    fam = args.prof_family or max(fam_share, key=lambda f: fam_share[f][0])
    fam_name = FAMILIES[fam]
    torch.cuda.synchronize()
    clocks = ClockSampler(local)
    barrier()
    torch.cuda.synchronize()
    clocks.start()
    n0 = L.les_kernel_launch_count()
    ms, per, prof = timed_steps(torch, lg, ctx, args.steps, prof_family=fam)
    torch.cuda.synchronize()
    launches = int(L.les_kernel_launch_count() - n0)
    ck = clocks.stop()
    barrier()
    ms_max, _, value = aggregate(ms, pts * args.steps, device="cuda")

    hbm, src = measured_peaks()
    n_l, ms_l, bytes_l = prof
    achieved = (bytes_l / n_l) / (ms_l / n_l / 1e3) / 1e9 if n_l else None
    ratio = TRAFFIC_RATIO.get((args.form, fam))
    roofline = {"bound": "hbm", "achieved": achieved, "peak": hbm, "unit": "GB/s",
                "frac": achieved / hbm if achieved else None,
                "traffic": (ratio * bytes_l / n_l) if (ratio and n_l) else None,
                "peak_source": src, "kernel": fam_name, "launches_timed": n_l,
                "avg_launch_us": 1e3 * ms_l / n_l if n_l else None,
                "algorithmic_bytes_per_launch": bytes_l / n_l if n_l else None,
                "share_of_step": ms_l / ms if ms else None}
    families = {FAMILIES[f]: {"share_of_step": v[0], "launches_per_step": v[1], "achieved_gbs": v[2],
                              "frac": v[2] / hbm} for f, v in sorted(fam_share.items())}
    from les_gb300.ledger import bytes_per_point
    bpp = bytes_per_point(args.form)
    ledger = {"bytes_per_point": bpp, "gb_per_step": bpp * pts / 1e9,
              "achieved_gbs": bpp * pts / (ms / args.steps / 1e3) / 1e9,
              "frac": bpp * pts / (ms / args.steps / 1e3) / 1e9 / hbm,
              "definition": "routine-interface ledger (les_gb300/ledger.py) at the form's element sizes"}

    e2e = None
    if not args.no_e2e:
        e2e = e2e_run(torch, lg, ctx, cfg, world)

    compare = None
    if rank == 0 and args.form == "mixed" and not args.no_fp64:
        # the FP64 step of the same member, same warm-up and step count
        ctx.close()
        ctx = None
        cfg_m, ctx_m = new_member(lg, args.grid, "mixed", 1234)
        cfg_d, ctx_d = new_member(lg, args.grid, "fp64", 1234)
        for _ in range(warm):
            ctx_d.step(1)
            ctx_m.step(1)
        torch.cuda.synchronize()
        ms_d, per_d, _ = timed_steps(torch, lg, ctx_d, args.steps)
        ctx_m.step(args.steps)
        err = {}
        for nm in ("u", "v", "w", "theta"):
            a = ctx_m.get(nm)[:-1, :, :cfg.nx]
            d = ctx_d.get(nm)[:-1, :, :cfg.nx]
            err[nm] = float(np.linalg.norm(a - d) / np.linalg.norm(d))
        bpp_d = bytes_per_point("fp64")
        compare = {"fp64_ms_per_step": ms_d / args.steps, "fp64_value": pts * args.steps / (ms_d / 1e3),
                   "mixed_over_fp64": (pts * args.steps / (ms / 1e3)) / (pts * args.steps / (ms_d / 1e3)),
                   "steps_compared": warm + args.steps, "rel_err": err,
                   "rmsdiv_mixed": ctx_m.rmsdiv(), "rmsdiv_fp64": ctx_d.rmsdiv(),
                   "fp64_step_ledger_frac": bpp_d * pts / (ms_d / args.steps / 1e3) / 1e9 / hbm}
        ctx_m.close()
        # the FP64 state with float-float transforms (precision 2), same steps
        cfg_f, ctx_f = new_member(lg, args.grid, "ff", 1234)
        for _ in range(warm):
            ctx_f.step(1)
        torch.cuda.synchronize()
        ms_f, _, _ = timed_steps(torch, lg, ctx_f, args.steps)
        err_f = {}
        for nm in ("u", "v", "w", "theta"):
            a = ctx_f.get(nm)[:-1, :, :cfg.nx]
            d = ctx_d.get(nm)[:-1, :, :cfg.nx]
            err_f[nm] = float(np.linalg.norm(a - d) / np.linalg.norm(d))
        compare["ff"] = {"ms_per_step": ms_f / args.steps, "value": pts * args.steps / (ms_f / 1e3),
                         "over_fp64": ms_d / ms_f, "rel_err_vs_fp64": err_f, "rmsdiv": ctx_f.rmsdiv()}
        if not args.no_e2e:
            compare["ff"]["e2e"] = e2e_run(torch, lg, ctx_f, cfg_f, world)
        ctx_f.close()
        if not args.no_e2e:
            compare["fp64_e2e"] = e2e_run(torch, lg, ctx_d, cfg_d, world)
        ctx_d.close()
    served = None
    if rank == 0 and world == 1 and not args.no_serve:
        try:
            from les_gb300.serve_bench import serve
            served = serve(requests=args.serve_requests, rate=200.0, seed=11, baseline_requests=0)
        except Exception as ex:  # reported, never fatal
            served = {"error": str(ex)[:200]}
    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu:
        try:
            cpu = cpu_baseline(lg, args.grid)
        except Exception as ex:  # reported, never fatal
            cpu = {"value": None, "error": str(ex)[:200]}
    if rank == 0:
        line = {"metric": METRIC, "value": value, "unit": "pt-steps/s", "n_gpus": world, "steps": args.steps,
                "warmup": warm, "ms_per_step": ms_max / args.steps, "higher_is_better": True,
                "scaling": "weak", "vs_baseline": None,
                "dtype": {"fp64": "f64", "ff": "f64 (float-float transforms)"}.get(args.form, "f32/f64-mixed"),
                "data": "synthetic (seeded SplitMix64 initial state, x-striped surface)",
                "config": {"workload": workload_name(cfg), "grid": [cfg.nx, cfg.ny, cfg.nz - 1],
                           "form": args.form, "dt": cfg.dt, "cflu": cflu, "visc_stab": visc,
                           "cflu_note": "CFLu of the seeded state; the reference stops above 0.1 in its "
                                        "every-500-steps check (main.f90:451-458); the in-step check is off "
                                        "(rmsdiv_every = 0)",
                           "l2": "inputs larger than L2 (member state %.1f GB resident)"
                                 % (lg.estimate_device_bytes(cfg) / 1e9),
                           "parallelism": "replicas x%d" % world},
                "step_latency_ms": {"p50": float(np.percentile(per, 50)), "p99": float(np.percentile(per, 99)),
                                    "max": float(max(per))},
                "served_ensemble": served,
                "fp64_comparison": compare,
                "roofline": roofline, "roofline_families": families, "step_ledger": ledger,
                "cpu_baseline": cpu, "e2e": e2e, "clocks": ck,
                "gpu_launches": launches}
        print(json.dumps(line), flush=True)
    if ctx is not None:
        ctx.close()
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
