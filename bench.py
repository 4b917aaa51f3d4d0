"""Benchmark of the per-timestep spectral core (pt-steps/s = Nx*Ny*Nz*steps / s).

  python bench.py [--gpus N] [--steps K] [--warmup W] [--form fp64|mixed]
                  [--impl ours|reference] [--grid 256]

Workload: the 256^3 member of the precision study (box 2pi x 2pi x 1, active
theta, x-striped z0 = 1e-4/1e-2 and surface heat flux 0.05/0.15 K m/s,
Lagrangian scale-dependent SGS, dt = 2e-4), seeded synthetic initial state.
A step is one call of the fused time step (main.f90:202-478) on the
device-resident member.  With N > 1 (torchrun) every rank advances its own
independent member: replicas only, no collective (weak scaling).

`--impl reference` times the CPU restatement of the reference step (the
oracle; the Fortran reference has no compiler here) on all host cores on the
same configuration.
"""
import argparse
import json
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

PEAKS = os.path.join(ROOT, "MEASURED_PEAKS.json")
FP64_PEAK_TFLOPS = 1.197  # measured FP64 FMA rate on this machine's GB300 (profiles/)

# Algorithmic bytes per grid point per step: the routine I/O ledger (each
# routine reads each interface array once and writes each output once;
# padded 3/2 arrays count x2.25).  Velocity only 152.6 field units, velocity
# plus theta 227 units; 8 B (FP64) per unit.
LEDGER_UNITS = {0: 152.6, 1: 227.0}


def parse():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=10)  # multiple of cs_count (5)
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--form", default="fp64", choices=["fp64", "mixed"])
    p.add_argument("--impl", default="ours", choices=["ours", "reference"])
    p.add_argument("--grid", type=int, default=256)
    p.add_argument("--no-e2e", action="store_true")
    p.add_argument("--no-cpu", action="store_true")
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
                sm.append(float(s[0])); mx.append(float(s[1]))
                for k, nm in enumerate(names):
                    if s[3 + k].lower().startswith("active"):
                        reasons.add(nm)
            except Exception:
                continue
        return {"sm_mhz": float(np.median(sm)) if sm else None,
                "sm_max_mhz": float(max(mx)) if mx else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def workload_config(args, lg):
    precision = 1 if args.form == "mixed" else 0
    cfg = lg.make_config(args.grid, s_flag=1, precision=precision, rmsdiv_every=0)
    surf = lg.striped_surface(cfg)
    return cfg, surf


def cpu_baseline(args, lg, rank):
    """Oracle (CPU restatement) timed on the host cores on one step of the
    same workload (bounded sample)."""
    from oracle.oracle import Oracle
    oracle_build()
    cfg, surf = workload_config(args, lg)
    cfg.precision = 0
    o = Oracle(cfg, surf)
    cores = Oracle.max_threads()
    st = lg.initial_state(cfg, surf, seed=1234)
    for k, v in st.items():
        o.set(k, v)
    o.step(1)  # first (Euler) step, untimed
    t0 = time.perf_counter()
    o.step(1)
    dt = time.perf_counter() - t0
    pts = cfg.nx * cfg.ny * (cfg.nz - 1)
    return {"value": pts / dt, "unit": "pt-steps/s", "cores": cores, "kind": "port",
            "sample": "1 FP64 step of the %dx%dx%d workload after one untimed step (%.2f s)"
                      % (cfg.nx, cfg.ny, cfg.nz - 1, dt)}


def oracle_build():
    from oracle import oracle as o
    o.build()


def run_reference(args):
    import les_gb300.config as cfgmod
    rank, world, _ = dist_env()
    if rank != 0:
        return
    from oracle.oracle import Oracle
    oracle_build()

    class LG:  # config helpers only
        make_config = staticmethod(cfgmod.make_config)
        striped_surface = staticmethod(cfgmod.striped_surface)
        initial_state = staticmethod(cfgmod.initial_state)
    cfg, surf = workload_config(args, LG)
    cfg.precision = 0
    o = Oracle(cfg, surf)
    cores = Oracle.max_threads()
    st = cfgmod.initial_state(cfg, surf, seed=1234)
    for k, v in st.items():
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
    line = {"metric": "pt-steps/s at %d^3 (%s step)" % (args.grid, "FP64"), "value": val,
            "unit": "pt-steps/s", "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": 1e3 * tot / args.steps, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded)", "impl": "reference",
            "config": {"workload": "les %dx%dx%d theta striped-surface lagrangian-sdep" % (cfg.nx, cfg.ny, cfg.nz - 1),
                       "grid": [cfg.nx, cfg.ny, cfg.nz - 1], "form": "fp64"},
            "cpu_baseline": {"value": val, "unit": "pt-steps/s", "cores": cores, "kind": "port",
                             "sample": "%d FP64 steps of the workload on %d host threads (CPU restatement "
                                       "of the reference; no Fortran compiler available)" % (args.steps, cores)},
            "e2e": {"value": val, "unit": "pt-steps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def main():
    args = parse()
    if args.impl == "reference":
        run_reference(args)
        return
    rank, world, local = dist_env()
    import torch
    import les_gb300 as lg
    from les_gb300 import build as b
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl" if torch.cuda.is_available() else "gloo")
    torch.cuda.set_device(local)
    b.build()
    cfg, surf = workload_config(args, lg)
    ctx = lg.Context(cfg, surf)
    st = lg.initial_state(cfg, surf, seed=1234 + rank)
    for k, v in st.items():
        ctx.set(k, v)
    stream = torch.cuda.ExternalStream(ctx.stream())
    pts = cfg.nx * cfg.ny * (cfg.nz - 1)
    for _ in range(max(args.warmup, 3)):
        ctx.step(1)
    torch.cuda.synchronize()

    def barrier():
        if world > 1:
            import torch.distributed as dist
            dist.barrier()
    clocks = ClockSampler(local)
    barrier()
    torch.cuda.synchronize()
    clocks.start()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    lib = lg.lib()
    lib.les_kernel_launch_count.restype = __import__("ctypes").c_ulonglong
    n0 = lib.les_kernel_launch_count()
    e0.record(stream)
    for _ in range(args.steps):
        ctx.step(1)
    e1.record(stream)
    e1.synchronize()
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1)
    ck = clocks.stop()
    launches = int(lib.les_kernel_launch_count() - n0)
    barrier()
    from les_gb300.dist import aggregate
    ms_max, _, value = aggregate(ms, pts * args.steps, device="cuda")

    # per-step kernel profile (dominant kernel = the whole step here: HBM ledger)
    hbm, src = measured_peaks()
    units = LEDGER_UNITS[1]
    bytes_per_step = units * 8.0 * pts
    achieved = bytes_per_step / (ms_max / args.steps / 1e3) / 1e9
    roofline = {"bound": "hbm", "achieved": achieved, "peak": hbm, "unit": "GB/s",
                "frac": achieved / hbm, "traffic": None, "peak_source": src,
                "scope": "whole step, algorithmic ledger bytes (227 FP64 field units per point)"}

    # e2e through the public API with pinned host buffers: H2D of the
    # prognostic fields, one step, D2H of the prognostic fields
    e2e = None
    if not args.no_e2e:
        names = ["u", "v", "w", "theta"]
        host = {}
        for nm in names:
            a = torch.empty(lg.field_shape(cfg, nm), dtype=torch.float64, pin_memory=True).numpy()
            a[...] = ctx.get(nm)
            host[nm] = a
        nbytes = sum(a.nbytes for a in host.values())
        ke = 5
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for _ in range(ke):
            for nm in names:
                lg.check(ctx.L.les_set_field(ctx.h, lg.FIELD_ID[nm], lg._ptr(host[nm])))
            ctx.step(1)
            for nm in names:
                lg.check(ctx.L.les_get_field(ctx.h, lg.FIELD_ID[nm], lg._ptr(host[nm])))
        dt = time.perf_counter() - t0
        e2e = {"value": pts * ke * world / dt, "unit": "pt-steps/s", "h2d_bytes_per_step": nbytes,
               "d2h_bytes_per_step": nbytes}
    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu:
        try:
            cpu = cpu_baseline(args, lg, rank)
        except Exception as ex:  # reported, never fatal
            cpu = {"value": None, "error": str(ex)[:200]}
    if rank == 0:
        line = {"metric": "pt-steps/s at %d^3 (%s step)" % (args.grid, "FP32-mixed" if args.form == "mixed" else "FP64"),
                "value": value, "unit": "pt-steps/s", "n_gpus": world, "steps": args.steps,
                "warmup": max(args.warmup, 3), "ms_per_step": ms_max / args.steps, "higher_is_better": True,
                "scaling": "weak", "vs_baseline": None,
                "dtype": "f64" if args.form == "fp64" else "f32/f64-mixed",
                "data": "synthetic (seeded SplitMix64 initial state, x-striped surface)",
                "config": {"workload": "les %dx%dx%d theta striped-surface lagrangian-sdep" % (cfg.nx, cfg.ny, cfg.nz - 1),
                           "grid": [cfg.nx, cfg.ny, cfg.nz - 1], "form": args.form, "dt": cfg.dt,
                           "l2": "inputs larger than L2 (state %.1f GB resident)" % (ctx.device_bytes() / 1e9),
                           "parallelism": "replicas x%d" % world},
                "roofline": roofline, "cpu_baseline": cpu, "e2e": e2e, "clocks": ck,
                "gpu_launches": launches}
        print(json.dumps(line), flush=True)
    ctx.close()
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
