"""Batched-ensemble measurement: 64 independent members (16 x 32^3,
16 x 64^2x48, 16 x 96^2x64, 16 x 128^3), each with a seeded z0 patch pattern
(patch width from {N/16, N/8, N/4}, z0 log-uniform in [1e-5, 1e-2]) and
seeded initial noise, FP32-mixed step, launch shapes autotuned per grid size,
advanced by one CUDA-graph launch per ensemble step.

  python -m les_gb300.ensemble_bench [--steps 20] [--warmup 11] [--precision 1]
"""
import argparse
import json
import time

import numpy as np


def build(precision, per_size=16, autotune=True):
    import les_gb300 as lg
    shapes = [(32, 32, 32), (64, 64, 48), (96, 96, 64), (128, 128, 128)]
    members, tune = [], {}
    k = 0
    for (nx, ny, nz) in shapes:
        for i in range(per_size):
            cfg = lg.make_config(nx, ny, nz, s_flag=1, jt_total0=500, precision=precision, rmsdiv_every=0)
            surf = lg.patch_surface(cfg, 5000 + k)
            surf.wt_s[:] = 0.05
            ctx = lg.Context(cfg, surf)
            for name, v in lg.initial_state(cfg, surf, seed=5000 + k).items():
                ctx.set(name, v)
            if autotune:
                tune["%dx%dx%d" % (nx, ny, nz)] = ctx.autotune()
            members.append(ctx)
            k += 1
    return members, shapes, tune


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=11)
    ap.add_argument("--precision", type=int, default=1)
    ap.add_argument("--per-size", type=int, default=16)
    args = ap.parse_args()
    import torch
    import les_gb300 as lg
    members, shapes, tune = build(args.precision, args.per_size)
    pts = sum(m.cfg.nx * m.cfg.ny * (m.cfg.nz - 1) for m in members)
    ens = lg.Ensemble(members)
    stream = torch.cuda.ExternalStream(ens.stream())
    ens.step(args.warmup)
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    ens.step(args.steps)
    e1.record(stream)
    e1.synchronize()
    ms = e0.elapsed_time(e1)
    # the same members stepped one after another without graphs (eager, serial)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(5):
        for m in members:
            m.step(1)
            m.synchronize()
    t_eager = (time.perf_counter() - t0) / 5
    out = {"members": len(members), "shapes": shapes, "precision": args.precision,
           "ensemble_ms_per_step": ms / args.steps, "pt_steps_per_s": pts * args.steps / (ms / 1e3),
           "serial_eager_ms_per_step": 1e3 * t_eager, "serial_eager_pt_steps_per_s": pts / t_eager,
           "autotuned": tune}
    print(json.dumps(out))
    ens.close()
    for m in members:
        m.close()


if __name__ == "__main__":
    main()
