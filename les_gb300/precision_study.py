"""Precision study: the FP32-mixed step against the FP64 step on the same
seeded member (active theta, x-striped z0 1e-4/1e-2 and heat flux
0.05/0.15 K m/s), both on the GPU.  Every `--every` steps it reports, per
field, the relative L2 error and the share of the squared error in the
lowest four levels, both forms' rmsdiv, and the largest first-level explicit
SGS diffusion number Nu_t dt / dz^2 of the FP64 member.

With --pert X a third member runs the FP64 step from the same state with
every interior u, v, w value multiplied by (1 + X r), r uniform in [-1, 1]
(X = 1e-15: a perturbation at the size of FP64 rounding), and its difference
from the FP64 member is reported beside the mixed form's: it shows how the
configuration itself amplifies a difference of rounding size.  With --ff the
FP64 state with float-float transforms (precision 2) runs beside them too.

  python -m les_gb300.precision_study [--grid 256] [--steps 500] [--every 50]
                                      [--jt0 0] [--dt 2e-4] [--pert 1e-15] [--ff]
"""
import argparse
import json

import numpy as np


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--grid", type=int, default=256)
    ap.add_argument("--steps", type=int, default=500)
    ap.add_argument("--every", type=int, default=50)
    # jt_total starts at 0 as in a fresh reference run: Cs^2 = 0.16^2 for
    # jt_total < 500 (sgs_stag.f90:166-173) while the Lagrangian averages
    # build up; a cold-started dynamic Cs^2 on the white-noise initial state
    # is unstable at 256^3 (Cs^2 up to 4, explicit SGS diffusion number > 0.2)
    ap.add_argument("--jt0", type=int, default=0)
    ap.add_argument("--dt", type=float, default=2e-4)
    ap.add_argument("--pert", type=float, default=0.0)
    ap.add_argument("--ff", action="store_true", help="also the float-float transform form (precision 2)")
    args = ap.parse_args()
    import les_gb300 as lg
    from les_gb300.config import splitmix64_uniform
    n = args.grid
    forms = [("mixed", 1, 0.0), ("fp64", 0, 0.0)]
    if args.pert > 0:
        forms.append(("fp64_pert", 0, args.pert))
    if args.ff:
        forms.append(("ff", 2, 0.0))
    ctxs = {}
    for name, prec, pert in forms:
        # rmsdiv is read directly (les_rmsdiv) so the reference's CFL stop
        # (main.f90:455-458, CFLu > 0.1) does not end the study
        cfg = lg.make_config(n, s_flag=1, precision=prec, jt_total0=args.jt0, rmsdiv_every=0, dt=args.dt)
        surf = lg.striped_surface(cfg)
        c = lg.Context(cfg, surf)
        st = lg.initial_state(cfg, surf, seed=2024)
        if pert > 0:
            r = splitmix64_uniform(77, 3 * st["u"].size).reshape((3,) + st["u"].shape)
            for q, k in enumerate("uvw"):
                a = st[k]
                a[:-1, :, :n] *= 1.0 + pert * (2.0 * r[q][:-1, :, :n] - 1.0)
        for k, v in st.items():
            c.set(k, v)
        ctxs[name] = c
    dz = 1.0 / n
    done = 0
    while done < args.steps:
        for c in ctxs.values():
            c.step_graph(args.every)
        done += args.every
        rec = {"step": done}
        ref = {nm: ctxs["fp64"].get(nm)[:-1, :, :n] for nm in ("u", "v", "w", "theta", "F_LM")}
        for other in [k for k in ctxs if k != "fp64"]:
            out = {}
            for nm, b in ref.items():
                d = ctxs[other].get(nm)[:-1, :, :n] - b
                lev = (d ** 2).sum(axis=(1, 2))
                out[nm] = {"rel_l2": float(np.linalg.norm(d) / np.linalg.norm(b)),
                           "wall4": float(lev[:4].sum() / max(lev.sum(), 1e-300))}
            out["rmsdiv"] = ctxs[other].rmsdiv()
            rec[other] = out
        rec["rmsdiv_fp64"] = ctxs["fp64"].rmsdiv()
        rec["cflu"], rec["visc_stab"] = ctxs["fp64"].timestep_conditions()
        nut1 = ctxs["fp64"].get("Nu_t")[0, :, :n]
        rec["nut_dt_dz2_level1_max"] = float(nut1.max() * args.dt / dz ** 2)
        print(json.dumps(rec), flush=True)
    for c in ctxs.values():
        c.close()


if __name__ == "__main__":
    main()
