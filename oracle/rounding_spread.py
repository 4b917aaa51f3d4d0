"""TEST INFRASTRUCTURE: the oracle's own sensitivity to floating-point
rounding, used to set the tolerances of the GPU parity tests where the
reference algorithm amplifies rounding differences.

The oracle is built a second time with FMA contraction
(-ffp-contract=fast instead of -ffp-contract=off) into oracle/_build, both
builds run the same seeded configuration, and the relative L2 difference of
each field is printed.  Two cases:

  model3   32^3, theta, striped surface, jt_total0 = 500, model 3, 10 steps:
           the plane-averaged quintic of scaledep_dynamic (sgsmodule.f90:37-59)
           is ill-conditioned.
  humid0, humid500
           32^3, theta and qmix with the striped moisture flux, jt_total0 = 0
           or 500 (the dynamic Cs^2 feeds back from step 5), 10 steps.
  model7   the humid500 case with SGS model 7 (the scalars' Lagrangian
           dynamic Prandtl number Pr_t = Cs_opt2 / Cs2_Pr, both rounded
           through FP32 by the reference) and theta perturbed on every level.
  c2       128^3, theta, striped surface, jt_total from 0, model 5, 200 steps
           (every 10 steps): the first level's explicit SGS diffusion number
           Nu_t dt / dz^2 is above the AB2 stability limit, so from about
           step 55 rounding differences at level 1 grow until they saturate.

  python -m oracle.rounding_spread model3|humid0|humid500|model7|c2
"""
import json
import os
import subprocess
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
FMA_LIB = os.path.join(HERE, "_build", "liblesoracle_fma.so")


def build_fma():
    import platform
    os.makedirs(os.path.join(HERE, "_build"), exist_ok=True)
    # aarch64 has fused multiply-add in its base instruction set; x86-64 needs -mfma
    isa = ["-mfma"] if platform.machine() in ("x86_64", "AMD64") else []
    cmd = ["g++", "-O3", "-std=c++17", "-fPIC", "-fopenmp", "-ffp-contract=fast", "-Wall", "-Wno-unused-variable"] + \
        isa + ["-shared", "-o", FMA_LIB, os.path.join(HERE, "les_oracle.cpp")]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(r.stdout + r.stderr)


def run_case(case, lib_path, out_path):
    sys.path.insert(0, ROOT)
    import oracle.oracle as oo
    import les_gb300.config as lc
    if lib_path:
        oo.LIB = lib_path
    oo.Oracle.set_threads(max(1, oo.Oracle.max_threads()))
    if case == "model3":
        cfg = lc.make_config(32, s_flag=1, jt_total0=500, model=3, rmsdiv_every=1)
        seed, blocks, every = 11, 1, 10
    elif case in ("humid0", "humid500"):
        cfg = lc.make_config(32, s_flag=1, q_flag=1, jt_total0=0 if case == "humid0" else 500, rmsdiv_every=1)
        seed, blocks, every = 41, 1, 10
    elif case == "model7":
        cfg = lc.make_config(32, s_flag=1, q_flag=1, jt_total0=500, model=7, rmsdiv_every=1)
        seed, blocks, every = 41, 1, 10
    else:
        cfg = lc.make_config(128, s_flag=1, rmsdiv_every=10)
        seed, blocks, every = 21, 20, 10
    surf = lc.striped_surface(cfg)
    o = oo.Oracle(cfg, surf)
    if getattr(cfg, "q_flag", 0):
        o.set("wq_s", lc.moisture_flux(cfg))
    levels = {"theta_levels": cfg.nz} if case == "model7" else {}
    for k, v in lc.initial_state(cfg, surf, seed=seed, **levels).items():
        o.set(k, v)
    n = cfg.nx
    out = {}
    for b in range(blocks):
        o.step(every)
        step = (b + 1) * every
        for nm in ("u", "v", "w", "theta", "Cs_opt2") + (("q",) if getattr(cfg, "q_flag", 0) else ()) + \
                (("Pr_t", "G_LM", "G_QN") if cfg.model == 7 else ()):
            out["%s_%d" % (nm, step)] = o.get(nm)[:-1, :, :n]
        out["rmsdiv_%d" % step] = np.array(o.rmsdiv())
    np.savez(out_path, **out)


def main():
    case = sys.argv[1] if len(sys.argv) > 1 else "model3"
    if len(sys.argv) > 3 and sys.argv[2] == "--run":
        run_case(case, sys.argv[3] if sys.argv[3] != "-" else None, sys.argv[4])
        return
    from oracle import oracle as oo
    oo.build()
    build_fma()
    tmp = os.environ.get("TMPDIR", "/tmp")
    paths = {}
    for tag, lib in (("plain", "-"), ("fma", FMA_LIB)):
        paths[tag] = os.path.join(tmp, "les_spread_%s_%s.npz" % (case, tag))
        subprocess.run([sys.executable, "-m", "oracle.rounding_spread", case, "--run", lib, paths[tag]],
                       check=True, cwd=ROOT)
    a, b = np.load(paths["plain"]), np.load(paths["fma"])
    steps = sorted({int(k.split("_")[-1]) for k in a.files})
    for s in steps:
        rec = {"step": s}
        for nm in [f.rsplit("_", 1)[0] for f in a.files if f.endswith("_%d" % s) and not f.startswith("rmsdiv")]:
            x, y = a["%s_%d" % (nm, s)], b["%s_%d" % (nm, s)]
            rec[nm] = float(np.linalg.norm(x - y) / max(np.linalg.norm(x), 1e-300))
        x, y = float(a["rmsdiv_%d" % s]), float(b["rmsdiv_%d" % s])
        rec["rmsdiv"] = abs(x - y) / abs(x)
        print(json.dumps(rec))
    for p in paths.values():
        os.remove(p)


if __name__ == "__main__":
    main()
