"""Generates tests/golden/*.npz: oracle (CPU restatement of the reference
step) outputs on small seeded cases (SGS models 5, 2 and 4), used as
regression pins of the oracle by tests/test_golden.py.

  python tests/golden/make_golden.py            # every case
  python tests/golden/make_golden.py NAME ...   # the named cases
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

import les_gb300.config as C  # noqa: E402
from oracle.oracle import Oracle, build  # noqa: E402

CASES = {
    # name: (nx, nz_levels, s_flag, jt_total0, model, steps, surface)
    "neutral_16_jt0": (16, 8, 0, 0, 5, 10, "uniform"),
    "theta_16_dyn": (16, 8, 1, 500, 5, 10, "striped"),
    "theta_24_dyn": (24, 12, 1, 500, 5, 6, "striped"),
    "theta_16_std": (16, 8, 1, 500, 2, 10, "striped"),   # std_dynamic
    "theta_16_ssim": (16, 8, 1, 500, 4, 10, "striped"),  # lagrange_Ssim
}
FIELDS = ["u", "v", "w", "theta", "Cs_opt2", "F_LM", "F_MM", "p", "RHSx", "Nu_t"]


def run(name):
    nx, nzl, s_flag, jt0, model, steps, surf_kind = CASES[name]
    cfg = C.make_config(nx, nx, nzl, s_flag=s_flag, jt_total0=jt0, model=model, rmsdiv_every=1)
    surf = C.striped_surface(cfg) if surf_kind == "striped" else C.uniform_surface(cfg)
    o = Oracle(cfg, surf)
    st = C.initial_state(cfg, surf, seed=99)
    for k, v in st.items():
        o.set(k, v)
    assert o.step(steps) == 0
    out = {k: o.get(k)[..., :nx] for k in FIELDS}
    out["rmsdiv"] = np.array(o.rmsdiv())
    return cfg, out


if __name__ == "__main__":
    build()
    for name in (sys.argv[1:] or CASES):
        cfg, out = run(name)
        np.savez_compressed(os.path.join(HERE, name + ".npz"), **out)
        print(name, {k: v.shape for k, v in out.items()})
