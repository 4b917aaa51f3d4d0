"""Run configuration and seeded synthetic inputs.

``LesConfig`` is the ctypes mirror of ``les_config`` in include/les_gb300.h,
which restates the compile-time parameters of the reference's param.f90
(grid :56, model :115, S_FLAG :158, cs_count :100) and its run-time namelist
param_nml (param.f90:183-190) as per-context run-time values.

The reference builds its initial state from a restart file or ran3 noise
(initial.f90:265-502); the workloads here are seeded synthetic states with
the same structure: a log-law mean wind u(z) = ln(z/z0)/kappa on the uvp
nodes, uniform noise, w = 0 at the walls, top values copied from the level
below (initial.f90:412-425).  Random numbers come from SplitMix64 so the
inputs are identical on every host and numpy version.
"""
import ctypes
import math
from dataclasses import dataclass

import numpy as np


class LesConfig(ctypes.Structure):
    _fields_ = [
        ("nx", ctypes.c_int), ("ny", ctypes.c_int), ("nz", ctypes.c_int),
        ("model", ctypes.c_int), ("s_flag", ctypes.c_int),
        ("initu", ctypes.c_int), ("initsc", ctypes.c_int),
        ("cs_count", ctypes.c_int), ("jt_total0", ctypes.c_int),
        ("precision", ctypes.c_int), ("rmsdiv_every", ctypes.c_int),
        ("q_flag", ctypes.c_int),
        ("l_x", ctypes.c_double), ("l_y", ctypes.c_double),
        ("lz_over_zi", ctypes.c_double), ("z_i", ctypes.c_double),
        ("u_star", ctypes.c_double), ("dt", ctypes.c_double),
        ("vonk", ctypes.c_double), ("t_scale", ctypes.c_double),
        ("dtdz_top", ctypes.c_double), ("pr", ctypes.c_double),
        ("g", ctypes.c_double),
        ("q_scale", ctypes.c_double), ("dqdz_top", ctypes.c_double),
    ]


# les_field enumeration (include/les_gb300.h)
FIELDS = [
    "u", "v", "w", "theta",
    "dudx", "dudy", "dudz", "dvdx", "dvdy", "dvdz", "dwdx", "dwdy", "dwdz",
    "RHSx", "RHSy", "RHSz", "RHSx_f", "RHSy_f", "RHSz_f",
    "dpdx", "dpdy", "dpdz",
    "txx", "txy", "tyy", "txz", "tyz", "tzz",
    "divtx", "divty", "divtz",
    "p",
    "F_LM", "F_MM", "F_QN", "F_NN", "Beta", "Cs_opt2", "Nu_t",
    "u_lag", "v_lag", "w_lag",
    "RHS_T", "RHS_Tf", "beta_scal", "dTdx", "dTdy", "dTdz",
    "S11", "S12", "S13", "S22", "S23", "S33",
    "q", "RHS_q", "RHS_qf", "dqdx", "dqdy", "dqdz",
    "G_LM", "G_MM", "G_QN", "G_NN", "Pr_t", "u_lag_s", "v_lag_s", "w_lag_s", "TnLMMM", "TnQNNN",
    "zo", "wt_s", "ustar_avg", "phi_m", "psi_m", "psi_m0",
    "phi_h", "psi_h", "psi_h0", "sgs_t3", "wq_s", "sgs_q3",
]
FIELD_ID = {n: i for i, n in enumerate(FIELDS)}
SURFACE_FIELDS = set(FIELDS[FIELDS.index("zo"):])
# humidity arrays, stored only with q_flag = 1
Q_FIELDS = {"q", "RHS_q", "RHS_qf", "dqdx", "dqdy", "dqdz", "wq_s", "sgs_q3"}
# model 7 arrays, stored only with model = 7
M7_FIELDS = {"G_LM", "G_MM", "G_QN", "G_NN", "Pr_t", "u_lag_s", "v_lag_s", "w_lag_s", "TnLMMM", "TnQNNN"}


def make_config(nx, ny=None, nz_levels=None, *, model=5, s_flag=0, jt_total0=0,
                precision=0, dt=2e-4, vonk=0.4, cs_count=5, rmsdiv_every=500,
                t_scale=400.0, dtdz_top=0.005, initu=0, initsc=0, q_flag=0, q_scale=100.0,
                dqdz_top=-0.004):
    """Config for an nx x ny x nz_levels grid on the 2pi x 2pi x 1 box.

    ``nz_levels`` is the number of uvp levels; the Fortran extent is +1."""
    ny = nx if ny is None else ny
    nzl = nx if nz_levels is None else nz_levels
    c = LesConfig()
    c.nx, c.ny, c.nz = nx, ny, nzl + 1
    c.model, c.s_flag = model, s_flag
    c.initu, c.initsc = initu, initsc
    c.cs_count, c.jt_total0 = cs_count, jt_total0
    c.precision, c.rmsdiv_every = precision, rmsdiv_every
    c.l_x = 2.0 * 3.1415926535897932384626433
    c.l_y = 2.0 * 3.1415926535897932384626433
    c.lz_over_zi, c.z_i = 1.0, 1000.0
    c.u_star, c.dt, c.vonk = 1.0, dt, vonk
    c.t_scale, c.dtdz_top, c.pr, c.g = t_scale, dtdz_top, 0.55, 9.81
    c.q_flag, c.q_scale, c.dqdz_top = q_flag, q_scale, dqdz_top
    return c


def dims(cfg):
    nx, ny, nz = cfg.nx, cfg.ny, cfg.nz
    ld = nx + 2
    return dict(nx=nx, ny=ny, nz=nz, ld=ld, lh=nx // 2 + 1, nx2=3 * nx // 2,
                ny2=3 * ny // 2, ld_big=3 * nx // 2 + 2, lh_big=3 * nx // 4 + 1)


def field_shape(cfg, name):
    """numpy shape (C order, i.e. reversed Fortran order) of a module array."""
    d = dims(cfg)
    if name in SURFACE_FIELDS:
        return (d["ny"], d["nx"])
    if name == "p":
        return (d["nz"] + 1, d["ny"], d["ld"])
    return (d["nz"], d["ny"], d["ld"])


# ---- SplitMix64 ------------------------------------------------------------
_M64 = (1 << 64) - 1


def splitmix64_uniform(seed, n):
    """n uniform doubles in [0,1) from SplitMix64 (counter-based, seeded)."""
    with np.errstate(over="ignore"):
        idx = np.arange(1, n + 1, dtype=np.uint64)
        z = np.uint64(seed & _M64) + idx * np.uint64(0x9E3779B97F4A7C15)
        z = (z ^ (z >> np.uint64(30))) * np.uint64(0xBF58476D1CE4E5B9)
        z = (z ^ (z >> np.uint64(27))) * np.uint64(0x94D049BB133111EB)
        z = z ^ (z >> np.uint64(31))
    return (z >> np.uint64(11)).astype(np.float64) * (1.0 / 9007199254740992.0)


@dataclass
class Surface:
    zo: np.ndarray      # (ny, nx) nondimensional roughness
    wt_s: np.ndarray    # (ny, nx) kinematic heat flux [K m/s]


def uniform_surface(cfg, z0=1e-4, wt=0.0):
    return Surface(np.full((cfg.ny, cfg.nx), z0), np.full((cfg.ny, cfg.nx), wt))


def striped_surface(cfg, z0=(1e-4, 1e-2), wt=(0.05, 0.15), width=None):
    """x-stripes of width nx/8 alternating z0 and surface heat flux."""
    width = cfg.nx // 8 if width is None else width
    jx = np.arange(cfg.nx)
    sel = (jx // width) % 2
    zo = np.where(sel == 0, z0[0], z0[1])[None, :].repeat(cfg.ny, 0)
    ws = np.where(sel == 0, wt[0], wt[1])[None, :].repeat(cfg.ny, 0)
    return Surface(np.ascontiguousarray(zo), np.ascontiguousarray(ws))


def patch_surface(cfg, seed):
    """Seeded patch pattern: patch width from {N/16, N/8, N/4}, z0 log-uniform
    in [1e-5, 1e-2] per patch (ensemble members)."""
    r = splitmix64_uniform(seed, 3 + 4096)
    width = [cfg.nx // 16, cfg.nx // 8, cfg.nx // 4][min(int(r[0] * 3), 2)]
    width = max(width, 1)
    npx = (cfg.nx + width - 1) // width
    npy = (cfg.ny + width - 1) // width
    lz = np.log(1e-5) + r[3:3 + npx * npy] * (np.log(1e-2) - np.log(1e-5))
    z = np.exp(lz).reshape(npy, npx)
    jy, jx = np.meshgrid(np.arange(cfg.ny) // width, np.arange(cfg.nx) // width, indexing="ij")
    return Surface(np.ascontiguousarray(z[jy, jx]), np.zeros((cfg.ny, cfg.nx)))


def initial_state(cfg, surface, seed=1234, noise=0.1, theta_k=300.0, theta_noise=0.1,
                  theta_levels=10):
    """Seeded initial u, v, w (and theta) in the reference's layout."""
    d = dims(cfg)
    nx, ny, nz, ld = d["nx"], d["ny"], d["nz"], d["ld"]
    dz = cfg.lz_over_zi / (nz - 1)
    z = (np.arange(1, nz + 1) - 0.5) * dz
    z0m = float(np.mean(surface.zo))
    ubar = (1.0 / cfg.vonk) * np.log(z / z0m)
    n = nz * ny * nx
    r = splitmix64_uniform(seed, 4 * n).reshape(4, nz, ny, nx)
    u = np.zeros((nz, ny, ld)); v = np.zeros((nz, ny, ld)); w = np.zeros((nz, ny, ld))
    th = np.zeros((nz, ny, ld))
    u[:, :, :nx] = ubar[:, None, None] + noise * (2.0 * r[0] - 1.0)
    v[:, :, :nx] = noise * (2.0 * r[1] - 1.0)
    w[:, :, :nx] = noise * (2.0 * r[2] - 1.0)
    w[0] = 0.0
    w[nz - 1] = 0.0
    u[nz - 1] = u[nz - 2]
    v[nz - 1] = v[nz - 2]
    if cfg.s_flag:
        th[:, :, :nx] = theta_k / cfg.t_scale
        k = min(theta_levels, nz - 1)
        th[:k, :, :nx] += theta_noise * (2.0 * r[3, :k] - 1.0) / cfg.t_scale
        th[nz - 1] = th[nz - 2]
    out = {"u": u, "v": v, "w": w, "theta": th}
    if getattr(cfg, "q_flag", 0):
        # humidity: 10 g/kg with a seeded +-0.2 g/kg perturbation in the lowest
        # levels (nondimensional qmix = q / q_scale)
        q = np.zeros((nz, ny, ld))
        rq = splitmix64_uniform(seed + 7, n).reshape(nz, ny, nx)
        q[:, :, :nx] = 10.0 / cfg.q_scale
        k = min(theta_levels, nz - 1)
        q[:k, :, :nx] += 0.2 * (2.0 * rq[:k] - 1.0) / cfg.q_scale
        q[nz - 1] = q[nz - 2]
        out["q"] = q
    return out


def moisture_flux(cfg, wq=(0.02, 0.06), width=None):
    """x-striped kinematic surface moisture flux [g/kg m/s] on the stripes of
    striped_surface (width nx/8), for the wq_s plane of q_flag = 1."""
    width = cfg.nx // 8 if width is None else width
    sel = (np.arange(cfg.nx) // width) % 2
    return np.ascontiguousarray(np.where(sel == 0, wq[0], wq[1])[None, :].repeat(cfg.ny, 0).astype(np.float64))


# Named workloads (one per configuration of the benchmark definition).
def workload(name):
    """Return (config, surface-builder) for a named workload:
    neutral_32 (32^3 FP64, uniform z0 = 1e-4, no scalar), theta_striped_128
    (128^3 FP64, theta, x-striped z0 and heat flux) and theta_striped_256_mixed
    (256^3, the same surface, FP32-mixed)."""
    if name == "neutral_32":
        return make_config(32), lambda c: uniform_surface(c, 1e-4, 0.0)
    if name == "theta_striped_128":
        return make_config(128, s_flag=1), lambda c: striped_surface(c)
    if name == "theta_striped_256_mixed":
        return make_config(256, s_flag=1, precision=1), lambda c: striped_surface(c)
    raise KeyError(name)
