"""Algorithmic bytes of one time step: the routine-interface ledger.

Each routine of the step reads each of its interface arrays once and writes
each output once; copies (RHS_f = RHS, theta_old) and diagnostics nothing
reads are excluded; a 3/2-grid array counts 2.25 field units.  Totals, in
field units per grid point per step: 152.6 for the velocity step and 74.5
more for the active scalar theta (227.1).  The FP64 form stores every array
in 8 bytes.  The FP32-mixed form stores the arrays listed in
`MIXED_FP32_UNITS` in 4 bytes (the horizontal velocity and theta gradients,
S_ij, Nu_t, tau_ij, the 3/2-grid products and the stress and flux
divergence intermediates) and the rest (u, v, w, theta, the vertical
gradients, RHS, F_*, Cs^2, pressure) in 8.  The ledger is fixed here, not
derived from measured bytes.
"""

# (routine, field units per point per step, of which FP32-held in the mixed form)
ROUTINES = [
    ("filt_da u, v, w (f in/out, df/dx, df/dy out)", 12.0, 6.0),
    ("ddz_uv / ddz_w of u, v, w", 6.0, 0.0),
    ("divstress_uv (tau in, derivatives, divt out)", 20.0, 16.0),
    ("divstress_w", 10.0, 8.0),
    ("convec (u, v, w, 6 derivatives in; cx, cy, cz out)", 12.0, 4.0),
    ("calc_Sij (9 derivatives in, S_ij out)", 15.0, 12.0),
    ("sgs_stag (lag sums, |S|, Nu_t, tau_ij)", 23.0, 13.0),
    ("lagrange_Sdep (/ cs_count)", 3.8, 1.2),
    ("interpolag_Sdep (/ cs_count)", 2.8, 0.0),
    ("press_stag_array", 6.0, 0.0),
    ("tridag_array", 5.0, 0.0),
    ("RHS, AB2 predictor, grad p", 33.0, 0.0),
    ("project", 9.0, 0.0),
]
VELOCITY_UNITS = 152.6
THETA_UNITS = 74.5
THETA_FP32_UNITS = 37.0  # dealias1 3/2-grid outputs, dT/dx, dT/dy, SGS fluxes

_RAW = sum(r[1] for r in ROUTINES)
_SCALE = VELOCITY_UNITS / _RAW  # the rows above restate the velocity total to within 3 %
MIXED_FP32_UNITS = sum(r[2] for r in ROUTINES) * _SCALE


def bytes_per_point(form, theta=True):
    """Algorithmic bytes per grid point per step ("fp64", "ff" or "mixed";
    the float-float transform form stores every array in 8 bytes like FP64)."""
    units = VELOCITY_UNITS + (THETA_UNITS if theta else 0.0)
    if form in ("fp64", "ff"):
        return 8.0 * units
    f32 = MIXED_FP32_UNITS + (THETA_FP32_UNITS if theta else 0.0)
    return 8.0 * (units - f32) + 4.0 * f32


def step_bytes(form, nx, ny, nz_levels, theta=True):
    return bytes_per_point(form, theta) * nx * ny * nz_levels
