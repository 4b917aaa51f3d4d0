"""The drop-in boundary, entry by entry: every per-routine C-ABI entry point
that the Fortran shim binds (include/les_gb300.h) called on seeded host
arrays against the matching routine of the CPU oracle, FP64 form.

Each case first advances a GPU context and an oracle from the same seeded
32^3 state (a striped surface, active theta), then copies the GPU's module
arrays that the routine reads into the oracle, so both sides see bit-identical
inputs; the routine is then called on both and its outputs compared at the
FP64 parity tolerance of the step.  Reference interfaces: convec.f90:1,
divstress_uv.f90:1, divstress_w.f90:4, press_stag_array.f90:1,
lagrange_Sdep.f90:4, interpolag_Sdep.f90:2, scaledep_dynamic.f90:4,
scalars_module.f90:508 (obukhov), forcing.f90:128 (project), padd.f90:1,
unpadd.f90:1, ddxy.f90:1, ddz_uv.f90:5, ddz_w.f90:6,
test_filtermodule.f90:32 (test_filter_init).

The last case is the resident mode a Fortran caller uses: module arrays
bound once with les_register_field, les_sync_from_host, les_step,
les_sync_to_host.
"""
import ctypes

import numpy as np
import pytest

import les_gb300 as lg

pytestmark = pytest.mark.gpu

TOL = 1e-12   # FP64 parity tolerance of the step (relative L2)


def rel(a, b):
    nb = np.linalg.norm(b)
    return np.linalg.norm(a - b) / (nb if nb > 0 else 1.0)


@pytest.fixture(scope="module")
def libs(gpu_lib, oracle_lib):
    return gpu_lib, oracle_lib


def advanced_pair(n=32, steps=6, model=5):
    """GPU context and oracle advanced `steps` steps from the same state."""
    from oracle.oracle import Oracle
    cfg = lg.make_config(n, s_flag=1, model=model, rmsdiv_every=0)
    surf = lg.striped_surface(cfg)
    g = lg.Context(cfg, surf)
    o = Oracle(cfg, surf)
    for k, v in lg.initial_state(cfg, surf, seed=17).items():
        g.set(k, v)
        o.set(k, v)
    g.step(steps)
    o.step(steps)
    assert g.counters() == o.counters()
    return cfg, g, o


def copy_state(g, o, names):
    """Make the oracle's module arrays bit-identical to the GPU's."""
    for nm in names:
        o.set(nm, g.get(nm))


def inner(cfg, a, levels):
    return a[levels, :, :cfg.nx]


def test_convec(libs):
    cfg, g, o = advanced_pair()
    copy_state(g, o, ["u", "v", "w", "dudy", "dudz", "dvdx", "dvdz", "dwdx", "dwdy"])
    shp = lg.config.field_shape(cfg, "u")
    out_g = [np.zeros(shp) for _ in range(3)]
    out_o = [np.zeros(shp) for _ in range(3)]
    g.call("convec", *out_g)
    o.call("convec", *out_o)
    lev = slice(0, cfg.nz - 1)
    for a, b in zip(out_g, out_o):
        assert rel(inner(cfg, a, lev), inner(cfg, b, lev)) < TOL


@pytest.mark.parametrize("which", ["divstress_uv", "divstress_w"])
def test_divstress(libs, which):
    cfg, g, o = advanced_pair(steps=1)
    shp = lg.config.field_shape(cfg, "u")
    rng = np.random.default_rng(41)
    tx, ty, tz = (rng.standard_normal(shp) for _ in range(3))
    dg, do = np.zeros(shp), np.zeros(shp)
    g.call(which, dg, tx, ty, tz)
    o.call(which, do, tx.copy(), ty.copy(), tz.copy())
    lev = slice(0, cfg.nz - 1) if which == "divstress_uv" else slice(0, cfg.nz)
    assert rel(inner(cfg, dg, lev), inner(cfg, do, lev)) < TOL


def test_press_stag_array(libs):
    cfg, g, o = advanced_pair()
    copy_state(g, o, ["u", "v", "w", "divtz"])
    shp = lg.config.field_shape(cfg, "u")
    pg, po = np.zeros(lg.config.field_shape(cfg, "p")), np.zeros(lg.config.field_shape(cfg, "p"))
    xg, xo, yg, yo = (np.zeros(shp) for _ in range(4))
    assert g.call("press_stag_array", pg, xg, yg) == 0
    assert o.call("press_stag_array", po, xo, yo) == 0
    # p_hat levels 0..nz-1 (the top level is BOGUS), derivatives 1..nz-1
    assert rel(pg[:cfg.nz, :, :cfg.nx], po[:cfg.nz, :, :cfg.nx]) < TOL
    lev = slice(0, cfg.nz - 1)
    assert rel(inner(cfg, xg, lev), inner(cfg, xo, lev)) < TOL
    assert rel(inner(cfg, yg, lev), inner(cfg, yo, lev)) < TOL


LAG_STATE = ["u", "v", "w", "F_LM", "F_MM", "F_QN", "F_NN", "u_lag", "v_lag", "w_lag", "Beta", "Cs_opt2"]
S_NAMES = ["S11", "S12", "S13", "S22", "S23", "S33"]


def test_interpolag_sdep(libs):
    cfg, g, o = advanced_pair(steps=7)   # lag arrays accumulated over two steps since the last update
    copy_state(g, o, LAG_STATE)
    g.call("interpolag_sdep")
    o.call("interpolag_sdep")
    lev = slice(0, cfg.nz - 1)
    for nm in ("F_LM", "F_MM", "F_QN", "F_NN"):
        assert rel(inner(cfg, g.get(nm), lev), inner(cfg, o.get(nm), lev)) < TOL, nm


def test_lagrange_sdep(libs):
    cfg, g, o = advanced_pair(steps=9)
    copy_state(g, o, LAG_STATE + S_NAMES)
    S = [g.get(nm) for nm in S_NAMES]
    g.call("lagrange_sdep", *S)
    o.call("lagrange_sdep")
    lev = slice(0, cfg.nz - 1)
    for nm in ("F_LM", "F_MM", "F_QN", "F_NN", "Beta", "Cs_opt2"):
        a, b = inner(cfg, g.get(nm), lev), inner(cfg, o.get(nm), lev)
        if nm == "Cs_opt2":
            # the reference rounds Cs^2 through FP32 (max(real(..), real(1e-24)));
            # inputs identical to the last bit, so the roundings agree too
            assert rel(a, b) < 1e-7, nm
        else:
            assert rel(a, b) < TOL, nm


def test_scaledep_dynamic(libs):
    cfg, g, o = advanced_pair(steps=4, model=3)
    copy_state(g, o, ["u", "v", "w"] + S_NAMES)
    S = [g.get(nm) for nm in S_NAMES]
    cg, co = np.zeros(cfg.nz), np.zeros(cfg.nz)
    g.call("scaledep_dynamic", cg, *S)
    o.call("scaledep_dynamic", co)
    # Cs^2(z) is a ratio of plane sums of the rtnewt-scaled contractions; the
    # reference algorithm is itself ill-conditioned here (the oracle built
    # with and without FMA contraction differs at this level)
    assert rel(cg[:cfg.nz - 1], co[:cfg.nz - 1]) < 1e-8


def test_obukhov(libs):
    cfg, g, o = advanced_pair(steps=3)
    names = ["u", "v", "theta", "psi_m", "psi_m0", "psi_h", "psi_h0", "sgs_t3"]
    copy_state(g, o, names)
    g.call("obukhov")
    o.call("obukhov")
    for nm in ("ustar_avg", "psi_m", "psi_m0", "psi_h", "psi_h0", "phi_m", "phi_h"):
        assert rel(g.get(nm), o.get(nm)) < TOL, nm


def test_project(libs):
    cfg, g, o = advanced_pair(steps=2)
    copy_state(g, o, ["u", "v", "w", "dpdx", "dpdy", "dpdz"])
    g.call("project")
    o.call("project")
    lev = slice(0, cfg.nz)
    for nm in ("u", "v", "w"):
        assert rel(inner(cfg, g.get(nm), lev), inner(cfg, o.get(nm), lev)) < TOL, nm


def test_padd_unpadd(libs):
    from oracle.oracle import Oracle
    cfg = lg.make_config(32, 32, 4)
    d = lg.dims(cfg)
    g, o = lg.Context(cfg), Oracle(cfg)
    rng = np.random.default_rng(43)
    npl = 3
    small = rng.standard_normal((npl, cfg.ny, d["ld"]))
    big = rng.standard_normal((npl, d["ny2"], d["ld_big"]))
    bg = np.zeros_like(big)
    g.call("padd", bg, small, ints=(npl,))
    for p in range(npl):
        bo = np.zeros_like(big[p])
        o.call("padd", bo, np.ascontiguousarray(small[p]))
        assert np.array_equal(bg[p], bo)
    sg = np.zeros_like(small)
    g.call("unpadd", sg, big, ints=(npl,))
    for p in range(npl):
        so = np.zeros_like(small[p])
        o.call("unpadd", so, np.ascontiguousarray(big[p]))
        # the padding columns ld-1:ld hold the kx = nx/2 column, zeroed by both
        assert np.array_equal(sg[p][:, :2 * (d["lh"])], so[:, :2 * d["lh"]])


def test_ddxy_ddz(libs):
    from oracle.oracle import Oracle
    cfg = lg.make_config(32, 32, 12)
    g, o = lg.Context(cfg), Oracle(cfg)
    shp = lg.config.field_shape(cfg, "u")
    rng = np.random.default_rng(44)
    f = rng.standard_normal(shp)
    ax, ay, bx, by = (np.zeros(shp) for _ in range(4))
    g.call("ddxy", ax, ay, f, ints=(cfg.nz,))
    o.call("ddxy", bx, by, f.copy(), ints=(cfg.nz,))
    assert rel(ax[:, :, :32], bx[:, :, :32]) < TOL
    assert rel(ay[:, :, :32], by[:, :, :32]) < TOL
    for name in ("ddz_uv", "ddz_w"):
        dg, do = np.full(shp, 7.0), np.full(shp, 7.0)   # untouched levels are kept
        g.call(name, dg, f)
        o.call(name, do, f.copy())
        assert rel(dg[:, :, :32], do[:, :, :32]) < TOL, name
        assert np.array_equal(dg[:, :, :32] == 7.0, do[:, :, :32] == 7.0), name


def test_test_filter_init(libs):
    from oracle.oracle import Oracle
    cfg = lg.make_config(48, 48, 8)
    d = lg.dims(cfg)
    g, o = lg.Context(cfg), Oracle(cfg)
    L = lg.lib()
    f = L.les_test_filter_init
    f.restype = ctypes.c_int
    f.argtypes = [ctypes.c_void_p, ctypes.c_double, ctypes.c_void_p]
    for which, alpha in ((0, 2.0), (1, 4.0)):
        G = np.zeros((cfg.ny, d["lh"]))
        assert f(g.h, alpha, G.ctypes.data) == 0
        Go = np.zeros_like(G)
        o.call("filter_G", Go, ints=(which,))
        assert np.array_equal(G, Go), which
        # the filter is the one the context applies: les_test_filter accepts it
        x = np.random.default_rng(45).standard_normal((2, cfg.ny, d["ld"]))
        g.call("test_filter", x, G, ints=(2,))
    # a non-positive width is refused
    assert f(g.h, 0.0, np.zeros((cfg.ny, d["lh"])).ctypes.data) == -1


def test_resident_mode(libs):
    """register -> sync_from_host -> step -> sync_to_host, as the Fortran
    shim drives a device-resident member; bit-identical to the set/get path
    and within the step tolerance of the oracle."""
    from oracle.oracle import Oracle
    cfg = lg.make_config(32, s_flag=1, rmsdiv_every=0)
    surf = lg.striped_surface(cfg)
    st = lg.initial_state(cfg, surf, seed=23)
    L = lg.lib()
    for name in ("les_register_field", "les_sync_from_host", "les_sync_to_host"):
        getattr(L, name).restype = ctypes.c_int
    L.les_register_field.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p]
    L.les_sync_from_host.argtypes = [ctypes.c_void_p]
    L.les_sync_to_host.argtypes = [ctypes.c_void_p]
    res = lg.Context(cfg, surf)
    host = {k: np.ascontiguousarray(v.copy()) for k, v in st.items()}
    for k, a in host.items():
        assert L.les_register_field(res.h, lg.FIELD_ID[k], a.ctypes.data) == 0
    assert L.les_sync_from_host(res.h) == 0
    res.step(4)
    for a in host.values():
        a[...] = -1.0     # sync_to_host must overwrite every registered array
    assert L.les_sync_to_host(res.h) == 0
    ref = lg.Context(cfg, surf)
    orc = Oracle(cfg, surf)
    for k, v in st.items():
        ref.set(k, v)
        orc.set(k, v)
    ref.step(4)
    orc.step(4)
    for k in host:
        assert np.array_equal(host[k], ref.get(k)), k
        assert rel(host[k][:-1, :, :32], orc.get(k)[:-1, :, :32]) < TOL, k
    # the step continues from the synced state: edit u on the host, sync in
    host["u"][3, 5, 7] += 1e-3
    assert L.les_sync_from_host(res.h) == 0
    assert res.get("u")[3, 5, 7] == host["u"][3, 5, 7]
