"""TEST INFRASTRUCTURE: ctypes binding of the CPU oracle library.

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline and
reference legs use this module, as the checker or the timed CPU baseline.
"""
import ctypes
import os
import subprocess

import numpy as np

from les_gb300.config import FIELD_ID, field_shape, dims

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "_build", "liblesoracle.so")


def build(quiet=True):
    r = subprocess.run(["make", "-C", HERE], capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("oracle build failed:\n" + r.stdout + r.stderr)
    return LIB


_lib = None


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB):
            build()
        L = ctypes.CDLL(LIB)
        vp, dp, ip = ctypes.c_void_p, ctypes.POINTER(ctypes.c_double), ctypes.c_int
        L.lo_create.restype = vp
        L.lo_field.restype = dp
        L.lo_field.argtypes = [vp, ip, ctypes.POINTER(ctypes.c_long)]
        L.lo_rmsdiv.restype = ctypes.c_double
        L.lo_rmsdiv.argtypes = [vp]
        for name in ["lo_destroy", "lo_step", "lo_sgs_stag", "lo_calc_sij", "lo_lagrange_sdep",
                     "lo_interpolag_sdep", "lo_wallstress", "lo_obukhov", "lo_project",
                     "lo_theta_all_in_one"]:
            getattr(L, name).argtypes = [vp] + ([ip] if name == "lo_step" else [])
        _lib = L
    return _lib


def _p(a):
    assert a.dtype == np.float64 and a.flags.c_contiguous
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


class Oracle:
    """CPU restatement of the reference step on the reference layout."""

    def __init__(self, cfg, surface=None):
        self.cfg = cfg
        self.L = lib()
        self.h = self.L.lo_create(ctypes.byref(cfg))
        if not self.h:
            raise RuntimeError("oracle create failed")
        self.d = dims(cfg)
        if surface is not None:
            self.set_surface(surface)

    def __del__(self):
        try:
            if self.h:
                self.L.lo_destroy(ctypes.c_void_p(self.h))
        except Exception:
            pass

    @staticmethod
    def set_threads(n):
        lib().lo_set_threads(int(n))

    @staticmethod
    def max_threads():
        return lib().lo_max_threads()

    def set_surface(self, s):
        zo = np.ascontiguousarray(s.zo, dtype=np.float64)
        wt = np.ascontiguousarray(s.wt_s, dtype=np.float64)
        self.L.lo_set_surface(ctypes.c_void_p(self.h), _p(zo), _p(wt))

    def view(self, name):
        n = ctypes.c_long()
        ptr = self.L.lo_field(ctypes.c_void_p(self.h), FIELD_ID[name], ctypes.byref(n))
        arr = np.ctypeslib.as_array(ptr, shape=(n.value,))
        return arr.reshape(field_shape(self.cfg, name))

    def get(self, name):
        return self.view(name).copy()

    def set(self, name, value):
        self.view(name)[...] = value

    def step(self, n=1):
        return self.L.lo_step(ctypes.c_void_p(self.h), int(n))

    def counters(self):
        a, b = ctypes.c_int(), ctypes.c_int()
        self.L.lo_counters(ctypes.c_void_p(self.h), ctypes.byref(a), ctypes.byref(b))
        return a.value, b.value

    def rmsdiv(self):
        return self.L.lo_rmsdiv(ctypes.c_void_p(self.h))

    def call(self, name, *arrays, ints=()):
        args = [ctypes.c_void_p(self.h)] + [_p(a) for a in arrays] + [ctypes.c_int(i) for i in ints]
        return getattr(self.L, "lo_" + name)(*args)

    # running statistics (io.f90:403-1218), by the reference's array names
    def stats_enable(self, c_count, p_count):
        self.L.lo_stats_enable(ctypes.c_void_p(self.h), int(c_count), int(p_count))

    def stats_accumulate(self):
        self.L.lo_stats_accumulate(ctypes.c_void_p(self.h))

    def stats_reset(self, group):
        self.L.lo_stats_reset(ctypes.c_void_p(self.h), int(group))

    def stats_get(self, name):
        out = np.zeros((self.cfg.nz - 1, self.cfg.ny, self.cfg.nx))
        f = self.L.lo_stats_get
        f.restype = ctypes.c_int
        if f(ctypes.c_void_p(self.h), name.encode(), _p(out)) != 0:
            raise KeyError(name)
        return out
