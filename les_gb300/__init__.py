"""GB300-native per-timestep spectral core of the KhaledGhannam/LES code.

The compute path is the CUDA library les_gb300/_lib/liblesgb300.so built for
sm_103a (see build.py); this module is its ctypes binding.  The C ABI is
declared in include/les_gb300.h and mirrors the reference's Fortran
subroutine interfaces (ddx, filt_da, convec, press_stag_array, ...), with
the reference's column-major array layouts.  There is no CPU fallback: if
the library is missing or no GPU is present the calls raise.
"""
import ctypes
import os

import numpy as np

from .config import (LesConfig, FIELDS, FIELD_ID, SURFACE_FIELDS, make_config, dims,
                     field_shape, initial_state, uniform_surface, striped_surface,
                     patch_surface, workload)

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_lib", "liblesgb300.so")

STATUS = {0: "LES_OK", -1: "LES_ERR_ARG", -2: "LES_ERR_CUDA", -3: "LES_ERR_OOM",
          -4: "LES_ERR_PIVOT", -5: "LES_ERR_CFL", -6: "LES_ERR_NAN", -7: "LES_ERR_TIMEOUT",
          -8: "LES_ERR_STATE", -9: "LES_ERR_UNSUPPORTED", -10: "LES_ERR_IO"}


class LesError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__("%s (%d): %s" % (STATUS.get(code, "?"), code, msg))
        self.code = code


_lib = None


def lib():
    """Load the CUDA library (raises if it was not built)."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise RuntimeError("les_gb300 CUDA library not built: run les_gb300/build.py")
        L = ctypes.CDLL(LIB_PATH)
        vp, ip, dp = ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p
        L.les_last_error.restype = ctypes.c_char_p
        L.les_ctx_create.argtypes = [ctypes.POINTER(LesConfig), ctypes.POINTER(vp)]
        L.les_ctx_stream.restype = vp
        L.les_ctx_stream.argtypes = [vp]
        L.les_ctx_device_bytes.restype = ctypes.c_size_t
        L.les_ctx_device_bytes.argtypes = [vp]
        L.les_estimate_device_bytes.restype = ctypes.c_size_t
        L.les_estimate_device_bytes.argtypes = [ctypes.POINTER(LesConfig)]
        L.les_field_device_ptr.restype = vp
        L.les_field_device_ptr.argtypes = [vp, ip]
        L.les_field_elems.restype = ctypes.c_size_t
        L.les_field_elems.argtypes = [vp, ip]
        for name in ["les_ctx_destroy", "les_step", "les_set_field", "les_get_field",
                     "les_set_surface", "les_rmsdiv", "les_ctx_set_pointer_mode", "les_register_field",
                     "les_sync_from_host", "les_sync_to_host"]:
            getattr(L, name).restype = ip
        L.les_register_field.argtypes = [vp, ip, dp]
        L.les_sync_from_host.argtypes = [vp]
        L.les_sync_to_host.argtypes = [vp]
        L.les_ctx_destroy.argtypes = [vp]
        L.les_step.argtypes = [vp, ip]
        L.les_set_field.argtypes = [vp, ip, dp]
        L.les_get_field.argtypes = [vp, ip, dp]
        L.les_set_surface.argtypes = [vp, dp, dp]
        L.les_rmsdiv.argtypes = [vp, dp]
        L.les_ctx_set_pointer_mode.argtypes = [vp, ip]
        cp, ll = ctypes.c_char_p, ctypes.c_longlong
        for name in ["les_checkpoint_write", "les_checkpoint_read", "les_fortran_record_write",
                     "les_fortran_record_read"]:
            getattr(L, name).restype = ip
        L.les_checkpoint_write.argtypes = [vp, cp]
        L.les_checkpoint_read.argtypes = [vp, cp]
        L.les_fortran_record_write.argtypes = [cp, ip, ctypes.POINTER(vp), ctypes.POINTER(ctypes.c_size_t), ip, ll]
        L.les_fortran_record_read.argtypes = [cp, ll, ctypes.POINTER(vp), ctypes.POINTER(ctypes.c_size_t), ip,
                                              ctypes.POINTER(ll), ctypes.POINTER(ll)]
        _lib = L
    return _lib


def check(code):
    if code != 0:
        raise LesError(code, lib().les_last_error().decode(errors="replace"))
    return code


def _ptr(a):
    if isinstance(a, np.ndarray):
        assert a.dtype == np.float64 and a.flags.c_contiguous, "float64 C-contiguous array required"
        return ctypes.c_void_p(a.ctypes.data)
    if hasattr(a, "data_ptr"):  # torch tensor on the device
        return ctypes.c_void_p(a.data_ptr())
    return ctypes.c_void_p(int(a))


class Context:
    """One ensemble member: device-resident state plus the routines of the
    reference's time step (main.f90:202-478)."""

    def __init__(self, cfg, surface=None):
        self.cfg = cfg
        self.L = lib()
        h = ctypes.c_void_p()
        check(self.L.les_ctx_create(ctypes.byref(cfg), ctypes.byref(h)))
        self.h = h
        self.d = dims(cfg)
        if surface is not None:
            self.set_surface(surface)

    def close(self):
        if getattr(self, "h", None):
            self.L.les_ctx_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # --- state --------------------------------------------------------------
    def set_surface(self, s):
        zo = np.ascontiguousarray(s.zo, dtype=np.float64)
        wt = np.ascontiguousarray(s.wt_s, dtype=np.float64)
        check(self.L.les_set_surface(self.h, _ptr(zo), _ptr(wt)))

    def set(self, name, value):
        a = np.ascontiguousarray(np.broadcast_to(value, field_shape(self.cfg, name)), dtype=np.float64)
        check(self.L.les_set_field(self.h, FIELD_ID[name], _ptr(a)))

    def get(self, name):
        a = np.empty(field_shape(self.cfg, name), dtype=np.float64)
        check(self.L.les_get_field(self.h, FIELD_ID[name], _ptr(a)))
        return a

    def device_ptr(self, name):
        return self.L.les_field_device_ptr(self.h, FIELD_ID[name])

    def stream(self):
        return self.L.les_ctx_stream(self.h)

    def set_priority(self, priority):
        """Move the context to a stream of this CUDA priority (lower is more urgent)."""
        check(self.L.les_ctx_set_priority(self.h, int(priority)))

    def device_bytes(self):
        return self.L.les_ctx_device_bytes(self.h)

    def counters(self):
        a, b = ctypes.c_int(), ctypes.c_int()
        check(self.L.les_get_counters(self.h, ctypes.byref(a), ctypes.byref(b)))
        return a.value, b.value

    # --- time stepping --------------------------------------------------------
    def step(self, n=1):
        check(self.L.les_step(self.h, int(n)))

    def step_graph(self, n=1):
        """Advance n steps replaying captured CUDA graphs (les_step_graph)."""
        check(self.L.les_step_graph(self.h, int(n)))

    def graph_prepare(self):
        """Capture the step graphs step_graph will replay, without stepping
        (les_step_graph_prepare)."""
        f = self.L.les_step_graph_prepare
        f.restype = ctypes.c_int
        f.argtypes = [ctypes.c_void_p]
        check(f(self.h))

    def autotune(self):
        a, b, c = ctypes.c_int(), ctypes.c_int(), ctypes.c_int()
        check(self.L.les_autotune(self.h, ctypes.byref(a), ctypes.byref(b), ctypes.byref(c)))
        return {"tx64": a.value, "tx32": b.value, "rpc_scale": c.value}

    def synchronize(self):
        check(self.L.les_rmsdiv(self.h, ctypes.byref(ctypes.c_double())))  # stream-ordered read

    def rmsdiv(self):
        r = ctypes.c_double()
        check(self.L.les_rmsdiv(self.h, ctypes.byref(r)))
        return r.value

    def timestep_conditions(self):
        a, b = ctypes.c_double(), ctypes.c_double()
        check(self.L.les_timestep_conditions(self.h, ctypes.byref(a), ctypes.byref(b)))
        return a.value, b.value

    # --- per-routine entry points (host arrays) --------------------------------
    def call(self, name, *arrays, ints=(), doubles=()):
        args = [self.h] + [_ptr(a) for a in arrays] + [ctypes.c_int(i) for i in ints] + \
            [ctypes.c_double(x) for x in doubles]
        fn = getattr(self.L, "les_" + name)
        fn.restype = ctypes.c_int
        return check(fn(*args))

    def set_pointer_mode(self, device):
        check(self.L.les_ctx_set_pointer_mode(self.h, 1 if device else 0))

    # --- whole-state image (serving: spill and resume) ------------------------
    def state_bytes(self):
        f = self.L.les_state_bytes
        f.restype = ctypes.c_size_t
        f.argtypes = [ctypes.c_void_p]
        return int(f(self.h))

    def state_save(self, buf):
        """Whole member state into `buf` (a uint8 numpy array of at least
        state_bytes() bytes, pinned memory copies fastest)."""
        f = self.L.les_state_save
        f.restype = ctypes.c_int
        f.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_size_t]
        check(f(self.h, ctypes.c_void_p(buf.ctypes.data), ctypes.c_size_t(buf.nbytes)))

    def state_restore(self, buf):
        f = self.L.les_state_restore
        f.restype = ctypes.c_int
        f.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_size_t]
        check(f(self.h, ctypes.c_void_p(buf.ctypes.data), ctypes.c_size_t(buf.nbytes)))

    # --- running statistics (io.f90:403-1218 MM_XYZ_Out) ---------------------
    def stats_enable(self, c_count, p_count, auto=False):
        check(self.L.les_stats_enable(self.h, int(c_count), int(p_count), 1 if auto else 0))

    def stats_accumulate(self):
        check(self.L.les_stats_accumulate(self.h))

    def stats_reset(self, group):
        check(self.L.les_stats_reset(self.h, int(group)))

    def stats_get(self, name):
        """One statistic by the reference's array name, (nz-1, ny, nx)."""
        i = stats_names().index(name)
        out = np.empty((self.cfg.nz - 1, self.cfg.ny, self.cfg.nx))
        check(self.L.les_stats_get(self.h, int(i), _ptr(out)))
        return out

    # --- checkpoint record (io.f90:1314-1338, initial.f90:54-160) ------------
    def checkpoint_write(self, path):
        check(self.L.les_checkpoint_write(self.h, os.fsencode(path)))

    def checkpoint_read(self, path):
        check(self.L.les_checkpoint_read(self.h, os.fsencode(path)))


def fortran_record_write(path, parts, append=False, max_subrecord=0):
    """Write the concatenation of the byte buffers in parts as one Fortran
    unformatted sequential record (les_fortran_record_write)."""
    L = lib()
    bufs = [np.ascontiguousarray(p).view(np.uint8).ravel() for p in parts]
    ptrs = (ctypes.c_void_p * max(1, len(bufs)))(*[b.ctypes.data for b in bufs])
    sizes = (ctypes.c_size_t * max(1, len(bufs)))(*[b.nbytes for b in bufs])
    check(L.les_fortran_record_write(os.fsencode(path), 1 if append else 0, ptrs, sizes, len(bufs),
                                     ctypes.c_longlong(max_subrecord)))


def fortran_record_read(path, nbytes, offset=0):
    """Read the record at byte offset into buffers of the given sizes;
    returns (buffers, record length, offset of the next record)."""
    L = lib()
    bufs = [np.empty(int(n), dtype=np.uint8) for n in nbytes]
    ptrs = (ctypes.c_void_p * max(1, len(bufs)))(*[b.ctypes.data for b in bufs])
    sizes = (ctypes.c_size_t * max(1, len(bufs)))(*[b.nbytes for b in bufs])
    rec, nxt = ctypes.c_longlong(), ctypes.c_longlong()
    check(L.les_fortran_record_read(os.fsencode(path), ctypes.c_longlong(offset), ptrs, sizes, len(bufs),
                                    ctypes.byref(rec), ctypes.byref(nxt)))
    return bufs, rec.value, nxt.value


class Ensemble:
    """Independent members advanced together: one CUDA graph launch per
    ensemble step runs one step of every member on its own stream branch."""

    def __init__(self, members):
        self.members = list(members)
        self.L = lib()
        arr = (ctypes.c_void_p * len(self.members))(*[m.h.value for m in self.members])
        h = ctypes.c_void_p()
        self.L.les_ensemble_stream.restype = ctypes.c_void_p
        self.L.les_ensemble_stream.argtypes = [ctypes.c_void_p]
        check(self.L.les_ensemble_create(arr, len(self.members), ctypes.byref(h)))
        self.h = h

    def step(self, n=1):
        check(self.L.les_ensemble_step(self.h, int(n)))

    def stream(self):
        return self.L.les_ensemble_stream(self.h)

    def close(self):
        if getattr(self, "h", None):
            self.L.les_ensemble_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def stats_names():
    """Names of the running statistics in the library's order."""
    L = lib()
    L.les_stats_name.restype = ctypes.c_char_p
    L.les_stats_name.argtypes = [ctypes.c_int]
    return [L.les_stats_name(i).decode() for i in range(L.les_stats_count())]


def stats_groups():
    L = lib()
    return {n: L.les_stats_group(i) for i, n in enumerate(stats_names())}


def estimate_device_bytes(cfg):
    return lib().les_estimate_device_bytes(ctypes.byref(cfg))
