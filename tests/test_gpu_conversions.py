"""The FP32 transform kernels convert between float and double with integer
operations (the hardware conversion issues on the scarce FP64 pipe).  Their
results must be bit-identical to the hardware conversion: exact widening,
narrowing rounded to nearest with ties to even."""
import ctypes

import pytest

import les_gb300 as lg

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("seed", [1, 20261203])
def test_conversions_match_hardware(gpu_lib, seed):
    L = lg.lib()
    f = L.les_selftest_conversions
    f.restype = ctypes.c_int
    f.argtypes = [ctypes.c_size_t, ctypes.c_ulonglong, ctypes.POINTER(ctypes.c_ulonglong)]
    bad = ctypes.c_ulonglong(123)
    lg.check(f(1 << 24, seed, ctypes.byref(bad)))
    assert bad.value == 0
