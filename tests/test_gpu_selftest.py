"""Known-answer tests of the tensor-core building blocks of the mixed
reciprocal sum: the tcgen05 3xTF32 product from hand-built shared-memory
tiles, and the TMA path (operand images in TF32 hi/lo planes, 3-d boxes with
128-byte swizzle, zero fill past the end, swizzled MMA descriptors).

Bar: error relative to the sum of absolute products below 1e-6 (3xTF32
carries about 1e-7)."""
import ctypes as C

import pytest

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("name", ["stokes_gpu_selftest_tensor", "stokes_gpu_selftest_tma"])
def test_tensor_core_known_answer(lib, name):
    err = C.c_double(-1.0)
    rc = getattr(lib, name)(C.byref(err))
    assert rc == 0, lib.stokes_gpu_last_error_message().decode()
    assert 0.0 <= err.value < 1e-6, err.value
