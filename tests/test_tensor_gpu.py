"""The tcgen05 tensor-core datapath (kind::tf32, A in tensor memory, B in
shared memory) against an FP64 product, through the C ABI."""
import ctypes

import pytest

from p4gpu import _lib

pytestmark = pytest.mark.gpu


def test_tf32_mma_selftest(lib):
    err = ctypes.c_double(-1.0)
    rc = lib.p4g_tensorSelfTest(0, ctypes.byref(err))
    assert rc == 0, _lib.last_error()
    # inputs are multiples of 2^-8 in [-1, 1): every product and sum is exact
    assert err.value == 0.0, err.value
