"""The tensor-core (integer-slice) trailing update of the real batched Cholesky against the
FP64 CUDA-core factorisation (needs a GB300).

librpa_gb300_selftest_chol_ozaki factors the same random SPD matrices both ways on the
device; the slice products are exact, so the factors agree to FP64 rounding.
"""
import ctypes
import math

import pytest

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("N,batch,spread", [(64, 2, 0), (200, 3, 0), (1000, 2, 0), (777, 2, 4), (1300, 1, 2)])
def test_ozaki_cholesky_matches_fp64(lib, N, batch, spread):
    rel = ctypes.c_double(float("nan"))
    dl = lib.librpa_gb300_selftest_chol_ozaki(N, batch, 5 + N, spread, ctypes.byref(rel))
    assert not math.isnan(dl), lib.librpa_get_last_error(None).decode()
    # ln det sums N logs of O(1) pivots: FP64 rounding of the two orders of summation
    assert dl <= 1e-11 * N, dl
    assert rel.value <= 1e-12, rel.value
