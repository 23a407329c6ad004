"""The tensor-core (integer-slice) Cholesky against the FP64 CUDA-core factorisation (needs a
GB300).

librpa_gb300_selftest_chol_ozaki factors the same random SPD matrices D (X X^T / N + shift I) D
both ways on the device.  The slice products are exact, so the trailing updates agree with FP64
to rounding; the panel solve multiplies by the FP64 inverse of the diagonal block, whose error
grows with that block's condition number, so the ill-conditioned case (shift 1e-6, condition
number about 4e6) gets a bound scaled by it.
"""
import ctypes
import math

import pytest

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("N,batch,spread,shift,ltol", [
    (64, 2, 0, 0.05, 1e-12), (200, 3, 0, 0.05, 1e-12), (1000, 2, 0, 0.05, 1e-12), (777, 2, 4, 0.05, 1e-12),
    (1300, 1, 2, 0.05, 1e-12), (700, 2, 0, 1e-6, 1e-9)])
def test_ozaki_cholesky_matches_fp64(lib, N, batch, spread, shift, ltol):
    rel = ctypes.c_double(float("nan"))
    dl = lib.librpa_gb300_selftest_chol_ozaki(N, batch, 5 + N, spread, shift, ctypes.byref(rel))
    assert not math.isnan(dl), lib.librpa_get_last_error(None).decode()
    # ln det sums N logs of the pivots: FP64 rounding of the two orders of summation
    assert dl <= (1e-11 if shift > 1e-3 else 1e-8) * N, dl
    assert rel.value <= ltol, rel.value
