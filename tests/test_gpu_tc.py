"""tcgen05 split-precision GEMM against the FP64 CUDA-core GEMM (needs a GB300)."""
import math

import pytest

import librpa_gb300 as L

pytestmark = pytest.mark.gpu


SHAPES = [(128, 128, 64), (256, 128, 512), (300, 200, 1000), (128, 384, 4096), (1000, 520, 5616)]


@pytest.mark.parametrize("M,N,K", SHAPES)
def test_tc_gemm_bf16x3_accuracy(lib, M, N, K):
    err = lib.librpa_gb300_selftest_tc_gemm(M, N, K, 7, 2)
    assert not math.isnan(err), L.load_library().librpa_get_last_error(None).decode()
    # 3-term BF16 split with FP32 accumulation: ~2^-16 per product, sqrt(K) growth at most
    assert err < 2e-5 * max(1.0, math.sqrt(K / 64)), err


@pytest.mark.parametrize("M,N,K", SHAPES)
def test_tc_gemm_bf16x6_accuracy(lib, M, N, K):
    err = lib.librpa_gb300_selftest_tc_gemm(M, N, K, 11, 3)
    assert not math.isnan(err), L.load_library().librpa_get_last_error(None).decode()
    # 3-piece split (6 products): limited by the tensor core's FP32 accumulation (6 adds per
    # K=16 step), measured ~1.3e-6 * sqrt(K/64) on GB300 -- 5x below the 2-piece split
    assert err < 3e-6 * max(1.0, math.sqrt(K / 64)), err
