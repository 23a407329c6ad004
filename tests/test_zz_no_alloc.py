"""The allocation-free split GEMM entry point against the allocating one (needs a GB300).

librpa_gb300_tc_gemm_noalloc runs the same tcgen05 split GEMM as
librpa_gb300_selftest_tc_gemm with its scratch in a fixed device array. The test feeds it
the self-test's seeded inputs, checks that two calls in a row give bit-identical results,
that its error against the FP64 product equals the error the allocating entry point
reports for the same inputs, and that oversized requests are rejected.
"""
import ctypes
import math

import numpy as np
import pytest

import librpa_gb300 as L

pytestmark = pytest.mark.gpu

MASK = (1 << 64) - 1


def selftest_inputs(M, N, K, seed):
    """The seeded xorshift inputs of librpa_gb300_selftest_tc_gemm: A (M x K) then B (K x N)."""
    x = (0x9E3779B97F4A7C15 * (seed + 1)) & MASK
    out = np.empty(M * K + K * N)
    for t in range(out.size):
        x ^= (x << 13) & MASK
        x ^= x >> 7
        x ^= (x << 17) & MASK
        out[t] = (x >> 11) / 9007199254740992.0 * 2.0 - 1.0
    return out[:M * K].reshape(M, K), out[M * K:].reshape(K, N)


def bound(pieces, K):
    # the tolerances of the split GEMM accuracy tests
    return (3e-6 if pieces == 3 else 2e-5) * max(1.0, math.sqrt(K / 64))


@pytest.mark.parametrize("M,N,K,pieces,seed", [(300, 200, 1000, 3, 11), (256, 128, 512, 2, 7)])
def test_noalloc_gemm_matches_allocating_entry(lib, M, N, K, pieces, seed):
    torch = pytest.importorskip("torch")
    a, b = selftest_inputs(M, N, K, seed)
    ref = a @ b
    dev = torch.device("cuda", torch.cuda.current_device())
    da = torch.from_numpy(a).to(dev)
    db = torch.from_numpy(b).to(dev)
    outs = []
    free_before, free_after = [], []
    stream = torch.cuda.current_stream()
    for _ in range(2):
        dd = torch.full((M, N), float("nan"), dtype=torch.float32, device=dev)
        torch.cuda.synchronize()
        free_before.append(torch.cuda.mem_get_info()[0])
        rc = lib.librpa_gb300_tc_gemm_noalloc(M, N, K, da.data_ptr(), db.data_ptr(), dd.data_ptr(), pieces,
                                              ctypes.c_void_p(stream.cuda_stream))
        assert rc == 0, lib.librpa_get_last_error(None).decode()
        torch.cuda.synchronize()
        free_after.append(torch.cuda.mem_get_info()[0])
        outs.append(dd.cpu().numpy().astype(np.float64))
    # two calls in a row: identical results
    assert np.array_equal(outs[0], outs[1])
    err_new = np.abs(outs[0] - ref).max() / np.abs(ref).max()
    err_old = lib.librpa_gb300_selftest_tc_gemm(M, N, K, seed, pieces)
    assert not math.isnan(err_old), lib.librpa_get_last_error(None).decode()
    assert err_new < bound(pieces, K), err_new
    # same kernel on the same inputs: the two entry points' errors agree up to the FP64
    # reference products' own rounding difference
    assert abs(err_new - err_old) <= 1e-9, (err_new, err_old)
    # the second call (set-up done) took no device memory
    assert free_after[1] == free_before[1], (free_before, free_after)


def test_noalloc_gemm_rejects_oversized(lib):
    torch = pytest.importorskip("torch")
    dev = torch.device("cuda", torch.cuda.current_device())
    t = torch.zeros(8, dtype=torch.float64, device=dev)
    # 3 pieces * (4096 + 4096) rows * 4096 * 2 bytes = 192 MiB > 32 MiB of scratch
    rc = lib.librpa_gb300_tc_gemm_noalloc(4096, 4096, 4096, t.data_ptr(), t.data_ptr(), t.data_ptr(), 3, None)
    assert rc != 0
    msg = lib.librpa_get_last_error(None).decode()
    assert "scratch" in msg and "33554432" in msg, msg
    rc = lib.librpa_gb300_tc_gemm_noalloc(64, 64, 64, t.data_ptr(), t.data_ptr(), t.data_ptr(), 4, None)
    assert rc != 0 and "pieces" in lib.librpa_get_last_error(None).decode()


def test_noalloc_gemm_at_the_scratch_limit(lib):
    """The largest request that fits the 32 MiB scratch runs and gives the split GEMM's accuracy
    on two calls in a row; one row more is rejected, and the entry point still works after the
    rejection.  Each operand piece takes its size rounded up to 256 bytes, and the error flag
    one more 256-byte slot, so the need is pieces * (a_piece + b_piece) + 256.  2^25 - 256 is
    256 times a prime, so no request fills the array exactly: the largest (2 pieces, K = 64,
    M + N = 131070 rows of 128 bytes) leaves its last 256 bytes unused and puts the error flag
    in the 256 bytes before them."""
    torch = pytest.importorskip("torch")
    dev = torch.device("cuda", torch.cuda.current_device())
    limit = 32 << 20

    def need(m, n, k, pieces):
        kpad = (k + 63) // 64 * 64
        r = lambda x: (x + 255) // 256 * 256
        return pieces * (r(m * kpad * 2) + r(n * kpad * 2)) + 256

    K, N = 64, 128
    M = 131070 - N
    assert need(M, N, K, 2) == limit - 256 and need(M + 1, N, K, 2) > limit
    rng = np.random.default_rng(5)
    a = rng.uniform(-1, 1, (M, K))
    b = rng.uniform(-1, 1, (K, N))
    ref = a @ b
    da = torch.from_numpy(a).to(dev)
    db = torch.from_numpy(b).to(dev)
    outs = []
    for _ in range(2):
        dd = torch.full((M, N), float("nan"), dtype=torch.float32, device=dev)
        rc = lib.librpa_gb300_tc_gemm_noalloc(M, N, K, da.data_ptr(), db.data_ptr(), dd.data_ptr(), 2, None)
        assert rc == 0, lib.librpa_get_last_error(None).decode()
        torch.cuda.synchronize()
        outs.append(dd.cpu().numpy().astype(np.float64))
    assert np.array_equal(outs[0], outs[1])
    assert np.abs(outs[0] - ref).max() / np.abs(ref).max() < bound(2, K)
    # one more row needs 256 bytes beyond the array
    big = torch.zeros((M + 1) * K, dtype=torch.float64, device=dev)
    dd = torch.zeros((M + 1) * N, dtype=torch.float32, device=dev)
    rc = lib.librpa_gb300_tc_gemm_noalloc(M + 1, N, K, big.data_ptr(), db.data_ptr(), dd.data_ptr(), 2, None)
    assert rc != 0 and "scratch" in lib.librpa_get_last_error(None).decode()
    dd = torch.full((M, N), float("nan"), dtype=torch.float32, device=dev)
    rc = lib.librpa_gb300_tc_gemm_noalloc(M, N, K, da.data_ptr(), db.data_ptr(), dd.data_ptr(), 2, None)
    assert rc == 0, lib.librpa_get_last_error(None).decode()
    torch.cuda.synchronize()
    assert np.array_equal(dd.cpu().numpy().astype(np.float64), outs[0])
