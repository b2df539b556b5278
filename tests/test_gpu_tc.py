"""Tensor-core (tcgen05) evolve of the 20-state trial kernel: 128-site tiles,
operands split into TF32 hi + lo, three products accumulated in FP32, two
barrier phases into two TMEM column ranges per tile (the largest case puts
several tiles on each SM).  Checked against FP64 products with an
FP32-order error bound."""
import numpy as np
import pytest

from pplacer_gb300 import lib as L


@pytest.mark.gpu
@pytest.mark.parametrize("n,K,N", [(1, 20, 60), (128, 20, 60), (300, 20, 20), (257, 4, 12), (130, 24, 64),
                                   (1000, 20, 32), (152 * 4 * 128 + 5, 20, 60)])
def test_tc_evolve_matches_fp64(n, K, N):
    lib = L.load()
    rng = np.random.default_rng(n * 100 + K)
    # GLV-like rows over several binades, matrices with mixed signs
    A = (rng.random((n, K)) * np.exp2(rng.integers(-8, 2, size=(n, 1)))).astype(np.float32)
    B = rng.standard_normal((N, K)).astype(np.float32)
    out = np.full((n, N), np.nan, np.float32)
    st = lib.pgb_tc_evolve(A.ctypes.data, B.ctypes.data, out.ctypes.data, n, K, N)
    assert st == 0, lib.pgb_last_error()
    ref = A.astype(np.float64) @ B.astype(np.float64).T
    mag = np.abs(A).astype(np.float64) @ np.abs(B).astype(np.float64).T
    err = np.abs(out.astype(np.float64) - ref)
    assert np.all(np.isfinite(out))
    # FP32 arithmetic over K terms: a few units of 2^-24 per term
    assert np.all(err <= 2.0 ** -19 * mag + 1e-30), float(np.max(err / (mag + 1e-30)))


@pytest.mark.gpu
def test_tc_evolve_rejects_bad_shapes():
    lib = L.load()
    a = np.zeros((4, 20), np.float32)
    b = np.zeros((70, 20), np.float32)
    o = np.zeros((4, 70), np.float32)
    assert lib.pgb_tc_evolve(a.ctypes.data, b.ctypes.data, o.ctypes.data, 4, 20, 70) != 0
    assert lib.pgb_tc_evolve(a.ctypes.data, b.ctypes.data, o.ctypes.data, 4, 25, 8) != 0
