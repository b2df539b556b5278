"""The oracle pinned against the reference's own golden vectors and against
the reference's compiled linear_c.c (oracle/_ref, where it could be built)."""
import json
import math
import os

import numpy as np
import pytest

GOLD = os.path.join(os.path.dirname(__file__), "golden")


def load(name):
    with open(os.path.join(GOLD, name)) as f:
        return json.load(f)


@pytest.mark.parametrize("name", ["gtr", "jtt", "wag"])
def test_tree_loglike_goldens(oracle_lib, name):
    """tests/pplacer/test_like.ml:16-97: every edge's slow_log_like3 and
    supernode logdot equal PhyML's tree log likelihood to 1e-7 relative."""
    O = oracle_lib
    fx = load("like_%s.json" % name)
    ref = O.reference_from_fixture(fx)
    want = fx["expected_loglike"]
    for node in range(ref.n_nodes):
        a, b = ref.edge_loglike(node)
        assert abs(a - want) <= fx["rel_tol"] * abs(want), (node, a)
        assert abs(b - want) <= fx["rel_tol"] * abs(want), (node, b)


def test_masked_logdot_kat(oracle_lib):
    """tests/pplacer/test_linear.ml:4-28."""
    O = oracle_lib
    k = load("linear_kat.json")
    mask = np.array(k["mask"], dtype=np.uint16)
    m1, m2 = np.array(k["m1"]), np.array(k["m2"])
    assert math.isclose(O.lib().orc_mat_masked_logdot(m1, m2, mask, 3, 3), k["mat_expected"], rel_tol=1e-12)
    t1, t2 = np.array(k["t1"]), np.array(k["t2"])
    util = np.zeros(3)
    v = O.lib().orc_ten_masked_logdot(np.ascontiguousarray(t1), np.ascontiguousarray(t2), mask, util, 2, 3, 3)
    assert math.isclose(v, k["ten_expected"], rel_tol=1e-12)
    R = O.ref_lib()
    if R is not None:
        assert math.isclose(R.ref_mat_masked_logdot(m1, m2, mask, 3, 3), k["mat_expected"], rel_tol=1e-12)
        assert math.isclose(R.ref_ten_masked_logdot(np.ascontiguousarray(t1), np.ascontiguousarray(t2), mask,
                                                    util, 2, 3, 3), k["ten_expected"], rel_tol=1e-12)


def test_discrete_gamma_kat(oracle_lib):
    """Doc value of pplacer_src/gamma.ml:44-51."""
    k = load("gamma_kat.json")
    got = oracle_lib.discrete_gamma(k["n_cat"], k["alpha"])
    np.testing.assert_allclose(got, k["rates"], rtol=1e-12)


def test_diagd_exp_kat(oracle_lib):
    """tests/pplacer/test_diagd.ml:7-40 values.  diagd.ml builds
    x diag(l) x^-1 = B D (so exp rows sum to one), while that (disabled)
    reference test states expm(D B); the stated matrices are the transposes
    of what the reference code computes, and match them to the printed 8
    digits."""
    O = oracle_lib
    b = np.array([[-1., 0.15], [0.15, -2.]])
    d = np.array([0.25, 0.75])
    x, l, xit = O.diagd_of_d_b(d, b)
    exp1 = np.array([[0.77992929, 0.01668155], [0.05004464, 0.22387769]])
    exp4 = np.array([[0.37187386, 0.011053085], [0.03315925, 0.003437709]])
    np.testing.assert_allclose(O.diagd_to_exp(x, l, xit, 1.0).T, exp1, atol=1e-8)
    np.testing.assert_allclose(O.diagd_to_exp(x, l, xit, 4.0).T, exp4, atol=1e-8)
    # normed form: rows of P sum to one and pi is stationary
    x, l, xit = O.diagd_normed(b, d)
    P = O.diagd_to_exp(x, l, xit, 1.0)
    np.testing.assert_allclose(P.sum(1), 1.0, atol=1e-12)
    np.testing.assert_allclose(d @ P, d, atol=1e-12)


def test_restated_kernels_match_reference_linear_c(oracle_lib):
    """The oracle's restated L0 kernels equal the reference's own linear_c.c."""
    O = oracle_lib
    R = O.ref_lib()
    if R is None:
        pytest.skip("reference linear_c.c not built here")
    L = O.lib()
    rng = np.random.default_rng(7)
    for K in (4, 20, 7):
        for (Rr, S) in ((1, 1), (4, 33), (3, 257)):
            x, y, z = (rng.random((Rr, S, K)) for _ in range(3))
            statd = rng.dirichlet(np.ones(K))
            mask = (rng.random(S) < 0.6).astype(np.uint16)
            u1, u2 = np.zeros(S), np.zeros(S)
            assert L.orc_ten_log_like3(statd, x, y, z, u1, Rr, S, K) == R.ref_ten_log_like3(statd, x, y, z, u2, Rr, S, K)
            assert L.orc_ten_masked_logdot(x, y, mask, u1, Rr, S, K) == R.ref_ten_masked_logdot(x, y, mask, u2, Rr, S, K)
            f, l = S // 3, S - 1
            assert L.orc_ten_bounded_logdot(x, y, f, l, u1, Rr, S, K) == R.ref_ten_bounded_logdot(x, y, f, l, u2, Rr, S, K)
            x2, y2, z2 = x[0].copy(), y[0].copy(), z[0].copy()
            assert L.orc_mat_log_like3(statd, x2, y2, z2, S, K) == R.ref_mat_log_like3(statd, x2, y2, z2, S, K)
            assert L.orc_mat_masked_logdot(x2, y2, mask, S, K) == R.ref_mat_masked_logdot(x2, y2, mask, S, K)
            assert L.orc_mat_bounded_logdot(x2, y2, f, l, K) == R.ref_mat_bounded_logdot(x2, y2, f, l, S, K)
            a = rng.random((K, K))
            d1, d2 = np.zeros((S, K)), np.zeros((S, K))
            L.orc_gemmish(d1, a, x2, S, K)
            R.ref_gemmish(d2, a, x2, S, K)
            assert np.array_equal(d1, d2)
            lam = rng.random(K)
            e1, e2 = np.zeros((K, K)), np.zeros((K, K))
            L.orc_dediagonalize(e1, a, lam, y[0][:K].copy() if S >= K else rng.random((K, K)), K)
            R.ref_dediagonalize(e2, a, lam, y[0][:K].copy() if S >= K else rng.random((K, K)), K)
            if S >= K:
                assert np.array_equal(e1, e2)
            p1, p2 = np.zeros((Rr, S, K)), np.zeros((Rr, S, K))
            L.orc_statd_pairwise_prod(statd, p1, x, y, Rr * S, K)
            R.ref_ten_statd_pairwise_prod(statd, p2, x, y, Rr, S, K)
            assert np.array_equal(p1, p2)


def test_brent_matches_textbook_minimum(oracle_lib):
    """A smooth one-branch objective: the oracle's Brent finds the analytic
    optimum within its tolerance (placement of a query identical to a leaf
    prefers a zero-length pendant)."""
    O = oracle_lib
    from pplacer_gb300 import synth
    w = synth.make_workload("cpu_small", n_queries=3)
    m = O.Model(w.exch, w.statd, w.rates)
    ref = O.Reference(m, w.parent, w.bl, w.leaf_row, w.ref_seqs)
    q = w.query_seqs[1]
    res, st = ref.place([q])
    assert st[0] == 0 and res[0]
    edge, like, lwr, dist, pend = res[0][0]
    # at the optimum the derivatives vanish (or point out of the box)
    st, d = ref.loglike_derivs(q, edge, pend, dist)
    assert st == 0 and abs(d[0] - like) < 1e-6 * abs(like)
    # each coordinate is within Brent's final tolerance of a bound or of a
    # stationary point (Newton step below 1e-4)
    assert pend <= 1e-4 or abs(d[1] / d[3]) < 1e-4
    assert dist <= 1e-4 or dist >= w.bl[edge] - 1e-4 or abs(d[2] / d[4]) < 1e-4
