"""GPU drop-in for pplacer_src/linear_c.c against the oracle's restated
kernels (bit-identical to the reference's linear_c.c, see test_oracle.py) and
the reference's golden vectors."""
import json
import math
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

GOLD = os.path.join(os.path.dirname(__file__), "golden")
RTOL = 1e-12  # FP64 on the GPU; only the summation order differs


@pytest.fixture(scope="module")
def lin():
    from pplacer_gb300 import linear
    return linear


def test_kernels_vs_oracle(oracle_lib, lin):
    O = oracle_lib.lib()
    rng = np.random.default_rng(11)
    for K in (4, 20, 7):
        for R, S in ((1, 1), (4, 37), (4, 1500), (2, 3001)):
            x, y, z = (rng.random((R, S, K)) for _ in range(3))
            statd = rng.dirichlet(np.ones(K))
            mask = (rng.random(S) < 0.7).astype(np.uint16)
            if not mask.any():
                mask[0] = 1
            u1, u2 = np.zeros(S), np.zeros(S)
            want = O.orc_ten_log_like3(statd, x, y, z, u1, R, S, K)
            got = lin.ten_log_like3(statd, x, y, z, u2)
            assert math.isclose(got, want, rel_tol=RTOL)
            np.testing.assert_allclose(u2, u1, rtol=1e-14)
            want = O.orc_ten_masked_logdot(x, y, mask, u1, R, S, K)
            assert math.isclose(lin.ten_masked_logdot(x, y, mask, u2), want, rel_tol=RTOL)
            f, l = S // 4, S - 1
            want = O.orc_ten_bounded_logdot(x, y, f, l, u1, R, S, K)
            assert math.isclose(lin.ten_bounded_logdot(x, y, f, l, u2), want, rel_tol=RTOL)
            x2, y2, z2 = x[0].copy(), y[0].copy(), z[0].copy()
            assert math.isclose(lin.mat_log_like3(statd, x2, y2, z2), O.orc_mat_log_like3(statd, x2, y2, z2, S, K),
                                rel_tol=RTOL)
            assert math.isclose(lin.mat_masked_logdot(x2, y2, mask), O.orc_mat_masked_logdot(x2, y2, mask, S, K),
                                rel_tol=RTOL)
            assert math.isclose(lin.mat_bounded_logdot(x2, y2, f, l), O.orc_mat_bounded_logdot(x2, y2, f, l, K),
                                rel_tol=RTOL)
            a = rng.random((K, K))
            d1, d2 = np.zeros((S, K)), np.zeros((S, K))
            O.orc_gemmish(d1, a, x2, S, K)
            lin.gemmish(d2, a, x2)
            np.testing.assert_array_equal(d2, d1)  # same per-element summation order
            p1, p2 = np.zeros((R, S, K)), np.zeros((R, S, K))
            O.orc_statd_pairwise_prod(statd, p1, x, y, R * S, K)
            lin.ten_statd_pairwise_prod(statd, p2, x, y)
            np.testing.assert_array_equal(p2, p1)
            lin.ten_pairwise_prod(p2, x, y)
            np.testing.assert_array_equal(p2, x * y)
            m1 = np.zeros((S, K))
            lin.mat_pairwise_prod(m1, x2, y2)
            np.testing.assert_array_equal(m1, x2 * y2)
            lin.mat_statd_pairwise_prod(statd, m1, x2, y2)
            np.testing.assert_array_equal(m1, statd[None, :] * x2 * y2)
        lam, u, uit = rng.random(K), rng.random((K, K)), rng.random((K, K))
        e1, e2 = np.zeros((K, K)), np.zeros((K, K))
        O.orc_dediagonalize(e1, u, lam, uit, K)
        lin.dediagonalize(e2, u, lam, uit)
        np.testing.assert_array_equal(e2, e1)


def test_nbc_helpers(lin):
    rng = np.random.default_rng(5)
    x = rng.integers(0, 300, 1000).astype(np.uint16)
    y = rng.integers(0, 300, 1000).astype(np.uint16)
    assert lin.int_vec_tot(x) == int(x.astype(np.int64).sum())
    d = np.zeros(1000, dtype=np.uint16)
    lin.int_vec_pairwise_prod(d, x, y)
    np.testing.assert_array_equal(d, (x.astype(np.int64) * y.astype(np.int64) % 65536).astype(np.uint16))
    mat = rng.random((300, 17))
    vec = (rng.random(300) < 0.3).astype(np.uint16) * rng.integers(1, 5, 300).astype(np.uint16)
    dst = rng.random(17)
    want = dst + mat.T @ vec.astype(np.float64)
    lin.float_mat_int_vec_mul(dst, mat, vec)
    np.testing.assert_allclose(dst, want, rtol=1e-13)
    v1, v2 = rng.random(77), rng.random(77)
    out = np.zeros(77)
    lin.vec_pairwise_prod(out, v1, v2)
    np.testing.assert_array_equal(out, v1 * v2)


def test_masked_logdot_kat(lin):
    """tests/pplacer/test_linear.ml:4-28 through the GPU."""
    k = json.load(open(os.path.join(GOLD, "linear_kat.json")))
    mask = np.array(k["mask"], dtype=np.uint16)
    assert math.isclose(lin.mat_masked_logdot(np.array(k["m1"]), np.array(k["m2"]), mask), k["mat_expected"],
                        rel_tol=1e-12)
    assert math.isclose(lin.ten_masked_logdot(np.array(k["t1"]), np.array(k["t2"]), mask, np.zeros(3)),
                        k["ten_expected"], rel_tol=1e-12)


def _like_stree_via_dropin(lin, fx):
    """Like_stree.calc_distal_and_proximal + pull exponents + prep_supernodes
    (like_stree.ml:43-110, pplacer_run.ml:332-340) with every numeric kernel a
    call of the GPU drop-in, as the OCaml side would drive it; then the
    per-edge tree log likelihood of tests/pplacer/test_like.ml:57-66."""
    from pplacer_gb300 import model as M
    m = fx["model"]
    K = len(m["exch"])
    statd = M.emper_freq(fx["seqs"], K) if m["statd"] is None else np.array(m["statd"])
    rates = M.discrete_gamma(m["gamma_n_cats"], m["gamma_alpha"])
    x, lam, xit = M.diagd_normed(np.array(m["exch"]), statd)
    R, S = len(rates), len(fx["seqs"][0])
    parent = np.array(fx["parent"])
    bl = np.array(fx["bl"], dtype=np.float64)
    n = len(parent)
    root = int(np.where(parent < 0)[0][0])
    bl[root] = 0.0
    children = [[] for _ in range(n)]
    for i in range(n):
        if parent[i] >= 0:
            children[parent[i]].append(i)

    def multi_exp(t):
        ten = np.zeros((R, K, K))
        for r in range(R):
            lin.dediagonalize(ten[r], np.ascontiguousarray(x), np.exp(rates[r] * t * lam), np.ascontiguousarray(xit))
        return ten

    def evolve(src, t):
        a, e = src
        ten = multi_exp(t)
        out = np.zeros_like(a)
        for r in range(R):
            dst = np.zeros((S, K))
            lin.gemmish(dst, np.ascontiguousarray(ten[r]), np.ascontiguousarray(a[r]))
            out[r] = dst
        return out, e.copy()

    def pull(g, thr):
        a, e = g
        mx = a.max(axis=(0, 2))
        _, te = np.frexp(mx)
        sel = te < thr
        a[:, sel, :] *= np.ldexp(1.0, -te[sel])[None, :, None]
        e[sel] += te[sel]

    def prod(glvs):
        a, e = glvs[0][0].copy(), glvs[0][1].copy()
        for g in glvs[1:]:
            out = np.zeros_like(a)
            lin.ten_pairwise_prod(out, a, g[0])
            a = out
            e = e + g[1]
        return a, e

    distal, evd, prox = [None] * n, [None] * n, [None] * n
    for i in range(n):
        if not children[i]:
            lv = np.array([M.lv_of_char(c, K) for c in fx["seqs"][fx["leaf_row"][i]]])
            distal[i] = (np.broadcast_to(lv, (R, S, K)).copy(), np.zeros(S, dtype=np.int64))
        else:
            distal[i] = prod([evd[c] for c in children[i]])
            pull(distal[i], -50)
        evd[i] = evolve(distal[i], bl[i])
    prox[root] = (np.ones((R, S, K)), np.zeros(S, dtype=np.int64))
    for i in range(n - 1, -1, -1):
        if not children[i]:
            continue
        ep = evolve(prox[i], bl[i])
        for c in children[i]:
            prox[c] = prod([ep] + [evd[s] for s in children[i] if s != c])
            pull(prox[c], -50)
    util = np.zeros(S)
    one = np.ones((R, S, K))
    out = []
    for i in range(n):
        pull(distal[i], -10)
        pull(prox[i], -10)
        ud, up = evolve(distal[i], bl[i] / 2), evolve(prox[i], bl[i] / 2)
        sn = np.zeros((R, S, K))
        lin.ten_statd_pairwise_prod(statd, sn, ud[0], up[0])
        ll = lin.ten_bounded_logdot(sn, one, 0, S - 1, util) + math.log(2) * float((ud[1] + up[1]).sum())
        out.append(ll)
    return out


@pytest.mark.parametrize("name", ["gtr", "wag"])
def test_tree_loglike_golden_via_dropin(lin, name):
    fx = json.load(open(os.path.join(GOLD, "like_%s.json" % name)))
    lls = _like_stree_via_dropin(lin, fx)
    want = fx["expected_loglike"]
    for ll in lls:
        assert abs(ll - want) <= fx["rel_tol"] * abs(want), ll
