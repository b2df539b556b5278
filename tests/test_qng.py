"""The oracle's QNG integrator and calc_marg_prob (oracle/qng.py), the
reference's posterior-probability integral (three_tax.ml:124-215 over
Gsl.Integration.qng), on the CPU.

  * the rule tables (pplacer_gb300/csrc/qng_rules.h) integrate the Legendre
    polynomials exactly to their design degrees (G10: 19, K21: 31, P43: 65,
    P87: 131), and the generator reproduces them;
  * QNG returns at the first stage whose rescaled error estimate meets the
    tolerance, with the analytic value inside that estimate, and raises
    ETOL when the 87-point stage fails;
  * calc_marg_prob agrees with the adaptive quadrature of the same integral
    (oracle.marginal_like) to pp_rel_err on real placements, and halves the
    upper limit after an ETOL (the retry path), integrating exactly what
    the halved range holds.
"""
import math

import numpy as np
import pytest

from oracle import qng as Q


def _rule(level):
    R = Q.rules()
    x1, x2, x3, x4 = R["x1"], R["x2"], R["x3"], R["x4"]
    if level == 10:
        xs, ws, c = x1, R["w10"], None
    elif level == 21:
        xs, ws, c = x1 + x2, R["w21a"] + R["w21b"][:5], R["w21b"][5]
    elif level == 43:
        xs, ws, c = x1 + x2 + x3, R["w43a"] + R["w43b"][:11], R["w43b"][11]
    else:
        xs, ws, c = x1 + x2 + x3 + x4, R["w87a"] + R["w87b"][:22], R["w87b"][22]
    X = np.array(xs + [-x for x in xs] + ([0.0] if c is not None else []))
    W = np.array(ws + ws + ([c] if c is not None else []))
    return X, W


@pytest.mark.parametrize("level,degree", [(10, 19), (21, 31), (43, 65), (87, 131)])
def test_rules_exact_to_design_degree(level, degree):
    from numpy.polynomial import legendre as Lg
    X, W = _rule(level)
    assert len(X) == level and np.all(W > 0) and np.all(np.abs(X) < 1)
    assert len(set(np.round(X, 15))) == level  # distinct nodes
    for k in range(degree + 1):
        cf = np.zeros(k + 1)
        cf[k] = 1.0
        assert abs((W * Lg.legval(X, cf)).sum() - (2.0 if k == 0 else 0.0)) <= 2e-15 * level, (level, k)
    cf = np.zeros(degree + 2)
    cf[-1] = 1.0
    assert abs((W * Lg.legval(X, cf)).sum()) > 1e-10  # and not beyond (the next degree, even)


def test_generator_reproduces_header():
    pytest.importorskip("mpmath")
    import importlib.util
    import os
    path = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "pplacer_gb300", "csrc",
                        "make_qng_rules.py")
    spec = importlib.util.spec_from_file_location("make_qng_rules", path)
    m = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(m)
    assert m.rules() == Q.rules()


@pytest.mark.parametrize("f,want,rel,neval", [
    (lambda x: x ** 20, 1.0 / 21, 1e-10, 21),            # a polynomial within K21's degree: the first stage
    (lambda x: 1.0 / (1.0 + 25.0 * x * x), math.atan(5.0) / 5.0, 1e-6, 43),
    (math.sqrt, 2.0 / 3.0, 1e-3, 43),
    (math.exp, math.e - 1.0, 1e-12, 21),
])
def test_qng_stages(f, want, rel, neval):
    res, err, n = Q.qng(f, 0.0, 1.0, 0.0, rel)
    assert n == neval
    assert err < rel * abs(res)
    assert abs(res - want) <= max(err, 1e-15)


@pytest.mark.parametrize("f", [math.sqrt, lambda x: abs(x - 0.37)])
def test_qng_etol(f):
    with pytest.raises(Q.QngError) as ex:
        Q.qng(f, 0.0, 1.0, 0.0, 1e-8)
    assert ex.value.code == "ETOL" and ex.value.result is not None


def test_qng_badtol():
    with pytest.raises(Q.QngError) as ex:
        Q.qng(math.exp, 0.0, 1.0, 0.0, 1e-20)
    assert ex.value.code == "EBADTOL"


def test_brent_finds_the_minimum():
    x = Q.brent(lambda v: abs(v - 0.731), 1.05, 0.1, 2.0, 1e-6)
    assert abs(x - 0.731) < 1e-5
    with pytest.raises(Q.BrentError):
        Q.brent(lambda v: v, 0.1, 0.1, 2.0, 1e-6)  # start on the boundary: InvalidStartValues


def test_brent_matches_the_dropin_flow():
    """The oracle's GSL Brent and the one of the measured plain drop-in
    flow (pplacer_gb300/dropin_flow.py) probe the same points."""
    from pplacer_gb300 import dropin_flow as DF
    for f0 in (lambda x: (x - 0.37) ** 2 + 0.1 * math.sin(8 * x), lambda x: abs(x - 1.3) ** 1.5,
               lambda x: -math.exp(-((x - 0.05) / 0.2) ** 2)):
        seen = [[], []]

        def rec(k):
            def g(x):
                seen[k].append(x)
                return f0(x)
            return g
        a = Q.brent(rec(0), 1.0, 1e-8, 2.0, 1e-5)
        b = DF.brent(rec(1), 1.0, 1e-8, 2.0, 1e-5)
        assert a == b
        # the same points (the oracle re-evaluates the set-up points, as GSL's set does)
        assert set(seen[0]) == set(seen[1])


def test_retry_halves_the_upper_limit():
    """A pendant surface with a kink the 87-point rule cannot resolve to
    1%: ETOL, the upper limit halves, and the result is the nested QNG of
    exactly the halved range (here it excludes the peak, as the reference's
    retry can)."""
    a, c = 100.0, 0.3
    L = lambda p, d: -a * abs(p - c) - 50.0 * (d - 0.02) ** 2
    m, info = Q.calc_marg_prob(L, c, 0.02, 0.05, lambda p: 1.0, 2.0, 0.01)
    assert info["exceptions"] == 1
    U = info["upper"]
    base = L(c, 0.02)

    def inner(d):
        return Q.qng(lambda p: math.exp(L(p, d) - base), 0.0, U, 0.0, 0.01)[0]
    want = base + math.log(Q.qng(inner, 0.0, 0.05, 0.0, 0.01)[0] / 0.05)
    assert m == want
    # the true integral over the halved range, for scale
    from scipy import integrate
    v, _ = integrate.dblquad(lambda p, d: math.exp(L(p, d) - base), 0.0, 0.05, 0.0, U, epsrel=1e-10)
    assert abs(m - (base + math.log(v / 0.05))) < 0.01


def test_ten_failures_return_the_base_likelihood():
    """An integrand no rule resolves on any range (it oscillates far
    faster than the 87-point nodes): ten ETOLs, then the base likelihood
    (three_tax.ml:177-183)."""
    L = lambda p, d: math.sin(1e7 * p)
    m, info = Q.calc_marg_prob(L, 0.3, 0.0, 0.0, lambda p: 1.0, 2.0, 0.01)
    assert info["exceptions"] == 10 and m == L(0.3, 0.0)


def test_calc_marg_prob_vs_adaptive(oracle_lib):
    """On real placements (cpu_small), the reference's nested QNG at
    pp_rel_err 0.01 and the adaptive quadrature of the same integral at
    1e-8 agree to that relative error (0.01 in log units)."""
    from oracle import oracle as O
    from pplacer_gb300 import synth
    w = synth.make_workload("cpu_small", n_queries=6)
    oref = O.Reference(O.Model(w.exch, w.statd, w.rates), w.parent, w.bl, w.leaf_row, w.ref_seqs)
    checked = 0
    res_all, status = oref.place(w.query_seqs[:3])
    for q in range(3):
        seq = w.query_seqs[q]
        if status[q] != 0 or not res_all[q]:
            continue
        e, like, lwr, d, p = res_all[q][0]
        cut = float(oref.bl[e])
        L = lambda pp, dd: oref.loglike_derivs(seq, e, max(pp, 1e-12), min(max(dd, 0.0), cut))[1][0]
        for prior_kind, mu in ((1, None), (0, 0.1)):
            prior = (lambda x: 1.0) if prior_kind == 1 else (lambda x, mu=mu: math.exp(-x / mu) / mu)
            m_qng, info = Q.calc_marg_prob(L, p, d, cut, prior, 2.0, 0.01)
            m_ad = O.marginal_like(oref, seq, e, p, d, prior_kind, mu, rel=1e-8)
            assert abs(m_qng - m_ad) < 0.01, (q, prior_kind, m_qng, m_ad, info)
            checked += 1
    assert checked >= 4
