"""Batched GPU placement engine against the FP64 oracle.

Tolerances (FP32 GLVs with exact int32 exponents, FP64 per-site log sums and
scalar optimiser state):
  * logL of a fixed (query, edge, pendant, distal) point: 2e-7 relative
  * optimised logL: 1e-6 relative (the accuracy target of the placement path)
  * best edge identical for >= 99.9% of queries whose top two oracle
    placements are not tied (tie: within 1e-6 relative)
"""
import math

import numpy as np
import pytest

import parity

pytestmark = pytest.mark.gpu

LOGL_RTOL = 1e-6


# trial-kernel forms: one CTA (256 threads, windows in shared memory) or one
# warp per trial; for the nucleotide Gamma warp kernel the second number picks
# its form: 0 the transition matrices in registers, 1 the eigenbasis (8 warps
# per SM), 2 and 3 the eigenbasis at 12 and 16 warps per SM, 4 and 5 the
# eigenbasis on packed FP32 pairs at 12 and 16 warps per SM
FORMS = {"cta": (256, 1), "warp": (32, 0), "eig": (32, 1), "eig12": (32, 2), "eig16": (32, 3),
         "eig12x2": (32, 4), "eig16x2": (32, 5)}


@pytest.fixture(scope="module", params=sorted(FORMS))
def small(request, oracle_lib):
    from pplacer_gb300 import engine as E
    from pplacer_gb300 import synth
    w = synth.make_workload("cpu_small", n_queries=60)
    O = oracle_lib
    oref = O.Reference(O.Model(w.exch, w.statd, w.rates), w.parent, w.bl, w.leaf_row, w.ref_seqs)
    eng = E.engine_for_workload(w)
    eng.set_tuning(*FORMS[request.param])
    eng.load_queries(w.query_seqs)
    return w, oref, eng


def _scaled_log(a, e):
    with np.errstate(divide="ignore"):
        return np.log(a) + math.log(2) * e[None, :, None]


def test_precompute_matches_oracle(small):
    w, oref, eng = small
    for node in list(range(0, w.n_nodes, 17)) + [w.n_nodes - 1]:
        for which in (0, 1, 2):
            ga, ge = eng.get_glv(which, node)
            oa, oe = oref.glv(which, node)
            assert np.mean(ge == oe) >= 0.999
            same = ge == oe
            mx = oa.max(axis=(0, 2), keepdims=True)
            sig = (oa >= 1e-6 * mx) & same[None, :, None]
            np.testing.assert_allclose(ga[sig], oa[sig], rtol=2e-6)


def test_stage1_scores_match_oracle(small, oracle_lib):
    w, oref, eng = small
    sc = eng.stage1()
    edges = [i for i in range(w.n_nodes) if w.parent[i] >= 0]
    for q in range(0, 60, 7):
        st, ranking, _ = oref.trace(w.query_seqs[q], oracle_lib.make_prefs(max_strikes=1, max_pitches=0))
        want = dict(ranking)
        got = np.array([sc[q, i] for i in range(len(edges))])
        ref = np.array([want[e] for e in edges])
        np.testing.assert_allclose(got, ref, rtol=1e-6)


def test_stage1_ranking_matches_oracle_order(small, oracle_lib):
    """The GPU's ranked edge order against the oracle's ranking (core.ml:
    187-197 scored, fig.ml:143-147 sorted): position by position, the
    oracle's score of the GPU's edge equals the oracle's score at that
    position to the stage-1 tolerance (1e-6 relative), so the orders differ
    at most by swaps of scores that agree to that tolerance."""
    w, oref, eng = small
    eng.stage1()
    edges = [i for i in range(w.n_nodes) if w.parent[i] >= 0]
    E = len(edges)
    got = eng.rank(E)
    for q in range(0, 60, 5):
        st, ranking, _ = oref.trace(w.query_seqs[q], oracle_lib.make_prefs(max_strikes=1, max_pitches=0))
        if st != 0 or not ranking:
            continue
        want = dict(ranking)
        ordered = [s for _, s in ranking]
        assert len(ordered) == E
        for j in range(E):
            g = want[edges[got[q][j]]]
            assert abs(g - ordered[j]) <= 1e-6 * abs(ordered[j]), (q, j, g, ordered[j])


@pytest.mark.parametrize("rk", [1, 65, 130, 0])
def test_stage1_ranking(small, rk):
    """The rk best edges per query (0: every edge): scores descending, equal
    scores by increasing edge index, NaN last (fig.ml:143-147).  Short
    rankings read the scores from global memory, long ones stage them in
    shared memory and refill the lanes' caches."""
    w, oref, eng = small
    sc = eng.stage1()
    E = sc.shape[1]
    rk = min(E, rk) if rk else E
    got = eng.rank(rk)
    for q in range(sc.shape[0]):
        want = sorted(range(E), key=lambda i: (math.isnan(sc[q, i]), -sc[q, i] if not math.isnan(sc[q, i]) else 0.0, i))
        assert list(got[q]) == want[:rk], q


def _trial_list(w, n, seed):
    rng = np.random.default_rng(seed)
    edges = np.where(w.parent >= 0)[0]
    out = []
    for _ in range(n):
        q = int(rng.integers(len(w.query_seqs)))
        e = int(rng.choice(edges))
        out.append((q, e))
    return out


def test_loglike_at_fixed_points(small):
    w, oref, eng = small
    from pplacer_gb300 import engine as E
    pairs = _trial_list(w, 40, 1)
    rng = np.random.default_rng(2)
    trials = []
    for q, e in pairs:
        trials.append((q, e, float(rng.uniform(1e-8, 0.5)), float(rng.uniform(0, w.bl[e])), 0.01))
    got = eng.trials(trials, optimizer=E.NEWTON, mode=1)
    for (q, e, p, d, _), g in zip(trials, got):
        st, ref = oref.loglike_derivs(w.query_seqs[q], e, p, d)
        assert st == 0
        assert abs(g["like"] - ref[0]) <= 2e-7 * abs(ref[0]), (g["like"], ref[0])
        # adjoint: gradient and Hessian against the FP64 oracle
        hscale = math.sqrt(abs(ref[3] * ref[4])) + 1.0
        for k, (gv, rv) in enumerate(zip(g["derivs"][:5], ref[1:6])):
            tol = 2e-3 * abs(rv) + (1e-5 * abs(ref[3 + k]) + 1e-2 if k < 2 else 1e-3 * hscale + 1.0)
            assert abs(gv - rv) <= tol, (k, gv, rv)


def test_oracle_gradient_vs_central_fd(small):
    """The FP64 analytic derivatives (the adjoint's reference) against central
    finite differences with h = 1e-6."""
    w, oref, _ = small
    h = 1e-6
    for q, e in _trial_list(w, 12, 3):
        p, d = 0.05, 0.4 * w.bl[e]
        s = w.query_seqs[q]
        _, c = oref.loglike_derivs(s, e, p, d)
        _, pp = oref.loglike_derivs(s, e, p + h, d)
        _, pm = oref.loglike_derivs(s, e, p - h, d)
        _, dp = oref.loglike_derivs(s, e, p, d + h)
        _, dm = oref.loglike_derivs(s, e, p, d - h)
        fd_gp = (pp[0] - pm[0]) / (2 * h)
        fd_gd = (dp[0] - dm[0]) / (2 * h)
        noise = 4e-16 * abs(c[0]) / h
        assert abs(fd_gp - c[1]) <= 1e-6 * abs(c[1]) + noise
        assert abs(fd_gd - c[2]) <= 1e-6 * abs(c[2]) + noise
        fd_hpp = (pp[1] - pm[1]) / (2 * h)
        assert abs(fd_hpp - c[3]) <= 1e-5 * abs(c[3]) + 1e-3


def test_gpu_forward_vs_fd(small):
    """The GPU adjoint against central differences of the GPU forward (FP32
    forward: step sized to its noise, h = 1e-3 on the branch length)."""
    w, oref, eng = small
    from pplacer_gb300 import engine as E
    h = 1e-3
    trials = []
    pairs = _trial_list(w, 10, 4)
    for q, e in pairs:
        p, d = 0.08, 0.5 * w.bl[e]
        trials += [(q, e, p, d, 0.01), (q, e, p + h, d, 0.01), (q, e, p - h, d, 0.01),
                   (q, e, p, d + h, 0.01), (q, e, p, d - h, 0.01)]
    got = eng.trials(trials, optimizer=E.NEWTON, mode=1)
    for i in range(len(pairs)):
        c, pp, pm, dp, dm = got[5 * i:5 * i + 5]
        fd_gp = (pp["like"] - pm["like"]) / (2 * h)
        fd_gd = (dp["like"] - dm["like"]) / (2 * h)
        assert abs(fd_gp - c["derivs"][0]) <= 1e-2 * abs(c["derivs"][0]) + 0.05
        assert abs(fd_gd - c["derivs"][1]) <= 1e-2 * abs(c["derivs"][1]) + 0.05


@pytest.mark.parametrize("optimizer", [0, 1])
@pytest.mark.parametrize("tol", [0.01, 1e-5])
def test_single_location_optimisation(small, oracle_lib, optimizer, tol):
    """Three_tax.optimize from the default start at one location
    (core.ml:240-279).  Newton reaches the FP64-polished optimum; the Brent
    replica stops, like the reference, within its tolerance of it."""
    w, oref, eng = small
    O = oracle_lib
    pairs = _trial_list(w, 30, 5)
    trials = [(q, e, 0.1, w.bl[e] / 2.0, tol) for q, e in pairs]
    got = eng.trials(trials, optimizer=optimizer, mode=0)
    for (q, e, p0, d0, _), g in zip(trials, got):
        st, ref = oref.optimize_location(w.query_seqs[q], e, p0, d0, tol)
        assert st == 0 and g["status"] in (0, 1)
        rl = ref[0]
        star = O.polish(oref, w.query_seqs[q], e, ref[1], ref[2])[0]
        eps = LOGL_RTOL * abs(rl)
        assert g["like"] <= star + eps, (g, star)
        if optimizer == 1:
            assert g["like"] >= star - eps, (g, star)
        else:
            assert g["like"] >= rl - max(eps, 2 * (star - rl)) - (0.05 if tol > 1e-3 else 0.0), (g, ref, star)


def _compare_placements(O, oref, seqs, res_gpu, res_orc, oprefs=None, newton=True, min_logl_frac=1.0):
    """Whole placement records against the oracle (parity.compare): best
    edge and logL, kept set, branch lengths against the FP64-polished optima
    and like_weight_ratios.

    Two edges are tied when their FP64-polished optima (oracle.polish) agree
    to 1e-6 relative -- e.g. a query attaching exactly at a node is the same
    point of the tree seen from each of the node's edges.  The reference's
    alternating Brent can stop well below a location's optimum (on long
    queries by up to ~1 logL), which can change the location it ranks best.
    When the GPU's best location has the higher polished optimum -- it found
    the better placement -- the query counts as agreeing, provided the GPU's
    logL there is that optimum.

    Tolerances: Newton -- best edge identical for >= 99.9% of non-tied
    queries, lengths within what the FP64 logL gap at them allows, gap <=
    1e-6 relative, like_weight_ratio 1e-4 (+ twice the gap); the Brent
    replica (the reference's search on FP32 likelihoods, whose rounding can
    steer its path) -- best edge for >= 95%, gap <= 1e-4 relative."""
    oprefs = oprefs or O.make_prefs()
    st, bad = parity.compare(O, oref, seqs, res_gpu, res_orc, keep_at_most=oprefs.keep_at_most,
                             keep_factor=oprefs.keep_factor, min_logl_frac=min_logl_frac, newton=newton,
                             gap_tol=1e-6 if newton else 1e-4, lwr_tol=1e-4,
                             max_mismatch_frac=0.001 if newton else 0.05,
                             oracle_stage2=parity.oracle_stage2(O, oref, seqs, oprefs))
    print("placement parity:", {k: (float(v) if isinstance(v, float) else v) for k, v in st.items()})
    assert not bad, "\n".join(bad[:20])
    assert st["records"] > 0 or st["non_tied"] == 0
    return st


@pytest.mark.parametrize("optimizer", [0, 1])
def test_place_all_edges_vs_oracle(small, oracle_lib, optimizer):
    """cpu_small preferences: every edge goes to stage 2 (max_strikes 0)."""
    from pplacer_gb300 import engine as E
    w, oref, eng = small
    O = oracle_lib
    op = O.make_prefs(max_strikes=0)
    ores, ost = oref.place(w.query_seqs, op, n_threads=8)
    gres, gst = eng.place(w.query_seqs, E.default_prefs(max_strikes=0, optimizer=optimizer))
    assert list(gst) == list(ost)
    _compare_placements(O, oref, w.query_seqs, gres, ores, op, newton=optimizer == 1)
    for g in gres:
        assert abs(sum(p[2] for p in g) - 1.0) < 1e-9 and all(a[2] >= b[2] for a, b in zip(g, g[1:]))


@pytest.mark.parametrize("form", sorted(FORMS))
def test_place_baseball_dna(oracle_lib, form):
    """dna_1k preferences (keep 7, strikes 6) on a 60-query sample.  The
    Brent replica follows the reference's search, whose path FP32 rounding can
    change, so it may end on a different coordinate-wise stopping point for
    a few queries; the Newton form reaches the optimum."""
    from pplacer_gb300 import engine as E
    from pplacer_gb300 import synth
    O = oracle_lib
    w = synth.make_workload("dna_1k", n_queries=60)
    oref = O.Reference(O.Model(w.exch, w.statd, w.rates), w.parent, w.bl, w.leaf_row, w.ref_seqs)
    ores, ost = oref.place(w.query_seqs, O.make_prefs(), n_threads=8)
    eng = E.engine_for_workload(w)
    eng.set_tuning(*FORMS[form])
    for optimizer, frac in ((1, 1.0), (0, 0.95)):
        gres, gst = eng.place(w.query_seqs, E.default_prefs(optimizer=optimizer))
        assert list(gst) == list(ost)
        _compare_placements(O, oref, w.query_seqs, gres, ores, newton=optimizer == 1, min_logl_frac=frac)


@pytest.mark.parametrize("form", sorted(FORMS))
@pytest.mark.parametrize("n_rates", [1, 2, 8])
def test_place_rate_counts(oracle_lib, n_rates, form):
    """Gamma mixtures of 1, 2 and 8 rates (the warp form's lane layout
    changes with the rate count)."""
    from pplacer_gb300 import engine as E
    from pplacer_gb300 import synth
    O = oracle_lib
    w = synth.make_workload("dna_1k", n_queries=25, taxa=80, sites=400, lo=60, hi=400, n_rates=n_rates)
    assert len(w.rates) == n_rates
    oref = O.Reference(O.Model(w.exch, w.statd, w.rates), w.parent, w.bl, w.leaf_row, w.ref_seqs)
    ores, ost = oref.place(w.query_seqs, O.make_prefs(), n_threads=8)
    eng = E.engine_for_workload(w)
    eng.set_tuning(*FORMS[form])
    gres, gst = eng.place(w.query_seqs, E.default_prefs(optimizer=1))
    assert list(gst) == list(ost)
    _compare_placements(O, oref, w.query_seqs, gres, ores)


def test_place_gcat_and_protein(oracle_lib):
    """Per-site CAT (Gcat_model) and 20-state Gamma models on small trees."""
    from pplacer_gb300 import engine as E
    from pplacer_gb300 import synth
    O = oracle_lib
    for name, kw in (("cat_5k", dict(taxa=120, sites=300, lo=60, hi=300)),
                     ("aa_500", dict(taxa=60, sites=120, lo=40, hi=120))):
        w = synth.make_workload(name, n_queries=30, **kw)
        om = O.Model(w.exch, w.statd, w.rates, w.site_cats)
        oref = O.Reference(om, w.parent, w.bl, w.leaf_row, w.ref_seqs)
        ores, ost = oref.place(w.query_seqs, O.make_prefs(), n_threads=8)
        eng = E.engine_for_workload(w)
        for optimizer, frac in ((1, 1.0), (0, 0.95)):
            gres, gst = eng.place(w.query_seqs, E.default_prefs(optimizer=optimizer))
            assert list(gst) == list(ost), name
            _compare_placements(O, oref, w.query_seqs, gres, ores, newton=optimizer == 1, min_logl_frac=frac)


def test_edge_cases(small, oracle_lib):
    """All-gap query, unknown character, ambiguity codes, a one-site query,
    an empty batch, and a zero-length edge."""
    from pplacer_gb300 import engine as E
    w, oref, eng = small
    S = w.n_sites
    base = w.query_seqs[0]
    amb = "".join(("N" if i % 7 == 0 else "R" if i % 11 == 0 else c) if c != "-" else c for i, c in enumerate(base))
    one = "-" * 500 + base.strip("-")[0] + "-" * (S - 501)
    qs = ["-" * S, base[:10] + "Z" + base[11:], amb, one]
    gres, gst = eng.place(qs, E.default_prefs())
    ores, ost = oref.place(qs, oracle_lib.make_prefs(), n_threads=4)
    assert list(gst) == [1, 3, 0, 0] and list(ost) == [1, 3, 0, 0]
    for i in (2, 3):
        assert gres[i][0][0] == ores[i][0][0] or abs(gres[i][0][1] - ores[i][0][1]) <= 1e-6 * abs(ores[i][0][1])
        assert abs(gres[i][0][1] - ores[i][0][1]) <= LOGL_RTOL * abs(ores[i][0][1])
    r, s = eng.place([], E.default_prefs())
    assert r == [] and len(s) == 0
    # zero-length edge: distal is fixed at 0
    from pplacer_gb300 import synth
    w2 = synth.make_workload("cpu_small", n_queries=8, taxa=30, sites=200, lo=80, hi=200)
    w2.bl[3] = 0.0
    O = oracle_lib
    oref2 = O.Reference(O.Model(w2.exch, w2.statd, w2.rates), w2.parent, w2.bl, w2.leaf_row, w2.ref_seqs)
    eng2 = E.engine_for_workload(w2)
    eng2.set_tuning(*eng.get_tuning())
    eng2.load_queries(w2.query_seqs)
    got = eng2.trials([(0, 3, 0.1, 0.0, 1e-5)], optimizer=0)
    st, ref = oref2.optimize_location(w2.query_seqs[0], 3, 0.1, 0.0, 1e-5)
    assert got[0]["dist"] == 0.0 and abs(got[0]["like"] - ref[0]) <= LOGL_RTOL * abs(ref[0])


def test_jplace_of_engine_results(small):
    """Engine results through the jplace writer (placerun_io.ml:58-90)."""
    import json
    from pplacer_gb300 import engine as E
    from pplacer_gb300 import jplace
    w, oref, eng = small
    qs = w.query_seqs[:12]
    res, st = eng.place(qs, E.default_prefs())
    doc = json.loads(jplace.to_jplace(res, ["q%d" % i for i in range(len(qs))], w.parent, w.bl))
    assert len(doc["placements"]) == sum(1 for r in res if r)
    f = doc["fields"]
    for row, r in zip(doc["placements"], [r for r in res if r]):
        assert [p[f.index("edge_num")] for p in row["p"]] == [p[0] for p in r]
        assert abs(sum(p[f.index("like_weight_ratio")] for p in row["p"]) - 1.0) < 1e-9


@pytest.mark.parametrize("prior", [0, 1, 2])
def test_posterior_probabilities(oracle_lib, prior):
    """calc_pp (-p): marginal likelihoods of the kept placements against an
    FP64 adaptive quadrature of the same integral (three_tax.ml:169-215), and
    the posterior probabilities they give (core.ml:396-401).  pplacer's own
    QNG is accurate to pp_rel_err (0.01 relative, 0.01 in log units); the
    tolerance here is 2e-3."""
    import math
    from pplacer_gb300 import engine as E
    from pplacer_gb300 import synth
    O = oracle_lib
    w = synth.make_workload("cpu_small", n_queries=4, taxa=60, sites=400, lo=100, hi=300)
    oref = O.Reference(O.Model(w.exch, w.statd, w.rates), w.parent, w.bl, w.leaf_row, w.ref_seqs)
    eng = E.engine_for_workload(w)
    res, st = eng.place(w.query_seqs, E.default_prefs(calc_pp=1, prior=prior, prior_lower=0.01))
    mu = O.prior_means(w.parent, w.bl, prior, prior_lower=0.01)
    checked = 0
    for q in range(3):
        places = res[q][:3]
        assert places and all(len(p) == 7 for p in places)
        want = []
        for (e, like, lwr, d, p, pp, m) in places:
            ref_m = O.marginal_like(oref, w.query_seqs[q], e, p, d, prior, None if mu is None else mu[e], rel=1e-8)
            assert abs(m - ref_m) <= 2e-3, (q, e, m, ref_m)
            assert m <= like + 1e-9 or prior == 1  # a proper prior integrates to at most the peak
            want.append(ref_m)
            checked += 1
        if len(res[q]) == len(places):
            mx = max(want)
            tot = sum(math.exp(v - mx) for v in want)
            for (_, _, _, _, _, pp, _), v in zip(places, want):
                assert abs(pp - math.exp(v - mx) / tot) <= 2e-3
        assert abs(sum(p[5] for p in res[q]) - 1.0) < 1e-9
    assert checked >= 3


def test_marginal_trials_mode(oracle_lib):
    """pgb_queries_trials mode 2 at the oracle's polished optimum."""
    from pplacer_gb300 import engine as E
    from pplacer_gb300 import synth
    O = oracle_lib
    w = synth.make_workload("cpu_small", n_queries=4, taxa=60, sites=400, lo=100, hi=300)
    oref = O.Reference(O.Model(w.exch, w.statd, w.rates), w.parent, w.bl, w.leaf_row, w.ref_seqs)
    eng = E.engine_for_workload(w)
    eng.load_queries(w.query_seqs)
    mu = O.prior_means(w.parent, w.bl, 0)
    trials = []
    edges = np.where(w.parent >= 0)[0]
    for q, e in ((0, edges[5]), (1, edges[17]), (2, edges[29])):
        like, p, d = O.polish(oref, w.query_seqs[q], int(e), 0.1, float(w.bl[e]) / 2)
        trials.append((q, int(e), p, d, 0.01))
    got = eng.trials(trials, optimizer=E.NEWTON, mode=2, prefs=E.default_prefs(prior=0))
    for (q, e, p, d, _), g in zip(trials, got):
        ref_m = O.marginal_like(oref, w.query_seqs[q], e, p, d, 0, mu[e], rel=1e-8)
        assert g["status"] == 0 and abs(g["like"] - ref_m) <= 2e-3, (q, e, g["like"], ref_m)


def _qng_oracle_marginal(oref, seq, e, p, d, prior_kind, mu, rel, max_pend=2.0):
    """The reference's calc_marg_prob (oracle/qng.py) on the oracle's FP64
    likelihood; prior_kind as the engine's prefs.prior: 0 exponential
    (mean mu), 1 uniform."""
    import math
    from oracle import qng as Q
    cut = float(oref.bl[e])
    L = lambda pp, dd: oref.loglike_derivs(seq, e, max(pp, 1e-12), min(max(dd, 0.0), cut))[1][0]
    prior = (lambda x: 1.0) if prior_kind == 1 else (lambda x: math.exp(-x / mu) / mu)
    return Q.calc_marg_prob(L, p, d, cut, prior, max_pend, rel)


@pytest.mark.parametrize("prior", [0, 1])
def test_marginal_qng_replica(oracle_lib, prior):
    """pp_rule 1: the reference's own marginal likelihood (find_upper_limit's
    Brent search, nested QNG to pp_rel_err, ETOL retries) in the trial
    kernel, against the same computation in the oracle on the FP64
    likelihood: within pp_rel_err in log units (the two may stop at
    different QNG stages where the FP32 and FP64 integrands straddle a
    stage's tolerance), and most within 1e-3."""
    from pplacer_gb300 import engine as E
    from pplacer_gb300 import synth
    O = oracle_lib
    w = synth.make_workload("cpu_small", n_queries=6, taxa=60, sites=400, lo=100, hi=300)
    oref = O.Reference(O.Model(w.exch, w.statd, w.rates), w.parent, w.bl, w.leaf_row, w.ref_seqs)
    eng = E.engine_for_workload(w)
    eng.load_queries(w.query_seqs)
    mu = O.prior_means(w.parent, w.bl, 0)
    edges = np.where(w.parent >= 0)[0]
    trials = []
    for q, e in ((0, edges[5]), (1, edges[17]), (2, edges[29]), (3, edges[41]), (4, edges[53])):
        like, p, d = O.polish(oref, w.query_seqs[q], int(e), 0.1, float(w.bl[e]) / 2)
        trials.append((q, int(e), p, d, 0.01))
    got = eng.trials(trials, optimizer=E.NEWTON, mode=2, prefs=E.default_prefs(prior=prior, pp_rule=1))
    close = 0
    for (q, e, p, d, _), g in zip(trials, got):
        ref_m, info = _qng_oracle_marginal(oref, w.query_seqs[q], e, p, d, prior, mu[e], 0.01)
        assert g["status"] == 0 and abs(g["like"] - ref_m) <= 0.0101, (q, e, g["like"], ref_m, info)
        close += abs(g["like"] - ref_m) <= 1e-3
    assert close >= len(trials) - 1


def test_marginal_qng_retries_exhausted(oracle_lib):
    """pp_rule 1 at the smallest relative error QNG accepts (just above 50
    DBL_EPSILON): no stage meets it on the FP32-evaluated integrand, so every
    attempt ends in ETOL, the upper limit halves ten times, and the result is
    the base likelihood, the trial's own evaluation at the optimum
    (three_tax.ml:177-183).  A converged integral (the oracle's, at 0.01)
    lies well below it, so the two outcomes are told apart."""
    from pplacer_gb300 import engine as E
    from pplacer_gb300 import synth
    O = oracle_lib
    w = synth.make_workload("cpu_small", n_queries=3, taxa=60, sites=400, lo=100, hi=300)
    oref = O.Reference(O.Model(w.exch, w.statd, w.rates), w.parent, w.bl, w.leaf_row, w.ref_seqs)
    eng = E.engine_for_workload(w)
    eng.load_queries(w.query_seqs)
    edges = np.where(w.parent >= 0)[0]
    trials = []
    for q, e in ((0, edges[7]), (1, edges[19])):
        like, p, d = O.polish(oref, w.query_seqs[q], int(e), 0.1, float(w.bl[e]) / 2)
        trials.append((q, int(e), p, d, 0.01))
    prefs = E.default_prefs(prior=1, pp_rule=1, pp_rel_err=1.2e-14)
    got = eng.trials(trials, optimizer=E.NEWTON, mode=2, prefs=prefs)
    at = eng.trials(trials, optimizer=E.NEWTON, mode=1, prefs=prefs)
    for (q, e, p, d, _), g, a in zip(trials, got, at):
        ref_m, info = _qng_oracle_marginal(oref, w.query_seqs[q], e, p, d, 1, None, 0.01)
        assert g["status"] == 0 and abs(g["like"] - a["like"]) <= 1e-7 * abs(a["like"]), (g, a)
        assert ref_m < a["like"] - 0.05, (ref_m, a["like"])


def test_qng_tolerance_below_gsl_minimum_is_rejected():
    """pp_rule 1 refuses a pp_rel_err below 50 DBL_EPSILON, where GSL's qng
    returns GSL_EBADTOL."""
    import ctypes as C
    from pplacer_gb300 import engine as E
    from pplacer_gb300 import lib as L
    from pplacer_gb300 import synth
    w = synth.make_workload("cpu_small", n_queries=2)
    eng = E.engine_for_workload(w)
    eng.load_queries(w.query_seqs)
    prefs = E.default_prefs(pp_rule=1, pp_rel_err=1e-15, calc_pp=1)
    assert L.load().pgb_queries_run(eng.h, C.byref(prefs)) == 1
    assert b"pp_rel_err" in L.load().pgb_last_error()


def test_place_pp_qng_replica(oracle_lib):
    """Whole queries with calc_pp and pp_rule 1: each kept placement's
    marginal likelihood against the oracle's calc_marg_prob at the GPU's
    refined lengths, and post_prob their normalised ratios."""
    import math
    from pplacer_gb300 import engine as E
    from pplacer_gb300 import synth
    O = oracle_lib
    w = synth.make_workload("cpu_small", n_queries=5, taxa=60, sites=400, lo=100, hi=300)
    oref = O.Reference(O.Model(w.exch, w.statd, w.rates), w.parent, w.bl, w.leaf_row, w.ref_seqs)
    eng = E.engine_for_workload(w)
    mu = O.prior_means(w.parent, w.bl, 0)
    res, st = eng.place(w.query_seqs, E.default_prefs(optimizer=1, calc_pp=1, prior=0, pp_rule=1))
    n = 0
    for q, rows in enumerate(res):
        if not rows:
            continue
        for (e, like, lwr, dist, pend, pp, ml) in rows[:2]:
            ref_m, info = _qng_oracle_marginal(oref, w.query_seqs[q], e, pend, dist, 0, mu[e], 0.01)
            assert abs(ml - ref_m) <= 0.0101, (q, e, ml, ref_m, info)
            n += 1
        mls = [r[6] for r in rows]
        top = max(mls)
        tot = sum(math.exp(m - top) for m in mls)
        for r in rows:
            assert abs(r[5] - math.exp(r[6] - top) / tot) <= 1e-9
    assert n >= 5


def test_refine_categories(oracle_lib):
    """Gcat site-category refinement (gcat_model.ml:387-419) against the
    oracle, then placement with the refined categories."""
    from pplacer_gb300 import engine as E
    from pplacer_gb300 import synth
    from pplacer_gb300.model import Model
    O = oracle_lib
    w = synth.make_workload("cat_5k", n_queries=12, taxa=80, sites=300, lo=60, hi=300)
    S = w.n_sites
    want, scores = O.refine_categories(w.exch, w.statd, w.rates, w.parent, w.bl, w.leaf_row, w.ref_seqs)
    eng = E.Engine(Model.from_exchangeabilities(w.exch, w.statd, w.rates, np.zeros(S, dtype=np.int32)),
                   w.parent, w.bl)
    got = eng.refine_categories(w.leaf_row, w.ref_seqs)
    srt = np.sort(scores, axis=0)
    gap = srt[-1] - srt[-2]
    diff = got != want
    assert np.all(gap[diff] <= 1e-9 * np.abs(srt[-1][diff])), (np.where(diff), gap[diff])
    assert diff.sum() <= 0.01 * S
    eng.precompute(w.leaf_row, w.ref_seqs)
    oref = O.Reference(O.Model(w.exch, w.statd, w.rates, got), w.parent, w.bl, w.leaf_row, w.ref_seqs)
    ores, ost = oref.place(w.query_seqs, O.make_prefs(), n_threads=8)
    gres, gst = eng.place(w.query_seqs, E.default_prefs(optimizer=1))
    assert list(gst) == list(ost)
    _compare_placements(O, oref, w.query_seqs, gres, ores)


def test_place_host_batches(small, monkeypatch):
    """pgb_place (host buffers, device batches) gives the load/run/fetch
    results, with batches of 7 queries."""
    from pplacer_gb300 import engine as E
    w, oref, eng = small
    qs = w.query_seqs[:20]
    want, wst = eng.place(qs, E.default_prefs())
    monkeypatch.setenv("PGB_PLACE_BATCH", "7")
    got, gst = eng.place_host(qs, E.default_prefs())
    got5, gst5 = eng.place_host(qs, E.default_prefs(), batch=5)  # the caller's batch size (pgb_place_batch)
    for gg, ss in ((got, gst), (got5, gst5)):
        assert list(ss) == list(wst)
        for g, r in zip(gg, want):
            assert [p[0] for p in g] == [p[0] for p in r]
            for a, b in zip(g, r):
                assert a[1] == b[1] and a[3] == b[3] and a[4] == b[4]


def test_place_batch_from_page_locked_buffers(small):
    """pgb_place_batch with the query rows and the results in page-locked
    host memory from pgb_host_alloc: the same placements as load/run/fetch."""
    import ctypes as C
    from pplacer_gb300 import engine as E
    from pplacer_gb300 import lib as L
    w, oref, eng = small
    qs = w.query_seqs[:20]
    prefs = E.default_prefs()
    want, wst = eng.place(qs, prefs)
    Q, S, kam = len(qs), len(qs[0]), prefs.keep_at_most
    hin = L.HostBuffer(Q * S)
    hin.array(np.uint8, Q * S)[:] = np.frombuffer("".join(qs).encode(), dtype=np.uint8)
    psz = C.sizeof(L.Placement)
    hout = L.HostBuffer(Q * kam * psz + 8 * Q)
    L.check(L.load().pgb_place_batch(eng.h, C.byref(prefs), Q, hin.address, 6, hout.address,
                                     hout.address + Q * kam * psz, hout.address + Q * kam * psz + 4 * Q),
            "pgb_place_batch")
    out = (L.Placement * (Q * kam)).from_address(hout.address)
    tail = hout.array(np.int32, (Q * kam * psz) // 4 + 2 * Q)
    n_out, qst = tail[-2 * Q:-Q], tail[-Q:]
    assert list(qst) == list(wst)
    for q in range(Q):
        got = [(out[q * kam + i].edge, out[q * kam + i].like, out[q * kam + i].dist, out[q * kam + i].pend)
               for i in range(n_out[q])]
        assert got == [(r[0], r[1], r[3], r[4]) for r in want[q]]
    hin.close()
    hout.close()


def test_dropin_flow_vs_oracle(oracle_lib):
    """pplacer's per-query flow over the plain per-call drop-in (the measured
    Brent arm of the benchmark, dropin_flow.place_query): the same placements
    as the oracle's FP64 restatement of that flow, up to the FP32 rounding of
    the GLVs it reads back from the engine."""
    from pplacer_gb300 import dropin_flow as DF
    from pplacer_gb300 import engine as E
    from pplacer_gb300 import synth
    O = oracle_lib
    w = synth.make_workload("cpu_small", n_queries=3, taxa=30, sites=240, lo=80, hi=200)
    eng = E.engine_for_workload(w)
    m = eng.model
    model = DF.Model(m.statd, m.x, m.lam, m.xit, m.rates)
    edges = [i for i in range(len(w.parent)) if w.parent[i] >= 0]
    darr = {i: DF.Glv(*eng.get_glv(0, i)) for i in edges}
    parr = {i: DF.Glv(*eng.get_glv(1, i)) for i in edges}
    snodes = {i: DF.Glv(*eng.get_glv(2, i)) for i in edges}
    op = O.make_prefs()
    pf = {k: getattr(op, k) for k in ("start_pend", "max_pend", "initial_tolerance", "max_pitches", "max_strikes",
                                      "strike_box", "keep_at_most", "keep_factor")}
    oref = O.Reference(O.Model(w.exch, w.statd, w.rates), w.parent, w.bl, w.leaf_row, w.ref_seqs)
    ores, _ = oref.place(w.query_seqs, op)
    for q in range(3):
        res, calls = DF.place_query(model, w.query_seqs[q], darr, parr, snodes, w.bl, edges, pf)
        assert calls > 0 and res
        assert abs(sum(p[2] for p in res) - 1.0) < 1e-9
        ge, gl = res[0][0], res[0][1]
        oe, ol = ores[q][0][0], ores[q][0][1]
        if ge != oe:  # a tie: the same point seen from two edges
            g_star = O.polish(oref, w.query_seqs[q], ge, res[0][4], res[0][3])[0]
            o_star = O.polish(oref, w.query_seqs[q], oe, ores[q][0][4], ores[q][0][3])[0]
            assert abs(g_star - o_star) <= 1e-6 * abs(o_star), (q, ge, oe)
        assert abs(gl - ol) <= 1e-5 * abs(ol), (q, gl, ol)


def test_long_queries_gradients_and_placement(oracle_lib):
    """dna_2k shapes (3,000 sites, queries up to 3,000 informative sites):
    1,000 sampled (query, edge, pendant, distal) points, GPU value and adjoint
    against the FP64 oracle; central differences (h = 1e-6) of the oracle's
    FP64 value against its analytic gradient on 50 of them; and Newton
    placements against the oracle."""
    from pplacer_gb300 import engine as E
    from pplacer_gb300 import synth
    O = oracle_lib
    w = synth.make_workload("dna_2k", n_queries=40, taxa=300, lo=1500, hi=3000)
    oref = O.Reference(O.Model(w.exch, w.statd, w.rates), w.parent, w.bl, w.leaf_row, w.ref_seqs)
    eng = E.engine_for_workload(w)
    eng.load_queries(w.query_seqs)
    rng = np.random.default_rng(11)
    edges = np.where(w.parent >= 0)[0]
    pts = []
    for _ in range(1000):
        q = int(rng.integers(len(w.query_seqs)))
        e = int(rng.choice(edges))
        pts.append((q, e, float(rng.uniform(1e-3, 0.3)), float(rng.uniform(0, w.bl[e])), 0.01))
    got = eng.trials(pts, optimizer=E.NEWTON, mode=1)
    for i, ((q, e, p, d, _), g) in enumerate(zip(pts, got)):
        st, ref = oref.loglike_derivs(w.query_seqs[q], e, p, d)
        assert abs(g["like"] - ref[0]) <= 2e-7 * abs(ref[0]), (q, e, g["like"], ref[0])
        hscale = math.sqrt(abs(ref[3] * ref[4])) + 1.0
        for k, (gv, rv) in enumerate(zip(g["derivs"][:5], ref[1:6])):
            tol = 2e-3 * abs(rv) + (1e-5 * abs(ref[3 + k]) + 1e-2 if k < 2 else 1e-3 * hscale + 1.0)
            assert abs(gv - rv) <= tol, (i, k, gv, rv)
        if i < 50:
            h = 1e-6
            s = w.query_seqs[q]
            fp = (oref.loglike_derivs(s, e, p + h, d)[1][0] - oref.loglike_derivs(s, e, p - h, d)[1][0]) / (2 * h)
            assert abs(fp - ref[1]) <= 1e-6 * abs(ref[1]) + 4e-16 * abs(ref[0]) / h
    ores, ost = oref.place(w.query_seqs, O.make_prefs(), n_threads=8)
    for optimizer, frac in ((1, 1.0), (0, 0.95)):
        gres, gst = eng.place(w.query_seqs, E.default_prefs(optimizer=optimizer))
        assert list(gst) == list(ost)
        _compare_placements(O, oref, w.query_seqs, gres, ores, newton=optimizer == 1, min_logl_frac=frac)
