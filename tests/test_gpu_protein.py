"""20-state Gamma-mixture trials against the FP64 oracle, in both kernel
forms: the tensor-core CTA (tcgen05 3xTF32 evolves, tuning code 1) and the
CUDA-core CTA (256 threads, windows in shared memory).  Queries up to 300
sites span three 128-site MMA tiles; some carry ambiguity characters.  The
posterior probabilities of the round-based path (20 states, CAT) against
the oracle's quadrature.

Tolerances as in test_gpu_engine: fixed-point logL 2e-7 relative, optimised
logL 1e-6 relative, best edge identical for non-tied queries."""
import math

import numpy as np
import pytest

from test_gpu_engine import _compare_placements

pytestmark = pytest.mark.gpu

FORMS = {"tc": (1, 0), "cta": (256, 1)}


@pytest.fixture(scope="module")
def protein(oracle_lib):
    from pplacer_gb300 import synth
    w = synth.make_workload("aa_500", n_queries=40, taxa=60, sites=300, lo=40, hi=300)
    seqs = list(w.query_seqs)
    # ambiguity characters (B, Z, X) in every fifth query
    for q in range(0, len(seqs), 5):
        s = list(seqs[q])
        idx = [i for i, c in enumerate(s) if c not in "-?"]
        for k, i in enumerate(idx[::9]):
            s[i] = "BZX"[k % 3]
        seqs[q] = "".join(s)
    w.query_seqs = seqs
    O = oracle_lib
    oref = O.Reference(O.Model(w.exch, w.statd, w.rates), w.parent, w.bl, w.leaf_row, w.ref_seqs)
    return w, oref


@pytest.mark.parametrize("form", sorted(FORMS))
def test_protein_loglike_and_derivatives(protein, form):
    from pplacer_gb300 import engine as E
    w, oref = protein
    eng = E.engine_for_workload(w)
    eng.set_tuning(*FORMS[form])
    eng.load_queries(w.query_seqs)
    rng = np.random.default_rng(7)
    edges = np.where(w.parent >= 0)[0]
    trials = []
    for _ in range(40):
        q = int(rng.integers(len(w.query_seqs)))
        e = int(rng.choice(edges))
        trials.append((q, e, float(rng.uniform(1e-8, 0.5)), float(rng.uniform(0, w.bl[e])), 0.01))
    got = eng.trials(trials, optimizer=E.NEWTON, mode=1)
    for (q, e, p, d, _), g in zip(trials, got):
        st, ref = oref.loglike_derivs(w.query_seqs[q], e, p, d)
        assert st == 0
        assert abs(g["like"] - ref[0]) <= 2e-7 * abs(ref[0]), (q, e, g["like"], ref[0])
        hscale = math.sqrt(abs(ref[3] * ref[4])) + 1.0
        for k, (gv, rv) in enumerate(zip(g["derivs"][:5], ref[1:6])):
            tol = 2e-3 * abs(rv) + (1e-5 * abs(ref[3 + k]) + 1e-2 if k < 2 else 1e-3 * hscale + 1.0)
            assert abs(gv - rv) <= tol, (k, gv, rv)


@pytest.mark.parametrize("optimizer", [0, 1])
@pytest.mark.parametrize("form", sorted(FORMS))
def test_protein_placements(protein, oracle_lib, form, optimizer):
    from pplacer_gb300 import engine as E
    O = oracle_lib
    w, oref = protein
    ores, ost = oref.place(w.query_seqs, O.make_prefs(), n_threads=8)
    eng = E.engine_for_workload(w)
    eng.set_tuning(*FORMS[form])
    assert list(eng.get_tuning()[0]) == [FORMS[form][0]] * 6
    gres, gst = eng.place(w.query_seqs, E.default_prefs(optimizer=optimizer))
    assert list(gst) == list(ost)
    _compare_placements(O, oref, w.query_seqs, gres, ores, newton=optimizer == 1,
                        min_logl_frac=1.0 if optimizer else 0.95)


def _check_pp(O, oref, w, res, prior, mu, nq=3):
    import math
    checked = 0
    for q in range(nq):
        places = res[q][:3]
        assert places and all(len(p) == 7 for p in places)
        want = []
        for (e, like, lwr, d, p, pp, m) in places:
            ref_m = O.marginal_like(oref, w.query_seqs[q], e, p, d, prior, None if mu is None else mu[e], rel=1e-8)
            assert abs(m - ref_m) <= 2e-3, (q, e, m, ref_m)
            want.append(ref_m)
            checked += 1
        if len(res[q]) == len(places):
            mx = max(want)
            tot = sum(math.exp(v - mx) for v in want)
            for (_, _, _, _, _, pp, _), v in zip(places, want):
                assert abs(pp - math.exp(v - mx) / tot) <= 2e-3
        assert abs(sum(p[5] for p in res[q]) - 1.0) < 1e-9
    assert checked >= 3


@pytest.mark.parametrize("form", sorted(FORMS))
def test_protein_posterior_probabilities(oracle_lib, form):
    """calc_pp on the round-based path: one marginal-likelihood trial per
    kept location after the refinements, in either kernel form, against the
    FP64 quadrature of the same integral (three_tax.ml:169-215)."""
    from pplacer_gb300 import engine as E
    from pplacer_gb300 import synth
    O = oracle_lib
    w = synth.make_workload("aa_500", n_queries=3, taxa=30, sites=200, lo=80, hi=200)
    oref = O.Reference(O.Model(w.exch, w.statd, w.rates), w.parent, w.bl, w.leaf_row, w.ref_seqs)
    eng = E.engine_for_workload(w)
    eng.set_tuning(*FORMS[form])
    prior = 0
    res, st = eng.place(w.query_seqs, E.default_prefs(calc_pp=1, prior=prior, prior_lower=0.01))
    assert list(st) == [0, 0, 0]
    _check_pp(O, oref, w, res, prior, O.prior_means(w.parent, w.bl, prior, prior_lower=0.01))


def test_cat_posterior_probabilities(oracle_lib):
    """calc_pp for a per-site CAT model (Gcat_model) on the CTA kernel."""
    from pplacer_gb300 import engine as E
    from pplacer_gb300 import synth
    O = oracle_lib
    w = synth.make_workload("cat_5k", n_queries=3, taxa=40, sites=300, lo=100, hi=300)
    oref = O.Reference(O.Model(w.exch, w.statd, w.rates, w.site_cats), w.parent, w.bl, w.leaf_row, w.ref_seqs)
    eng = E.engine_for_workload(w)
    prior = 1
    res, st = eng.place(w.query_seqs, E.default_prefs(calc_pp=1, prior=prior))
    assert list(st) == [0, 0, 0]
    _check_pp(O, oref, w, res, prior, None)


def test_round_based_path(oracle_lib):
    """Bins tuned to different CTA sizes take the round-based path (baseball
    rounds, k_keep_emit, k_pp_emit, k_finalize) instead of whole queries:
    placements and posterior probabilities against the oracle."""
    from pplacer_gb300 import engine as E
    from pplacer_gb300 import synth
    O = oracle_lib
    w = synth.make_workload("cat_5k", n_queries=12, taxa=40, sites=300, lo=100, hi=300)
    oref = O.Reference(O.Model(w.exch, w.statd, w.rates, w.site_cats), w.parent, w.bl, w.leaf_row, w.ref_seqs)
    eng = E.engine_for_workload(w)
    eng.set_tuning([256, 128, 256, 128, 256, 128], [1, 0, 1, 0, 1, 0])
    ores, ost = oref.place(w.query_seqs, O.make_prefs(), n_threads=8)
    gres, gst = eng.place(w.query_seqs, E.default_prefs(optimizer=1))
    assert list(gst) == list(ost)
    assert eng.timings()[1][7] > 1  # more than one baseball round
    _compare_placements(O, oref, w.query_seqs, gres, ores)
    prior = 1
    res, st = eng.place(w.query_seqs[:3], E.default_prefs(calc_pp=1, prior=prior))
    assert list(st) == [0, 0, 0]
    w.query_seqs = w.query_seqs[:3]
    _check_pp(O, oref, w, res, prior, None)


@pytest.mark.parametrize("form", [(32, 0), (32, 1), (32, 2), (128, 1)], ids=["warp", "warp_eig", "warp_eig2", "cta"])
def test_cat_forms(oracle_lib, form):
    """Per-site CAT placements in the whole-query warp forms (sites_warp_cat:
    each lane's site reads its category's matrices; sites_warp_cat_eig: the
    eigenbasis, each site's category entering through its exp factors;
    sites_warp_cat_eig2: the same on packed FP32 pairs) and the whole-query
    CTA form, against the oracle; queries long enough to span many
    categories."""
    from pplacer_gb300 import engine as E
    from pplacer_gb300 import synth
    O = oracle_lib
    w = synth.make_workload("cat_5k", n_queries=30, taxa=120, sites=600, lo=100, hi=600)
    oref = O.Reference(O.Model(w.exch, w.statd, w.rates, w.site_cats), w.parent, w.bl, w.leaf_row, w.ref_seqs)
    ores, ost = oref.place(w.query_seqs, O.make_prefs(), n_threads=8)
    eng = E.engine_for_workload(w)
    eng.set_tuning(*form)
    for optimizer, frac in ((1, 1.0), (0, 0.95)):
        gres, gst = eng.place(w.query_seqs, E.default_prefs(optimizer=optimizer))
        assert list(gst) == list(ost)
        _compare_placements(O, oref, w.query_seqs, gres, ores, newton=optimizer == 1, min_logl_frac=frac)
    # the fixed-point likelihood and derivatives of the warp trials
    eng.load_queries(w.query_seqs)
    rng = np.random.default_rng(3)
    edges = np.where(w.parent >= 0)[0]
    trials = []
    for _ in range(30):
        q = int(rng.integers(len(w.query_seqs)))
        e = int(rng.choice(edges))
        trials.append((q, e, float(rng.uniform(1e-8, 0.5)), float(rng.uniform(0, w.bl[e])), 0.01))
    got = eng.trials(trials, optimizer=E.NEWTON, mode=1)
    for (q, e, p, d, _), g in zip(trials, got):
        st, ref = oref.loglike_derivs(w.query_seqs[q], e, p, d)
        assert abs(g["like"] - ref[0]) <= 2e-7 * abs(ref[0]), (q, e, g["like"], ref[0])
        hscale = math.sqrt(abs(ref[3] * ref[4])) + 1.0
        for k, (gv, rv) in enumerate(zip(g["derivs"][:5], ref[1:6])):
            tol = 2e-3 * abs(rv) + (1e-5 * abs(ref[3 + k]) + 1e-2 if k < 2 else 1e-3 * hscale + 1.0)
            assert abs(gv - rv) <= tol, (k, gv, rv)
