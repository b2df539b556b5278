"""pplacer's per-query placement flow over the plain drop-in.

This is what an unmodified pplacer does when its ``Linear`` externals
(pplacer_src/linear.ml:13-89) are bound to this library one for one: the
OCaml side keeps its FP64 GLVs on the host and every numeric kernel is one
call through the C ABI (a host-to-device copy, one kernel, a copy back).
The flow restates ``Core.pplacer_core.process_query`` (core.ml:113-409) for
Gamma mixtures (Gmix_model): stage-1 ``Glv.masked_logdot`` against every
supernode (core.ml:187-197), the ranking (fig.ml:143-147 with figs off), the
baseball of alternating Brent searches at the initial tolerance
(core.ml:283-318, three_tax.ml:48-83, minimization.ml:24-41,83-101), keep,
refinement at 1e-5 and like_weight_ratio (core.ml:336-377).  Brent follows
GSL's published algorithm (golden section 0.3819660, parabolic steps,
sqrt(DBL_EPSILON)|x| minimal step) as ``Gsl.Min.BRENT`` does.

It exists to measure that arm: the batched engine replaces exactly this.
"""
import math

import numpy as np

from . import linear as Lin
from .model import lv_of_char

LN2 = math.log(2.0)
SQRT_DBL_EPS = 1.4901161193847656e-08
GOLDEN = 0.3819660


class GslError(Exception):
    pass


class ExceededMaxIter(Exception):
    pass


class FindStartFailure(Exception):
    pass


class Glv:
    """A Gmix GLV: planes a [R][S][K] and per-site exponents e [S]."""

    def __init__(self, a, e):
        self.a = np.ascontiguousarray(a, dtype=np.float64)
        self.e = np.ascontiguousarray(e, dtype=np.int64)


class Model:
    """The Gmix model fields the flow uses: statd, Diagd (x, lambda, xit), rates."""

    def __init__(self, statd, x, lam, xit, rates):
        self.statd = np.ascontiguousarray(statd, dtype=np.float64)
        self.x = np.ascontiguousarray(x, dtype=np.float64)
        self.lam = np.ascontiguousarray(lam, dtype=np.float64)
        self.xit = np.ascontiguousarray(xit, dtype=np.float64)
        self.rates = [float(r) for r in rates]
        self.K = len(self.statd)
        self._P = np.zeros((self.K, self.K))

    def evolve_into(self, dst, src, bl):
        """Gmix_model.evolve_into (gmix_model.ml:308-315): exponents copied,
        per rate one dediagonalize of exp(rate bl lambda) and one gemmish."""
        dst.e[:] = src.e
        for r, rate in enumerate(self.rates):
            Lin.dediagonalize(self._P, self.x, np.exp(rate * bl * self.lam), self.xit)
            Lin.gemmish(dst.a[r], self._P, src.a[r])

    def log_like3(self, util, x, y, z):
        """Gmix_model.log_like3 (gmix_model.ml:298-304)."""
        return (Lin.ten_log_like3(self.statd, x.a, y.a, z.a, util)
                + LN2 * float(x.e.sum() + y.e.sum() + z.e.sum()))

    def masked_logdot(self, util, x, y, mask):
        """Glv.masked_logdot (gmix_model.ml:194-198)."""
        m = mask.astype(bool)
        return Lin.ten_masked_logdot(x.a, y.a, mask, util) + LN2 * float(x.e[m].sum() + y.e[m].sum())


class Edge:
    """Glv_edge (glv_edge.ml): an original GLV, its evolved copy, a length."""

    def __init__(self, model, orig, bl):
        self.model, self.orig, self.bl = model, orig, bl
        self.evolv = Glv(orig.a.copy(), orig.e.copy())
        self.recalculate()

    def recalculate(self):
        self.model.evolve_into(self.evolv, self.orig, self.bl)

    def set_bl(self, bl):
        self.bl = bl
        self.recalculate()


def _gsl_brent(f, x_min, lower, upper, tol, max_iters):
    """Gsl.Min.BRENT from x_min in [lower, upper], stopped as
    minimization.ml:83-101 stops it (interval width below tol)."""
    f_min, f_low, f_up = f(x_min), f(lower), f(upper)
    if not (f_min < f_low and f_min < f_up):
        raise GslError("endpoints do not enclose a minimum")
    v = lower + GOLDEN * (upper - lower)
    w = v
    d = e = 0.0
    fv = fw = f(v)
    z, fz = x_min, f_min
    for _ in range(max_iters):
        dd, ee = e, d  # GSL's iteration takes d and e with their roles swapped
        wl, wu = z - lower, upper - z
        tolerance = SQRT_DBL_EPS * abs(z)
        mid = 0.5 * (lower + upper)
        p = q = r = 0.0
        if abs(ee) > tolerance:
            r = (z - w) * (fz - fv)
            q = (z - v) * (fz - fw)
            p = (z - v) * q - (z - w) * r
            q = 2.0 * (q - r)
            if q > 0:
                p = -p
            else:
                q = -q
            r, ee = ee, dd
        if abs(p) < abs(0.5 * q * r) and p < q * wl and p < q * wu:
            t2 = 2.0 * tolerance
            dd = p / q
            u = z + dd
            if (u - lower) < t2 or (upper - u) < t2:
                dd = tolerance if z < mid else -tolerance
        else:
            ee = (upper - z) if z < mid else -(z - lower)
            dd = GOLDEN * ee
        u = z + dd if abs(dd) >= tolerance else z + (tolerance if dd > 0 else -tolerance)
        e, d = ee, dd
        fu = f(u)
        if fu <= fz:
            if u < z:
                upper = z
            else:
                lower = z
            v, fv, w, fw, z, fz = w, fw, z, fz, u, fu
        else:
            if u < z:
                lower = u
            else:
                upper = u
            if fu <= fw or w == z:
                v, fv, w, fw = w, fw, u, fu
            elif fu <= fv or v == z or v == w:
                v, fv = u, fu
        if upper - lower < tol:
            return z
    raise ExceededMaxIter()


def brent(f, raw_start, left, right, tol, max_iters=100):
    """Minimization.brent with the bisection start finder (minimization.ml:11-41,83-101)."""
    if left >= raw_start or raw_start >= right:
        raise GslError("invalid start values")
    fl, fr = f(left), f(right)
    smaller, miny = (left, fl) if fl < fr else (right, fr)
    start = raw_start
    for it in range(1, max_iters + 2):
        fs = f(start)
        if fs < miny:
            break
        if abs(start - smaller) < tol:
            return smaller  # FoundMin (the start was not below miny)
        if it > max_iters:
            raise FindStartFailure()
        start = 0.5 * (start + smaller)
    return _gsl_brent(f, start, left, right, tol, max_iters)


class ThreeTax:
    """Three_tax (three_tax.ml:15-83) on the drop-in."""

    def __init__(self, model, util, prox, dist, pend):
        self.m, self.util, self.prox, self.dist, self.pend = model, util, prox, dist, pend
        self.n_like_calls = 0

    def log_like(self):
        return self.m.log_like3(self.util, self.prox.evolv, self.dist.evolv, self.pend.evolv)

    def set_dist_bl(self, d):
        cut = self.dist.bl + self.prox.bl
        self.dist.set_bl(d)
        self.prox.set_bl(cut - d)

    def _opt(self, tol, setter, start, lo, hi):
        if lo == hi:
            return start

        def f(v):
            self.n_like_calls += 1
            setter(v)
            return -self.log_like()
        return brent(f, start, lo, hi, tol)

    def optimize(self, tol, max_pend, max_iter=200):
        prev_p, prev_d = self.pend.bl, self.dist.bl
        for _ in range(max_iter):
            cp = self._opt(tol, self.pend.set_bl, self.pend.bl, 1e-8, max_pend)
            cd = self._opt(tol, self.set_dist_bl, self.dist.bl, 0.0, self.dist.bl + self.prox.bl)
            if abs(prev_p - cp) <= tol and abs(prev_d - cd) <= tol:
                return
            prev_p, prev_d = cp, cd
        raise ExceededMaxIter()


def place_query(model, seq, darr, parr, snodes, bl, edges, prefs):
    """One query through process_query (core.ml:113-409); returns the sorted
    placements [(edge, like, lwr, distal, pendant)] and the number of
    likelihood evaluations of its Brent searches."""
    K = model.K
    S = len(seq)
    R = len(model.rates)
    lv = np.array([lv_of_char(c, K) for c in seq])
    full_orig = Glv(np.broadcast_to(lv, (R, S, K)).copy(), np.zeros(S))
    full_evolv = Glv(np.zeros((R, S, K)), np.zeros(S))
    model.evolve_into(full_evolv, full_orig, prefs["start_pend"])
    mask_arr = np.array([c not in "-?" for c in seq])
    mask_vec = np.ascontiguousarray(mask_arr.astype(np.uint16))
    reind = np.nonzero(mask_arr)[0]
    utilv = np.zeros(S)
    # stage 1 (core.ml:187-197) and the ranking (fig.ml:143-147): descending,
    # ties by edge order
    scores = [model.masked_logdot(utilv, full_evolv, snodes[e], mask_vec) for e in edges]
    ranking = sorted(range(len(edges)), key=lambda i: (-scores[i], i))
    q_lv = np.ascontiguousarray(np.broadcast_to(lv[reind], (R, len(reind), K)))
    query = Glv(q_lv.copy(), np.zeros(len(reind)))

    def masked(g):
        return Glv(g.a[:, reind, :].copy(), g.e[reind].copy())
    sp = prefs["start_pend"]
    dist_e = Edge(model, Glv(np.zeros_like(q_lv), np.zeros(len(reind))), sp)
    prox_e = Edge(model, Glv(np.zeros_like(q_lv), np.zeros(len(reind))), sp)
    pend_e = Edge(model, query, sp)
    tt = ThreeTax(model, np.zeros(len(reind)), prox_e, dist_e, pend_e)
    calls = 0

    def set_tt_edges(loc, pendant, distal):
        pend_e.set_bl(pendant)
        dist_e.orig = masked(darr[loc])
        dist_e.set_bl(distal)
        prox_e.orig = masked(parr[loc])
        prox_e.set_bl(bl[loc] - distal)

    def optimize_at(loc, tol):
        nonlocal calls
        tt.n_like_calls = 0
        try:
            tt.optimize(tol, prefs["max_pend"])
        except ExceededMaxIter:
            pass
        calls += tt.n_like_calls
        return tt.log_like(), pend_e.bl, dist_e.bl

    def safe_optimize(loc, tol):
        try:
            return optimize_at(loc, tol)
        except GslError:
            set_tt_edges(loc, sp, bl[loc] / 2.0)
            return optimize_at(loc, tol)
    results = []
    like_record, strikes = -math.inf, 0
    for i in ranking:  # play_ball (core.ml:283-318)
        loc = edges[i]
        set_tt_edges(loc, sp, bl[loc] / 2.0)
        try:
            res = safe_optimize(loc, prefs["initial_tolerance"])
        except (GslError, FindStartFailure):
            continue
        prior = results
        results = results + [(loc, res)]
        like = res[0]
        if len(prior) >= prefs["max_pitches"]:
            break
        if like > like_record:
            like_record = like
        elif like < like_record - prefs["strike_box"]:
            strikes += 1
            if strikes >= prefs["max_strikes"]:
                break
    srt = sorted(results, key=lambda r: -r[1][0])
    best = srt[0][1][0]
    keep = [r for j, r in enumerate(srt) if j < prefs["keep_at_most"] and r[1][0] >= math.log(prefs["keep_factor"]) + best]
    refined = []
    for loc, (_, p, d) in keep:  # final refinement at 1e-5 (core.ml:353-369)
        set_tt_edges(loc, p, d)
        try:
            refined.append((loc, safe_optimize(loc, 1e-5)))
        except (GslError, FindStartFailure):
            refined.append((loc, (_, p, d)))
    likes = np.array([r[1][0] for r in refined])
    w = np.exp(likes - likes.max())
    lwr = w / w.sum()
    out = [(loc, l, float(r), d, p) for (loc, (l, p, d)), r in zip(refined, lwr)]
    out.sort(key=lambda t: -t[2])
    return out, calls
