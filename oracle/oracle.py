"""ORACLE -- test infrastructure only.

ctypes binding for the FP64 CPU restatement of pplacer's placement path
(oracle/oracle.cpp -> oracle/_build/liboracle.so) and for the reference's own
pplacer_src/linear_c.c compiled against oracle/shim (oracle/_ref/liblinear_ref.so).

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg import
this module, and only as the checker; the product package never does.
"""
import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ORACLE_SO = os.path.join(HERE, "_build", "liboracle.so")
REF_SO = os.path.join(HERE, "_ref", "liblinear_ref.so")

_dp = np.ctypeslib.ndpointer(dtype=np.float64, flags="C_CONTIGUOUS")
_ip = np.ctypeslib.ndpointer(dtype=np.int32, flags="C_CONTIGUOUS")
_u16p = np.ctypeslib.ndpointer(dtype=np.uint16, flags="C_CONTIGUOUS")


def build(with_ref=True):
    """Compile the oracle (and, where the reference sources exist, oracle/_ref)."""
    target = "all" if with_ref else "_build/liboracle.so"
    subprocess.run(["make", "-s", "-C", HERE, target], check=True)


_lib = None
_ref = None


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(ORACLE_SO):
            build(with_ref=False)
        L = C.CDLL(ORACLE_SO)
        d, i = C.c_double, C.c_int
        L.orc_gemmish.argtypes = [_dp, _dp, _dp, i, i]
        L.orc_dediagonalize.argtypes = [_dp, _dp, _dp, _dp, i]
        L.orc_mat_log_like3.argtypes = [_dp, _dp, _dp, _dp, i, i]
        L.orc_mat_log_like3.restype = d
        L.orc_pairwise_prod.argtypes = [_dp, _dp, _dp, C.c_long]
        L.orc_statd_pairwise_prod.argtypes = [_dp, _dp, _dp, _dp, C.c_long, i]
        L.orc_mat_masked_logdot.argtypes = [_dp, _dp, _u16p, i, i]
        L.orc_mat_masked_logdot.restype = d
        L.orc_mat_bounded_logdot.argtypes = [_dp, _dp, i, i, i]
        L.orc_mat_bounded_logdot.restype = d
        L.orc_ten_log_like3.argtypes = [_dp, _dp, _dp, _dp, _dp, i, i, i]
        L.orc_ten_log_like3.restype = d
        L.orc_ten_masked_logdot.argtypes = [_dp, _dp, _u16p, _dp, i, i, i]
        L.orc_ten_masked_logdot.restype = d
        L.orc_ten_bounded_logdot.argtypes = [_dp, _dp, i, i, _dp, i, i, i]
        L.orc_ten_bounded_logdot.restype = d
        L.orc_discrete_gamma.argtypes = [i, d, _dp]
        L.orc_gamma_p.argtypes = [d, d]
        L.orc_gamma_p.restype = d
        L.orc_diagd_of_d_b.argtypes = [i, _dp, _dp, _dp, _dp, _dp]
        L.orc_diagd_normed.argtypes = [i, _dp, _dp, _dp, _dp, _dp]
        L.orc_diagd_to_exp.argtypes = [i, _dp, _dp, _dp, d, _dp]
        L.orc_model_new.argtypes = [i, _dp, _dp, i, _dp, i, C.c_void_p]
        L.orc_model_new.restype = C.c_void_p
        L.orc_model_diagd.argtypes = [C.c_void_p, _dp, _dp, _dp]
        L.orc_model_free.argtypes = [C.c_void_p]
        L.orc_evolve.argtypes = [C.c_void_p, _dp, _ip, i, d, C.c_void_p, _dp, _ip]
        L.orc_ref_new.argtypes = [C.c_void_p, i, _ip, _dp, i, _ip, C.c_char_p, C.POINTER(C.c_void_p)]
        L.orc_ref_new.restype = i
        L.orc_ref_free.argtypes = [C.c_void_p]
        L.orc_ref_glv.argtypes = [C.c_void_p, i, i, _dp, _ip]
        L.orc_ref_edge_loglike.argtypes = [C.c_void_p, i, _dp]
        L.orc_ref_root_site_loglike.argtypes = [C.c_void_p, _dp]
        L.orc_place.argtypes = [C.c_void_p, C.c_void_p, i, C.c_char_p, i, C.c_void_p, _ip, _ip]
        L.orc_query_trace.argtypes = [C.c_void_p, C.c_void_p, C.c_char_p, _ip, _dp, C.POINTER(C.c_int), _ip, _dp,
                                      C.POINTER(C.c_int)]
        L.orc_query_trace.restype = i
        L.orc_optimize_location.argtypes = [C.c_void_p, C.c_void_p, C.c_char_p, i, d, d, d, _dp]
        L.orc_optimize_location.restype = i
        L.orc_loglike_derivs.argtypes = [C.c_void_p, C.c_char_p, i, d, d, _dp]
        L.orc_loglike_derivs.restype = i
        _lib = L
    return _lib


def ref_lib():
    """The reference's own linear_c.c (None where it was not built)."""
    global _ref
    if _ref is None and os.path.exists(REF_SO):
        R = C.CDLL(REF_SO)
        d, i = C.c_double, C.c_int
        R.ref_gemmish.argtypes = [_dp, _dp, _dp, i, i]
        R.ref_dediagonalize.argtypes = [_dp, _dp, _dp, _dp, i]
        R.ref_mat_log_like3.argtypes = [_dp, _dp, _dp, _dp, i, i]
        R.ref_mat_log_like3.restype = d
        R.ref_mat_pairwise_prod.argtypes = [_dp, _dp, _dp, i, i]
        R.ref_mat_statd_pairwise_prod.argtypes = [_dp, _dp, _dp, _dp, i, i]
        R.ref_mat_masked_logdot.argtypes = [_dp, _dp, _u16p, i, i]
        R.ref_mat_masked_logdot.restype = d
        R.ref_mat_bounded_logdot.argtypes = [_dp, _dp, i, i, i, i]
        R.ref_mat_bounded_logdot.restype = d
        R.ref_ten_log_like3.argtypes = [_dp, _dp, _dp, _dp, _dp, i, i, i]
        R.ref_ten_log_like3.restype = d
        R.ref_ten_pairwise_prod.argtypes = [_dp, _dp, _dp, i, i, i]
        R.ref_ten_statd_pairwise_prod.argtypes = [_dp, _dp, _dp, _dp, i, i, i]
        R.ref_ten_masked_logdot.argtypes = [_dp, _dp, _u16p, _dp, i, i, i]
        R.ref_ten_masked_logdot.restype = d
        R.ref_ten_bounded_logdot.argtypes = [_dp, _dp, i, i, _dp, i, i, i]
        R.ref_ten_bounded_logdot.restype = d
        _ref = R
    return _ref


class OrcPrefs(C.Structure):
    _fields_ = [("start_pend", C.c_double), ("max_pend", C.c_double), ("initial_tolerance", C.c_double),
                ("max_strikes", C.c_int), ("strike_box", C.c_double), ("max_pitches", C.c_int),
                ("keep_at_most", C.c_int), ("keep_factor", C.c_double)]


class OrcPlacement(C.Structure):
    _fields_ = [("edge", C.c_int), ("pad", C.c_int), ("like", C.c_double), ("lwr", C.c_double),
                ("dist", C.c_double), ("pend", C.c_double)]


def make_prefs(**kw):
    p = dict(start_pend=0.1, max_pend=2.0, initial_tolerance=0.01, max_strikes=6, strike_box=3.0,
             max_pitches=40, keep_at_most=7, keep_factor=0.01)
    p.update(kw)
    return OrcPrefs(**p)


def discrete_gamma(n_cat, alpha):
    out = np.zeros(n_cat)
    lib().orc_discrete_gamma(n_cat, alpha, out)
    return out


def _f64(a):
    return np.ascontiguousarray(a, dtype=np.float64)


def diagd_normed(exch, statd):
    K = len(statd)
    x, l, xit = np.zeros((K, K)), np.zeros(K), np.zeros((K, K))
    lib().orc_diagd_normed(K, _f64(exch), _f64(statd), x, l, xit)
    return x, l, xit


def diagd_of_d_b(d, b):
    K = len(d)
    x, l, xit = np.zeros((K, K)), np.zeros(K), np.zeros((K, K))
    lib().orc_diagd_of_d_b(K, _f64(d), _f64(b), x, l, xit)
    return x, l, xit


def diagd_to_exp(x, l, xit, bl):
    K = len(l)
    out = np.zeros((K, K))
    lib().orc_diagd_to_exp(K, _f64(x), _f64(l), _f64(xit), bl, out)
    return out


class Model:
    """Gmix (site_cats None) or Gcat (per-site CAT categories) model."""

    def __init__(self, exch, statd, rates, site_cats=None):
        self.K = len(statd)
        self.rates = _f64(rates)
        self.gcat = site_cats is not None
        sc = np.ascontiguousarray(site_cats if self.gcat else [0], dtype=np.int32)
        self._sc = sc
        self.h = lib().orc_model_new(self.K, _f64(exch), _f64(statd), len(self.rates), self.rates,
                                     len(sc) if self.gcat else 0, sc.ctypes.data)
        self.R = 1 if self.gcat else len(self.rates)

    def diagd(self):
        K = self.K
        x, l, xit = np.zeros((K, K)), np.zeros(K), np.zeros((K, K))
        lib().orc_model_diagd(self.h, x, l, xit)
        return x, l, xit

    def __del__(self):
        if getattr(self, "h", None):
            lib().orc_model_free(self.h)
            self.h = None


class Reference:
    """darr / parr / snodes of a reference tree (FP64, oracle)."""

    def __init__(self, model, parent, bl, leaf_row, leaf_seqs):
        self.model = model
        self.parent = np.ascontiguousarray(parent, dtype=np.int32)
        self.bl = _f64(bl)
        self.n_nodes = len(self.parent)
        seqs = [s.encode() if isinstance(s, str) else s for s in leaf_seqs]
        self.S = len(seqs[0])
        buf = b"".join(seqs)
        h = C.c_void_p()
        rc = lib().orc_ref_new(model.h, self.n_nodes, self.parent, self.bl, self.S,
                               np.ascontiguousarray(leaf_row, dtype=np.int32), buf, C.byref(h))
        if rc != 0:
            raise RuntimeError("oracle reference build failed")
        self.h = h

    def glv(self, which, node):
        m = self.model
        a = np.zeros((m.R, self.S, m.K))
        e = np.zeros(self.S, dtype=np.int32)
        lib().orc_ref_glv(self.h, which, node, a, e)
        return a, e

    def edge_loglike(self, node):
        out = np.zeros(2)
        lib().orc_ref_edge_loglike(self.h, node, out)
        return out

    def root_site_loglike(self):
        """Per-site log likelihood of the whole tree (Like_stree.site_log_like_arr)."""
        out = np.zeros(self.S)
        lib().orc_ref_root_site_loglike(self.h, out)
        return out

    def place(self, seqs, prefs=None, n_threads=1):
        prefs = prefs or make_prefs()
        Q = len(seqs)
        buf = b"".join(s.encode() if isinstance(s, str) else s for s in seqs)
        kam = prefs.keep_at_most
        out = (OrcPlacement * (Q * kam))()
        n_out = np.zeros(Q, dtype=np.int32)
        status = np.zeros(Q, dtype=np.int32)
        lib().orc_place(self.h, C.byref(prefs), Q, buf, n_threads, out, n_out, status)
        res = []
        for q in range(Q):
            res.append([(out[q * kam + i].edge, out[q * kam + i].like, out[q * kam + i].lwr,
                         out[q * kam + i].dist, out[q * kam + i].pend) for i in range(n_out[q])])
        return res, status

    def trace(self, seq, prefs=None):
        prefs = prefs or make_prefs()
        n = self.n_nodes
        re, rs = np.zeros(n, dtype=np.int32), np.zeros(n)
        se, sl = np.zeros(n, dtype=np.int32), np.zeros(n)
        nr, ns = C.c_int(), C.c_int()
        st = lib().orc_query_trace(self.h, C.byref(prefs), seq.encode() if isinstance(seq, str) else seq,
                                   re, rs, C.byref(nr), se, sl, C.byref(ns))
        return st, list(zip(re[:nr.value], rs[:nr.value])), list(zip(se[:ns.value], sl[:ns.value]))

    def optimize_location(self, seq, loc, pend0, dist0, tol, prefs=None):
        prefs = prefs or make_prefs()
        out = np.zeros(3)
        st = lib().orc_optimize_location(self.h, C.byref(prefs), seq.encode() if isinstance(seq, str) else seq,
                                         loc, pend0, dist0, tol, out)
        return st, out

    def loglike_derivs(self, seq, loc, pend, dist):
        out = np.zeros(6)
        st = lib().orc_loglike_derivs(self.h, seq.encode() if isinstance(seq, str) else seq, loc, pend, dist, out)
        return st, out

    def __del__(self):
        if getattr(self, "h", None):
            lib().orc_ref_free(self.h)
            self.h = None


# Character -> likelihood vector tables (pplacer_src/nuc_models.ml:24-45,
# pplacer_src/prot_models.ml:5-43).
NUC_CODES = "ACGTRYMKSWHBVDN-?X"
NUC_BITS = [1, 2, 4, 8, 5, 10, 3, 12, 6, 9, 11, 14, 7, 13, 15, 15, 15, 15]
PROT_CODES = "ARNDCQEGHILKMFPSTWYV"


def lv_of_char(c, K):
    if K == 4:
        b = NUC_BITS[NUC_CODES.index(c)]
        return np.array([(b >> k) & 1 for k in range(4)], dtype=np.float64)
    v = np.zeros(K)
    if c in "-?X":
        v[:] = 1
    elif c == "B":
        v[PROT_CODES.index("D")] = v[PROT_CODES.index("N")] = 1
    elif c == "J":
        v[PROT_CODES.index("I")] = v[PROT_CODES.index("L")] = 1
    elif c == "Z":
        v[PROT_CODES.index("E")] = v[PROT_CODES.index("Q")] = 1
    else:
        v[PROT_CODES.index(c)] = 1
    return v


def emper_freq(seqs, K):
    """Alignment.emper_freq (common_src/alignment.ml:186-215): sum of the
    l1-normalised LVs of every non '-'/'?' character, l1-normalised."""
    total = np.zeros(K)
    cache = {}
    for s in seqs:
        for c in s:
            if c in "-?":
                continue
            if c not in cache:
                v = lv_of_char(c, K)
                cache[c] = v / np.abs(v).sum()
            total += cache[c]
    return total / np.abs(total).sum()


def model_from_fixture(fx):
    """Model of a tests/golden/like_*.json fixture (gmix_model.ml:386-413)."""
    m = fx["model"]
    K = len(m["exch"])
    statd = emper_freq(fx["seqs"], K) if m["statd"] is None else np.array(m["statd"])
    rates = discrete_gamma(m["gamma_n_cats"], m["gamma_alpha"])
    return Model(np.array(m["exch"], dtype=np.float64), statd, rates)


def reference_from_fixture(fx, model=None):
    model = model or model_from_fixture(fx)
    return Reference(model, fx["parent"], fx["bl"], fx["leaf_row"], fx["seqs"])


def polish(ref, seq, loc, pend, dist, max_pend=2.0, iters=100):
    """FP64 projected Newton on (pendant, distal) from (pend, dist) to the
    stationary point of the likelihood at location loc (box [1e-8, max_pend]
    x [0, bl]); returns (logL, pend, dist).  Used by tests to measure how far
    the reference's alternating Brent stops from the optimum."""
    cut = float(ref.bl[loc])
    p, d = float(pend), min(max(float(dist), 0.0), cut)
    st, v = ref.loglike_derivs(seq, loc, p, d)
    for _ in range(iters):
        L, gp, gd, hpp, hdd, hpd = v
        fp = not ((p <= 1e-8 and gp <= 0) or (p >= max_pend and gp >= 0))
        fd = cut > 0 and not ((d <= 0 and gd <= 0) or (d >= cut and gd >= 0))
        if not fp and not fd:
            break
        sp = sd = 0.0
        det = hpp * hdd - hpd * hpd
        if fp and fd and hpp < 0 and hdd < 0 and det > 0:
            sp = -(hdd * gp - hpd * gd) / det
            sd = -(hpp * gd - hpd * gp) / det
        else:
            if fp:
                sp = -gp / hpp if hpp < 0 else np.sign(gp) * max(0.5 * p, 0.01)
            if fd:
                sd = -gd / hdd if hdd < 0 else np.sign(gd) * 0.25 * cut
        ok = False
        for _ls in range(60):
            np_, nd = min(max(p + sp, 1e-8), max_pend), min(max(d + sd, 0.0), cut)
            st, nv = ref.loglike_derivs(seq, loc, np_, nd)
            if nv[0] >= L - 1e-12 * abs(L):
                ok = True
                break
            sp *= 0.5
            sd *= 0.5
        if not ok:
            break
        step = max(abs(np_ - p), abs(nd - d))
        p, d, v = np_, nd, nv
        if step < 1e-10:
            break
    return v[0], p, d


def prior_means(parent, bl, prior, prior_lower=0.0):
    """Pendant prior mean per node (pplacer_run.ml:379-389): prior 0 (the
    default) the flat exponential with mean tree length / edge count,
    2 the informative exponential of core.ml:34-51 (average distance from the
    node to the leaves below it, plus its branch length and prior_lower);
    prior 1 (uniform) has no mean (None)."""
    n = len(parent)
    if prior == 1:
        return None
    if prior == 0:
        edges = [i for i in range(n) if parent[i] >= 0]
        return [sum(bl[i] for i in edges) / len(edges)] * n
    children = [[] for _ in range(n)]
    for i, p in enumerate(parent):
        if p >= 0:
            children[p].append(i)

    def dists(i):  # leaf distances below node i, measured from node i
        if not children[i]:
            return [0.0]
        out = []
        for c in children[i]:
            out += [x + bl[c] for x in dists(c)]
        return out
    return [float(np.mean(dists(i))) + bl[i] + prior_lower for i in range(n)]


def marginal_like(ref, seq, loc, pend, dist, prior, mu=None, max_pend=2.0, rel=1e-9):
    """Three_tax.calc_marg_prob (three_tax.ml:169-215) in FP64:
    base + log((1/cut) int_0^cut int_0^U exp(L(p, d) - base) prior(p) dp dd),
    base = L at (pend, dist), the location's optimum; U = where
    L(., dist) + log prior has dropped 10 below its value at the optimum
    (find_upper_limit, three_tax.ml:124-159), found here by bisection to
    1e-10 where the reference runs 10 Brent iterations to 0.02 (the integral
    beyond either point is below e^-10 of the total); a zero-length edge
    integrates the pendant only, at the edge midpoint.  The integrals use
    adaptive Gauss-Kronrod quadrature (scipy.integrate.quad) to relative
    error `rel`, in place of GSL's QNG to pp_rel_err: both approximate the
    same integral."""
    import math
    from scipy import integrate
    cut = float(ref.bl[loc])

    def L(p, d):
        st, v = ref.loglike_derivs(seq, loc, max(p, 1e-12), min(max(d, 0.0), cut))
        return v[0]

    def lp(x):
        return 0.0 if prior == 1 else -math.log(mu) - x / mu
    base = L(pend, dist)
    target = base + lp(pend) - 10.0
    lo, hi, step = pend, pend, max(1e-4, 0.01 * pend)
    while True:
        q = min(hi + step, max_pend)
        if q <= hi:
            break
        if not (L(q, dist) + lp(q) > target):
            lo, hi = hi, q
            while hi - lo > 1e-10:
                m = 0.5 * (lo + hi)
                if L(m, dist) + lp(m) > target:
                    lo = m
                else:
                    hi = m
            break
        hi = q
        step *= 2
    U = hi

    def inner(d):
        pts = [pend] if 0 < pend < U else None
        v, _ = integrate.quad(lambda p: math.exp(L(p, d) - base + lp(p)), 0.0, U, epsabs=0.0, epsrel=rel,
                              points=pts, limit=400)
        return v
    if cut <= 1e-10:
        I = inner(0.5 * cut)
    else:
        pts = [dist] if 0 < dist < cut else None
        v, _ = integrate.quad(inner, 0.0, cut, epsabs=0.0, epsrel=rel, points=pts, limit=400)
        I = v / cut
    return base + math.log(I)


def refine_categories(exch, statd, rates, parent, bl, leaf_row, leaf_seqs):
    """Gcat_model.refine (gcat_model.ml:387-419): for every category c, the
    per-site tree log likelihood with every site in c, scored
    ll + 2 log(rate_c) - 3 rate_c; each site takes the first category with
    the highest score.  Returns (categories, scores [n_cat][S])."""
    S = len(leaf_seqs[0])
    scores = []
    for c, r in enumerate(rates):
        ref = Reference(Model(exch, statd, rates, np.full(S, c, dtype=np.int32)), parent, bl, leaf_row, leaf_seqs)
        scores.append(ref.root_site_loglike() + 2.0 * np.log(r) - 3.0 * r)
    scores = np.array(scores)
    best = np.full(S, -np.inf)
    cats = np.full(S, -1, dtype=np.int32)
    for c in range(len(rates)):
        up = scores[c] > best
        best[up] = scores[c][up]
        cats[up] = c
    return cats, scores
