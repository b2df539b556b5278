"""Python host mirror of the batched placement engine of include/pplacer_gb300.h.

Mirrors the reference's per-run flow (pplacer_src/pplacer_run.ml:167-783):
build the model, precompute darr / parr / snodes on the reference tree, then
place queries with ``Core.pplacer_core`` semantics (pplacer_src/core.ml:113-409).
All computation happens in the CUDA library; this module only marshals
arguments and results.
"""
import ctypes as C

import numpy as np

from . import lib as _L
from .model import Model

BRENT, NEWTON = 0, 1


def default_prefs(**kw):
    p = _L.Prefs()
    _L.load().pgb_prefs_default(C.byref(p))
    for k, v in kw.items():
        if not hasattr(p, k):
            raise KeyError(k)
        setattr(p, k, v)
    return p


class Engine:
    """Device-resident reference tree and placement."""

    def __init__(self, model: Model, parent, bl):
        L = _L.load()
        self.model = model
        self.K = model.K
        self.parent = np.ascontiguousarray(parent, dtype=np.int32)
        self.bl = np.ascontiguousarray(bl, dtype=np.float64)
        self.n_nodes = len(self.parent)
        self.S = None
        self.RP = 1 if model.gcat else len(model.rates)
        self._keep = {}  # arrays that must outlive the create call
        self._pp = False
        self.h = None

    def _create(self, n_sites):
        L = _L.load()
        m = self.model
        arrs = dict(statd=np.ascontiguousarray(m.statd, np.float64), x=np.ascontiguousarray(m.x, np.float64),
                    lam=np.ascontiguousarray(m.lam, np.float64), xit=np.ascontiguousarray(m.xit, np.float64),
                    rates=np.ascontiguousarray(m.rates, np.float64))
        sc = None if m.site_cats is None else np.ascontiguousarray(m.site_cats, np.int32)
        md = _L.ModelDesc(self.K, len(m.rates), 1 if m.gcat else 0, n_sites, arrs["statd"].ctypes.data,
                          arrs["x"].ctypes.data, arrs["lam"].ctypes.data, arrs["xit"].ctypes.data,
                          arrs["rates"].ctypes.data, None if sc is None else sc.ctypes.data)
        td = _L.TreeDesc(self.n_nodes, self.parent.ctypes.data, self.bl.ctypes.data)
        h = C.c_void_p()
        _L.check(L.pgb_engine_create(C.byref(md), C.byref(td), C.byref(h)), "pgb_engine_create")
        self.h = h
        self.S = n_sites

    def precompute(self, leaf_row, ref_seqs):
        """darr / parr / snodes on the GPU from the reference alignment rows."""
        S = len(ref_seqs[0])
        if self.h is None:
            self._create(S)
        lr = np.ascontiguousarray(leaf_row, dtype=np.int32)
        buf = "".join(ref_seqs).encode()
        _L.check(_L.load().pgb_engine_precompute(self.h, lr.ctypes.data, buf, len(ref_seqs)), "pgb_engine_precompute")

    def refine_categories(self, leaf_row, ref_seqs):
        """Gcat site-category refinement on the GPU (gcat_model.ml:387-419); returns the
        new categories.  Run precompute again before placing."""
        S = len(ref_seqs[0])
        if self.h is None:
            self._create(S)
        lr = np.ascontiguousarray(leaf_row, dtype=np.int32)
        cats = np.zeros(S, dtype=np.int32)
        buf = "".join(ref_seqs).encode()
        _L.check(_L.load().pgb_engine_refine_categories(self.h, lr.ctypes.data, buf, len(ref_seqs), cats.ctypes.data),
                 "pgb_engine_refine_categories")
        return cats

    def set_glvs(self, darr, darr_e, parr, parr_e, snodes=None, snodes_e=None):
        """Upload caller-computed FP64 GLVs ([n_nodes][R][S][K], exponents [n_nodes][S])."""
        S = darr.shape[2]
        if self.h is None:
            self._create(S)
        c = lambda a, t: np.ascontiguousarray(a, dtype=t)
        d, de, p, pe = c(darr, np.float64), c(darr_e, np.int32), c(parr, np.float64), c(parr_e, np.int32)
        sn = None if snodes is None else c(snodes, np.float64)
        se = None if snodes_e is None else c(snodes_e, np.int32)
        _L.check(_L.load().pgb_engine_set_glvs(self.h, d.ctypes.data, de.ctypes.data, p.ctypes.data, pe.ctypes.data,
                                               _L.ptr(sn), _L.ptr(se)), "pgb_engine_set_glvs")

    def get_glv(self, which, node):
        a = np.zeros((self.RP, self.S, self.K))
        e = np.zeros(self.S, dtype=np.int32)
        _L.check(_L.load().pgb_engine_get_glv(self.h, which, node, a.ctypes.data, e.ctypes.data), "pgb_engine_get_glv")
        return a, e

    # ---- queries ----
    def load_queries(self, seqs):
        self.Q = len(seqs)
        buf = "".join(seqs).encode() if self.Q else b""
        _L.check(_L.load().pgb_queries_load(self.h, self.Q, buf), "pgb_queries_load")

    def run(self, prefs):
        self._kam = prefs.keep_at_most
        self._pp = bool(prefs.calc_pp)
        _L.check(_L.load().pgb_queries_run(self.h, C.byref(prefs)), "pgb_queries_run")

    def fetch(self):
        Q, kam = self.Q, self._kam
        out = (_L.Placement * max(1, Q * kam))()
        n_out = np.zeros(max(Q, 1), dtype=np.int32)
        status = np.zeros(max(Q, 1), dtype=np.int32)
        _L.check(_L.load().pgb_queries_fetch(self.h, C.addressof(out), n_out.ctypes.data, status.ctypes.data),
                 "pgb_queries_fetch")
        def row(o):
            t = (o.edge, o.like, o.lwr, o.dist, o.pend)
            return t + (o.post_prob, o.marginal_like) if self._pp else t
        res = [[row(out[q * kam + i]) for i in range(n_out[q])] for q in range(Q)]
        return res, status[:Q]

    def place(self, seqs, prefs=None):
        """Place query rows; returns ([(edge, like, lwr, dist, pend), ...] per query, status per query);
        with prefs.calc_pp each tuple adds (post_prob, marginal_like)."""
        prefs = prefs or default_prefs()
        self.load_queries(seqs)
        self.run(prefs)
        return self.fetch()

    def place_host(self, seqs, prefs=None, batch=0):
        """Place through the single C-ABI call pgb_place_batch (host buffers in
        and out, device batches of `batch` queries; 0: automatic)."""
        prefs = prefs or default_prefs()
        Q, kam = len(seqs), prefs.keep_at_most
        out = (_L.Placement * max(1, Q * kam))()
        n_out = np.zeros(max(Q, 1), dtype=np.int32)
        status = np.zeros(max(Q, 1), dtype=np.int32)
        buf = "".join(seqs).encode() if Q else b""
        _L.check(_L.load().pgb_place_batch(self.h, C.byref(prefs), Q, buf, int(batch), C.addressof(out),
                                           n_out.ctypes.data, status.ctypes.data), "pgb_place_batch")
        res = [[(out[q * kam + i].edge, out[q * kam + i].like, out[q * kam + i].lwr, out[q * kam + i].dist,
                 out[q * kam + i].pend) for i in range(n_out[q])] for q in range(Q)]
        return res, status[:Q]

    def stage1(self, prefs=None):
        prefs = prefs or default_prefs()
        n_edges = self.n_nodes - 1
        sc = np.zeros((self.Q, n_edges))
        _L.check(_L.load().pgb_queries_stage1(self.h, C.byref(prefs), sc.ctypes.data), "pgb_queries_stage1")
        return sc

    def rank(self, rk, prefs=None):
        """Stage-1 ranking: the rk best edge columns per query (-1 for a query without placement)."""
        prefs = prefs or default_prefs()
        out = np.zeros((self.Q, rk), dtype=np.int32)
        _L.check(_L.load().pgb_queries_rank(self.h, C.byref(prefs), rk, out.ctypes.data), "pgb_queries_rank")
        return out

    def trials(self, trials, optimizer=NEWTON, mode=0, prefs=None):
        """trials: list of (query, edge_node, pend0, dist0, tol)."""
        prefs = prefs or default_prefs()
        n = len(trials)
        tin = (_L.Trial * max(1, n))(*[_L.Trial(*t) for t in trials])
        tout = (_L.TrialOut * max(1, n))()
        _L.check(_L.load().pgb_queries_trials(self.h, C.byref(prefs), optimizer, mode, n, C.addressof(tin),
                                              C.addressof(tout)), "pgb_queries_trials")
        return [dict(like=t.like, pend=t.pend, dist=t.dist, derivs=list(t.derivs), status=t.status,
                     n_evals=t.n_evals) for t in tout[:n]]

    def autotune(self, prefs=None):
        """Pick the trial-kernel shape per query-length bin on the loaded queries."""
        prefs = prefs or default_prefs()
        _L.check(_L.load().pgb_engine_autotune(self.h, C.byref(prefs)), "pgb_engine_autotune")
        return self.get_tuning()

    def get_tuning(self):
        th = np.zeros(6, dtype=np.int32)
        wi = np.zeros(6, dtype=np.int32)
        _L.check(_L.load().pgb_engine_get_tuning(self.h, th.ctypes.data, wi.ctypes.data), "pgb_engine_get_tuning")
        return list(th), list(wi)

    def set_tuning(self, threads, smem_windows):
        """Impose the trial-kernel shape per query-length bin (threads 32 = one
        warp per trial, 1 = the tensor-core CTA of 20-state models)."""
        th = np.ascontiguousarray(np.broadcast_to(threads, 6), dtype=np.int32)
        wi = np.ascontiguousarray(np.broadcast_to(smem_windows, 6), dtype=np.int32)
        _L.check(_L.load().pgb_engine_set_tuning(self.h, th.ctypes.data, wi.ctypes.data), "pgb_engine_set_tuning")

    def timings(self):
        ms = np.zeros(6)
        cnt = np.zeros(8)
        _L.check(_L.load().pgb_engine_timings(self.h, ms.ctypes.data, cnt.ctypes.data), "pgb_engine_timings")
        return ms, cnt

    def close(self):
        if self.h is not None:
            _L.load().pgb_engine_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def engine_for_workload(w):
    """Engine with precomputed GLVs for a synthetic workload (pplacer_gb300.synth)."""
    m = Model.from_exchangeabilities(w.exch, w.statd, w.rates, w.site_cats)
    e = Engine(m, w.parent, w.bl)
    e.precompute(w.leaf_row, w.ref_seqs)
    return e
