"""Parity of whole placement records against the FP64 oracle.

A placement record (core.ml:336-377, placement.ml:168-175) is, per query, up
to keep_at_most placements (edge_num, likelihood, like_weight_ratio,
distal_length, pendant_length).  `compare` checks all of it:

  * best edge identical for >= 99.9% of non-tied queries (tie: the
    FP64-polished optima of the two best edges within 1e-6 relative), and
    the best logL within 1e-6 relative of the oracle's;
  * the kept edge set: an edge kept by one side only must sit at a keep
    boundary -- its polished optimum within `delta_keep` logL units of the
    other side's weakest kept placement (keep_at_most) or of the keep_factor
    threshold.  The two sides rank stage-2 results found by different
    optimisers (Newton at the optimum, the reference's Brent within its 0.01
    tolerance), so near-equal candidates can fall either side of a boundary;
  * branch lengths of every placement kept by both: the GPU's (pendant,
    distal) against the FP64-polished optimum of that edge
    (oracle.polish).  The allowed distance is 1e-4 plus what the GPU's own
    FP64 logL gap to the optimum permits on the quadratic model there
    (sqrt(2 gap / |h|) along a curved coordinate, gap / |g| against a
    bound); the gap itself must stay within `gap_tol` (the refinement's
    stop tolerance, 1e-5 relative for the Brent replica's alternating
    search);
  * like_weight_ratio of every placement kept by both, when the kept sets
    agree: against the oracle's and against the softmax of the polished
    optima, `lwr_tol` absolute.

The measured worst cases are returned so tests can report them.
"""
import math

LOGL_RTOL = 1e-6


def _allowed(gap, g, h):
    """Branch-length distance from the optimum that a logL gap permits."""
    lim = math.inf
    if h < 0:
        lim = math.sqrt(2.0 * gap / -h)
    if abs(g) > 1e-9:
        lim = min(lim, gap / abs(g) + 1e-12)
    return 1e-4 + lim


def compare(O, oref, seqs, res_gpu, res_orc, keep_at_most=7, keep_factor=0.01, delta_keep=0.25,
            gap_tol=1e-6, lwr_tol=1e-4, min_logl_frac=1.0, check_records=True):
    st = dict(queries=0, non_tied=0, mismatch=0, better=0, logl_ok=0, same_set=0, boundary_swaps=0,
              records=0, bl_within_1e4=0, max_dpend=0.0, max_ddist=0.0, max_gap_rel=0.0, max_lwr_vs_oracle=0.0,
              max_lwr_vs_optimum=0.0)
    bad = []
    log_kf = math.log(keep_factor)
    cache = {}

    def star(q, e, pend, dist):
        key = (q, e)
        if key not in cache:
            L, p, d = O.polish(oref, seqs[q], e, pend, dist)
            _, v = oref.loglike_derivs(seqs[q], e, p, d)
            cache[key] = (L, p, d, v)
        return cache[key]

    for q, (g, o) in enumerate(zip(res_gpu, res_orc)):
        if not o:
            if g:
                bad.append("q%d: GPU placed a query the oracle did not" % q)
            continue
        if not g:
            bad.append("q%d: GPU has no placement" % q)
            continue
        st["queries"] += 1
        ge, gl, _, gd, gp = g[0]
        oe, ol, _, od, op = o[0]
        o_star = star(q, oe, op, od)[0]
        tol = LOGL_RTOL * abs(ol)
        if ge != oe:
            g_star = star(q, ge, gp, gd)[0]
            if abs(g_star - o_star) <= tol:
                st["logl_ok"] += abs(gl - g_star) <= tol
                continue
            st["non_tied"] += 1
            if g_star > o_star + tol and abs(gl - g_star) <= tol:
                st["better"] += 1
                st["logl_ok"] += 1
            else:
                st["mismatch"] += 1
            continue
        st["non_tied"] += 1
        if gl > o_star + tol:
            bad.append("q%d: GPU logL %.9g above the polished optimum %.9g" % (q, gl, o_star))
        st["logl_ok"] += abs(gl - ol) <= tol + max(0.0, o_star - ol)
        if not check_records:
            continue
        # ---- kept set ----
        gset = {p[0]: p for p in g}
        oset = {p[0]: p for p in o}
        for e, p in list(gset.items()) + list(oset.items()):
            star(q, e, p[4], p[3])
        best_star = max(cache[(q, e)][0] for e in set(gset) | set(oset))
        if set(gset) == set(oset):
            st["same_set"] += 1
        else:
            for e in set(gset) ^ set(oset):
                other = oset if e in gset else gset
                bounds = [best_star + log_kf]
                if len(other) >= keep_at_most:
                    bounds.append(min(cache[(q, x)][0] for x in other))
                le = cache[(q, e)][0]
                if min(abs(le - b) for b in bounds) <= delta_keep:
                    st["boundary_swaps"] += 1
                else:
                    bad.append("q%d: edge %d kept by %s only, polished logL %.6g, boundaries %s" %
                               (q, e, "GPU" if e in gset else "oracle", le, ["%.6g" % b for b in bounds]))
        # ---- branch lengths of the placements both keep ----
        for e in set(gset) & set(oset):
            L, ps, ds, v = cache[(q, e)]
            _, gpd, gdd = gset[e][1], gset[e][4], gset[e][3]
            st_, vg = oref.loglike_derivs(seqs[q], e, gpd, gdd)
            gap = max(L - vg[0], 0.0)
            st["records"] += 1
            st["max_gap_rel"] = max(st["max_gap_rel"], gap / abs(L))
            if gap > gap_tol * abs(L):
                bad.append("q%d e%d: FP64 logL at the GPU's lengths %.9g is %.3g below the optimum" % (q, e, vg[0], gap))
            dp, dd = abs(gpd - ps), abs(gdd - ds)
            st["max_dpend"] = max(st["max_dpend"], dp)
            st["max_ddist"] = max(st["max_ddist"], dd)
            st["bl_within_1e4"] += dp <= 1e-4 and dd <= 1e-4
            ap = _allowed(gap, v[1], v[3])
            ad = _allowed(gap, v[2], v[4]) if oref.bl[e] > 0 else 1e-12
            if dp > ap or dd > ad:
                bad.append("q%d e%d: GPU (pend %.6g, dist %.6g) vs optimum (%.6g, %.6g), allowed (%.3g, %.3g)" %
                           (q, e, gpd, gdd, ps, ds, ap, ad))
        # ---- like_weight_ratios ----
        if set(gset) == set(oset):
            mx = max(cache[(q, e)][0] for e in gset)
            tot = sum(math.exp(cache[(q, e)][0] - mx) for e in gset)
            for e in gset:
                d1 = abs(gset[e][2] - oset[e][2])
                d2 = abs(gset[e][2] - math.exp(cache[(q, e)][0] - mx) / tot)
                st["max_lwr_vs_oracle"] = max(st["max_lwr_vs_oracle"], d1)
                st["max_lwr_vs_optimum"] = max(st["max_lwr_vs_optimum"], d2)
                if d1 > lwr_tol or d2 > lwr_tol:
                    bad.append("q%d e%d: like_weight_ratio %.8f vs oracle %.8f, vs optimum %.8f" %
                               (q, e, gset[e][2], oset[e][2], math.exp(cache[(q, e)][0] - mx) / tot))
    if st["mismatch"] > 0.001 * max(st["non_tied"], 1):
        bad.append("best edge differs for %d of %d non-tied queries" % (st["mismatch"], st["non_tied"]))
    if st["logl_ok"] < min_logl_frac * st["queries"]:
        bad.append("best logL within tolerance for %d of %d queries" % (st["logl_ok"], st["queries"]))
    return st, bad
