"""Parity of whole placement records against the FP64 oracle.

A placement record (core.ml:336-377, placement.ml:168-175) is, per query, up
to keep_at_most placements (edge_num, likelihood, like_weight_ratio,
distal_length, pendant_length).  `compare` checks all of it:

  * best edge identical for >= 99.9% of non-tied queries (tie: the
    FP64-polished optima of the two best edges within 1e-6 relative), and
    the best logL within 1e-6 relative of the oracle's;
  * the kept edge set, judged on the polished optima of the edges either
    side keeps: every GPU-kept edge clears the keep_factor threshold, and an
    edge only the oracle keeps lies below that threshold or below the GPU's
    weakest kept edge when the GPU's list is full (keep_at_most), each within
    `delta_keep` logL units.  An edge only the GPU keeps is classified: a
    near-tie at the oracle's own keep boundary, the oracle's stage-2 Brent
    (tolerance 0.01) stopping more than `delta_keep` below that edge's
    optimum -- it then ranks the edge too low to keep -- or the oracle's
    baseball ending before the edge (`oracle_stage2(q)` gives the oracle's
    stage-2 results); anything else fails;
  * branch lengths of every placement kept by both: the GPU's (pendant,
    distal) against the FP64-polished optimum of that edge
    (oracle.polish).  The allowed distance is 1e-4 plus what the GPU's own
    FP64 logL gap to the optimum permits on the quadratic model there; the
    gap itself must stay within `gap_tol` relative (1e-6, the logL target,
    for Newton; the Brent replica compares FP32 likelihoods whose rounding
    exceeds the differences its 1e-5 length tolerance resolves, and is held
    to 1e-4);
  * the GPU's reported logL of every placement kept by both against the
    FP64 logL at its own lengths: within 1e-6 relative (the evaluation's
    FP32 arithmetic);
  * like_weight_ratio of every placement kept by both, when the kept sets
    agree: against the softmax of the polished optima, `lwr_tol` absolute
    plus twice the largest distance of the query's reported GPU logLs from
    those optima (the FP64 gap plus the evaluation error; a ratio moves by
    at most about that much), and against the oracle's, that plus the
    oracle's own distance from the softmax.

The measured worst cases are returned so tests can report them.
"""
import math

LOGL_RTOL = 1e-6


def _allowed(gap, v, distal_free=True):
    """Distances from the optimum, in pendant and distal length, that a logL
    gap permits on the quadratic model there: sqrt(2 gap [(-H)^-1]_ii) along
    curved coordinates (the inverse Hessian's diagonal allows for the two
    lengths' correlation), gap / |g_i| against a bound; plus 1e-4."""
    _, gp, gd, hpp, hdd, hpd = v
    a, b, c = -hpp, -hdd, -hpd
    lim = [math.inf, math.inf]
    det = a * b - c * c
    if distal_free and a > 0 and b > 0 and det > 0:
        lim = [math.sqrt(2.0 * gap * b / det), math.sqrt(2.0 * gap * a / det)]
    else:
        if a > 0:
            lim[0] = math.sqrt(2.0 * gap / a)
        if distal_free and b > 0:
            lim[1] = math.sqrt(2.0 * gap / b)
    for i, g in enumerate((gp, gd)):
        if abs(g) > 1e-9:
            lim[i] = min(lim[i], gap / abs(g) + 1e-12)
    if not distal_free:
        lim[1] = 0.0
    return 1e-4 + lim[0], 1e-4 + lim[1]


def compare(O, oref, seqs, res_gpu, res_orc, keep_at_most=7, keep_factor=0.01, delta_keep=0.1,
            gap_tol=1e-6, lwr_tol=1e-4, min_logl_frac=1.0, check_records=True, oracle_stage2=None, newton=True,
            max_mismatch_frac=0.001):
    st = dict(queries=0, non_tied=0, mismatch=0, better=0, logl_ok=0, same_set=0, boundary_swaps=0,
              records=0, bl_within_1e4=0, max_dpend=0.0, max_ddist=0.0, max_gap_rel=0.0, max_gap=0.0,
              max_lwr_vs_oracle=0.0, max_lwr_vs_optimum=0.0, max_oracle_lwr_vs_optimum=0.0, max_eval_err_rel=0.0,
              oracle_only=0, gpu_only=0, gpu_only_boundary=0,
              gpu_only_oracle_brent_short=0, gpu_only_oracle_not_evaluated=0, gpu_only_unclassified=0,
              max_oracle_stage2_shortfall=0.0)
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
                st["logl_ok"] += int(abs(gl - g_star) <= tol)
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
        st["logl_ok"] += int(abs(gl - ol) <= tol + max(0.0, o_star - ol))
        if not check_records:
            continue
        # ---- kept set ----
        gset = {p[0]: p for p in g}
        oset = {p[0]: p for p in o}
        for e, p in list(gset.items()) + list(oset.items()):
            star(q, e, p[4], p[3])
        Ls = {e: cache[(q, e)][0] for e in set(gset) | set(oset)}
        best_star = max(Ls.values())
        thr = best_star + log_kf
        g_min = min(Ls[e] for e in gset)
        if set(gset) == set(oset):
            st["same_set"] += 1
        if not newton:
            # the Brent replica ranks stage-2 results of the reference's own
            # search: its kept set is the oracle's, up to near-ties at a
            # keep boundary, and up to the oracle's stage-2 Brent stopping
            # short of an edge the GPU keeps (the same search on FP32
            # likelihoods can stop elsewhere on a long query)
            o_min = min(Ls[e] for e in oset)
            for e in set(gset) ^ set(oset):
                other_min = o_min if e in gset else g_min
                other_n = len(oset) if e in gset else len(gset)
                bounds = [thr] + ([other_min] if other_n >= keep_at_most else [])
                st["gpu_only" if e in gset else "oracle_only"] += 1
                if min(abs(Ls[e] - b) for b in bounds) <= delta_keep:
                    continue
                s2 = oracle_stage2(q) if (oracle_stage2 and e in gset) else None
                if s2 is not None and e in s2 and s2[e] < Ls[e] - delta_keep:
                    st["gpu_only_oracle_brent_short"] += 1
                    st["max_oracle_stage2_shortfall"] = max(st["max_oracle_stage2_shortfall"], Ls[e] - s2[e])
                    continue
                bad.append("q%d: edge %d (polished %.4f) kept by one side only" % (q, e, Ls[e]))
        # the GPU's keep decisions, judged on the polished optima: every kept
        # edge clears the keep_factor threshold, and an edge only the oracle
        # keeps lies below that threshold or below the GPU's weakest kept
        # edge when the GPU's list is full
        for e in gset if newton else ():
            if Ls[e] < thr - delta_keep:
                bad.append("q%d: GPU keeps edge %d at %.4f below the keep threshold %.4f" % (q, e, Ls[e], thr))
        for e in set(oset) - set(gset) if newton else ():
            st["oracle_only"] += 1
            ok = Ls[e] < thr + delta_keep or (len(gset) >= keep_at_most and Ls[e] <= g_min + delta_keep)
            if not ok:
                bad.append("q%d: edge %d (polished %.4f) kept by the oracle only; GPU weakest %.4f of %d, threshold %.4f"
                           % (q, e, Ls[e], g_min, len(gset), thr))
        # why the oracle lacks an edge the GPU keeps: a near-tie at its own
        # keep boundary, its stage-2 Brent stopping short of that edge's
        # optimum, or its baseball ending before it
        o_min = min(Ls[e] for e in oset)
        for e in set(gset) - set(oset) if newton else ():
            st["gpu_only"] += 1
            bounds = [thr] + ([o_min] if len(oset) >= keep_at_most else [])
            if min(abs(Ls[e] - b) for b in bounds) <= delta_keep:
                st["gpu_only_boundary"] += 1
                continue
            s2 = oracle_stage2(q) if oracle_stage2 else None
            if s2 is not None and e in s2 and s2[e] < Ls[e] - delta_keep:
                st["gpu_only_oracle_brent_short"] += 1
                st["max_oracle_stage2_shortfall"] = max(st["max_oracle_stage2_shortfall"], Ls[e] - s2[e])
            elif s2 is not None and e not in s2:
                st["gpu_only_oracle_not_evaluated"] += 1
            elif s2 is None:
                st["gpu_only_unclassified"] += 1
            else:
                bad.append("q%d: edge %d (polished %.4f, oracle stage 2 %.4f) kept by the GPU only" % (q, e, Ls[e], s2[e]))
        # ---- branch lengths of the placements both keep ----
        q_dev = 0.0
        for e in set(gset) & set(oset):
            L, ps, ds, v = cache[(q, e)]
            gll, gpd, gdd = gset[e][1], gset[e][4], gset[e][3]
            st_, vg = oref.loglike_derivs(seqs[q], e, gpd, gdd)
            gap = max(L - vg[0], 0.0)
            q_dev = max(q_dev, abs(gll - L))
            err = abs(gll - vg[0])
            st["max_eval_err_rel"] = max(st["max_eval_err_rel"], err / abs(L))
            if err > LOGL_RTOL * abs(L):
                bad.append("q%d e%d: GPU logL %.9g vs FP64 %.9g at its lengths" % (q, e, gll, vg[0]))
            st["records"] += 1
            st["max_gap_rel"] = max(st["max_gap_rel"], gap / abs(L))
            st["max_gap"] = max(st["max_gap"], gap)
            if gap > gap_tol * abs(L):
                bad.append("q%d e%d: FP64 logL at the GPU's lengths %.9g is %.3g below the optimum" % (q, e, vg[0], gap))
            dp, dd = abs(gpd - ps), abs(gdd - ds)
            st["max_dpend"] = max(st["max_dpend"], dp)
            st["max_ddist"] = max(st["max_ddist"], dd)
            st["bl_within_1e4"] += int(dp <= 1e-4 and dd <= 1e-4)
            ap, ad = _allowed(gap, v, oref.bl[e] > 0)
            if dp > ap or dd > ad:
                bad.append("q%d e%d: GPU (pend %.6g, dist %.6g) vs optimum (%.6g, %.6g), allowed (%.3g, %.3g)" %
                           (q, e, gpd, gdd, ps, ds, ap, ad))
        # ---- like_weight_ratios ----
        # The oracle's own ratios sit off the optimum's by what its Brent
        # leaves in logL (absolute: ~1e-3 at a node, where the optimum lies on
        # an edge's end), so the GPU is held to lwr_tol against the optimum
        # and to lwr_tol plus the oracle's own deviation against the oracle.
        if set(gset) == set(oset):
            mx = max(cache[(q, e)][0] for e in gset)
            tot = sum(math.exp(cache[(q, e)][0] - mx) for e in gset)
            for e in gset:
                ideal = math.exp(cache[(q, e)][0] - mx) / tot
                d_or = abs(oset[e][2] - ideal)
                d1 = abs(gset[e][2] - oset[e][2])
                d2 = abs(gset[e][2] - ideal)
                st["max_lwr_vs_oracle"] = max(st["max_lwr_vs_oracle"], d1)
                st["max_lwr_vs_optimum"] = max(st["max_lwr_vs_optimum"], d2)
                st["max_oracle_lwr_vs_optimum"] = max(st["max_oracle_lwr_vs_optimum"], d_or)
                # a ratio moves by at most ~2x the largest logL error among
                # the query's placements: the GPU's reported logLs against
                # the polished optima
                tol = lwr_tol + 2.0 * q_dev
                if d2 > tol or d1 > tol + d_or:
                    bad.append("q%d e%d: like_weight_ratio %.8f vs oracle %.8f, vs optimum %.8f" %
                               (q, e, gset[e][2], oset[e][2], ideal))
    if st["mismatch"] > max_mismatch_frac * max(st["non_tied"], 1):
        bad.append("best edge differs for %d of %d non-tied queries" % (st["mismatch"], st["non_tied"]))
    if st["logl_ok"] < min_logl_frac * st["queries"]:
        bad.append("best logL within tolerance for %d of %d queries" % (st["logl_ok"], st["queries"]))
    return st, bad


def oracle_stage2(O, oref, seqs, prefs):
    """q -> {edge: the oracle's stage-2 logL} (its baseball trace), cached."""
    memo = {}

    def f(q):
        if q not in memo:
            _, _, s2 = oref.trace(seqs[q], prefs)
            memo[q] = {int(e): float(v) for e, v in s2}
        return memo[q]
    return f
