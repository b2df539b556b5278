"""CPU oracle (test infrastructure only): pplacer's posterior-probability
integral as the reference computes it -- GSL's non-adaptive QNG integrator
and Three_tax.calc_marg_prob with its upper-limit search and ETOL retries.

QNG restates the published QUADPACK algorithm (Piessens, de Doncker-Kapenga,
Ueberhuber and Kahaner, 1983), as GSL 2.x's gsl_integration_qng implements
it and pplacer reaches it through Gsl.Integration.qng (gsl 1.25.0 OCaml
bindings, pplacer_src/integration.ml:27-31): the 21-point Kronrod rule with
its embedded 10-point Gauss rule, then Patterson's 43- and 87-point
extensions, each reusing the previous rules' function values; the error
estimate of each stage is |I_n - I_prev| rescaled by the integrand's
variation (rescale_error); the first stage whose estimate is below
max(epsabs, epsrel |I|) returns, and failing the 87-point stage is the
ETOL error ("failed to reach tolerance with highest-order rule").  The node
and weight tables are read from pplacer_gb300/csrc/qng_rules.h, which
make_qng_rules.py computes from the rules' definition (tests/test_qng.py
checks their exactness degrees).

calc_marg_prob follows pplacer_src/three_tax.ml:124-215 and
minimization.ml:24-41,83-101 (the bisection start finder and GSL Brent).
"""
import math
import os
import re

DBL_EPSILON = 2.220446049250313e-16
DBL_MIN = 2.2250738585072014e-308
GOLDEN = 0.3819660
SQRT_DBL_EPSILON = 1.4901161193847656e-08

_RULES = None


def rules():
    """The QNG tables: x1, w10, x2, w21a, w21b, x3, w43a, w43b, x4, w87a, w87b."""
    global _RULES
    if _RULES is None:
        path = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "pplacer_gb300", "csrc",
                            "qng_rules.h")
        text = open(path).read()
        _RULES = {m.group(1): [float(v) for v in m.group(3).replace("\n", " ").split(",") if v.strip()]
                  for m in re.finditer(r"const double (\w+)\[(\d+)\] = \{([^}]*)\};", text)}
    return _RULES


class QngError(Exception):
    """A GSL error of qng: code 'ETOL' (tolerance not reached) or 'EBADTOL'."""

    def __init__(self, code, result=None, abserr=None):
        super().__init__(code)
        self.code, self.result, self.abserr = code, result, abserr


def rescale_error(err, result_abs, result_asc):
    err = abs(err)
    if result_asc != 0.0 and err != 0.0:
        scale = (200.0 * err / result_asc) ** 1.5
        err = result_asc * scale if scale < 1.0 else result_asc
    if result_abs > DBL_MIN / (50.0 * DBL_EPSILON):
        min_err = 50.0 * DBL_EPSILON * result_abs
        if min_err > err:
            err = min_err
    return err


def qng(f, a, b, epsabs, epsrel):
    """(result, abserr, neval); raises QngError('ETOL') after the 87-point
    stage fails, QngError('EBADTOL') for an unattainable tolerance."""
    R = rules()
    x1, w10, x2, w21a, w21b = R["x1"], R["w10"], R["x2"], R["w21a"], R["w21b"]
    x3, w43a, w43b, x4, w87a, w87b = R["x3"], R["w43a"], R["w43b"], R["x4"], R["w87a"], R["w87b"]
    half = 0.5 * (b - a)
    abs_half = abs(half)
    center = 0.5 * (b + a)
    f_center = f(center)
    if epsabs <= 0 and (epsrel < 50 * DBL_EPSILON or epsrel < 0.5e-28):
        raise QngError("EBADTOL")
    res10 = 0.0
    res21 = w21b[5] * f_center
    resabs = w21b[5] * abs(f_center)
    savfun = [0.0] * 21
    fv1, fv2, fv3, fv4 = [0.0] * 5, [0.0] * 5, [0.0] * 5, [0.0] * 5
    for k in range(5):
        h = half * x1[k]
        a1, a2 = f(center + h), f(center - h)
        s = a1 + a2
        res10 += w10[k] * s
        res21 += w21a[k] * s
        resabs += w21a[k] * (abs(a1) + abs(a2))
        savfun[k] = s
        fv1[k], fv2[k] = a1, a2
    for k in range(5):
        h = half * x2[k]
        a1, a2 = f(center + h), f(center - h)
        s = a1 + a2
        res21 += w21b[k] * s
        resabs += w21b[k] * (abs(a1) + abs(a2))
        savfun[k + 5] = s
        fv3[k], fv4[k] = a1, a2
    resabs *= abs_half
    mean = 0.5 * res21
    resasc = w21b[5] * abs(f_center - mean)
    for k in range(5):
        resasc += w21a[k] * (abs(fv1[k] - mean) + abs(fv2[k] - mean)) + w21b[k] * (abs(fv3[k] - mean) +
                                                                                  abs(fv4[k] - mean))
    resasc *= abs_half
    result = res21 * half
    err = rescale_error((res21 - res10) * half, resabs, resasc)
    if err < epsabs or err < epsrel * abs(result):
        return result, err, 21
    res43 = w43b[11] * f_center
    for k in range(10):
        res43 += savfun[k] * w43a[k]
    for k in range(11):
        h = half * x3[k]
        s = f(center + h) + f(center - h)
        res43 += s * w43b[k]
        savfun[k + 10] = s
    result = res43 * half
    err = rescale_error((res43 - res21) * half, resabs, resasc)
    if err < epsabs or err < epsrel * abs(result):
        return result, err, 43
    res87 = w87b[22] * f_center
    for k in range(21):
        res87 += savfun[k] * w87a[k]
    for k in range(22):
        h = half * x4[k]
        res87 += w87b[k] * (f(center + h) + f(center - h))
    result = res87 * half
    err = rescale_error((res87 - res43) * half, resabs, resasc)
    if err < epsabs or err < epsrel * abs(result):
        return result, err, 87
    raise QngError("ETOL", result, err)


class BrentError(Exception):
    """GSL_EINVAL / GSL_EBADFUNC from the minimiser, or minimization.ml's
    FindStartFailure / ExceededMaxIter / InvalidStartValues."""

    def __init__(self, code):
        super().__init__(code)
        self.code = code


def brent(f, raw_start, left, right, tol, max_iters=100):
    """Minimization.brent with the bisection start finder
    (minimization.ml:11-41,83-101) on GSL's Brent minimiser."""
    if left >= raw_start or raw_start >= right:
        raise BrentError("InvalidStartValues")
    lefty, righty = f(left), f(right)
    smaller, miny = (left, lefty) if lefty < righty else (right, righty)
    start, it = raw_start, 1
    while True:
        prev = f(start)
        if prev < miny:
            break
        if abs(start - smaller) < tol:
            return start if prev < miny else smaller  # FoundMin
        if it > max_iters:
            raise BrentError("FindStartFailure")
        start, it = 0.5 * (start + smaller), it + 1
    # gsl_min_fminimizer_set: f at the three points (a non-finite value is
    # GSL_EBADFUNC), the bracketing check (GSL_EINVAL)
    lower, upper, z = left, right, start
    fz, fl, fu = f(z), f(lower), f(upper)
    if not (math.isfinite(fz) and math.isfinite(fl) and math.isfinite(fu)):
        raise BrentError("EBADFUNC")
    if not (fz < fl and fz < fu):
        raise BrentError("EINVAL")
    v = w = lower + GOLDEN * (upper - lower)
    fv = fw = f(v)
    if not math.isfinite(fv):
        raise BrentError("EBADFUNC")
    d = e = 0.0
    for _ in range(max_iters):
        dd, ee = e, d  # GSL's iteration takes d and e with their roles swapped
        wl, wu = z - lower, upper - z
        tolerance = SQRT_DBL_EPSILON * abs(z)
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
        fu_ = f(u)
        if not math.isfinite(fu_):
            raise BrentError("EBADFUNC")
        if fu_ <= fz:
            if u < z:
                upper = z
            else:
                lower = z
            v, fv, w, fw, z, fz = w, fw, z, fz, u, fu_
        else:
            if u < z:
                lower = u
            else:
                upper = u
            if fu_ <= fw or w == z:
                v, fv, w, fw = w, fw, u, fu_
            elif fu_ <= fv or v == z or v == w:
                v, fv = u, fu_
        if upper - lower < tol:
            return z
    raise BrentError("ExceededMaxIter")


def find_upper_limit(L, dist, pend0, base, prior, max_pend):
    """Three_tax.find_upper_limit (three_tax.ml:124-159).  Returns (upper,
    note): note is None, 'EINVAL' (integrate to max_pend, as the reference
    does) or the name of an exception the reference does not catch there
    (the reference's query would fail; max_pend is used)."""
    if prior(pend0) == 0.0:
        cur = pend0
        while True:
            nxt = cur / 2.0
            if prior(nxt) > math.exp(-10.0):
                return cur, None
            cur = nxt
    target = -10.0 + base + math.log(prior(pend0))

    def f(p):
        like = L(p, dist) + math.log(prior(p))
        x = abs(target - like)
        return 100000.0 if x == math.inf else x
    start = pend0 + (max_pend - pend0) / 2.0
    try:
        return brent(f, start, pend0, max_pend, 0.02, max_iters=10), None
    except BrentError as ex:
        return max_pend, ex.code


def calc_marg_prob(L, pend0, dist0, cut, prior, max_pend, rel_err):
    """Three_tax.calc_marg_prob (three_tax.ml:169-215): base_ll +
    log((1/cut) int_0^cut int_0^U exp(L(p, d) - base_ll) prior(p) dp dd)
    by nested QNG (relative error rel_err, no absolute error); on ETOL from
    either integral the upper limit U is halved and the whole integral
    retried, at most 10 times, after which base_ll is returned.  Returns
    (marginal, info) with info = dict(upper, exceptions, evals, note)."""
    n_evals = [0]

    def Lc(p, d):
        n_evals[0] += 1
        return L(p, d)
    base = Lc(pend0, dist0)
    U, note = find_upper_limit(Lc, dist0, pend0, base, prior, max_pend)
    info = dict(upper=U, exceptions=0, note=note)
    while True:
        if info["exceptions"] >= 10:
            info["evals"] = n_evals[0]
            return base, info

        def inner(d, U=U):
            return qng(lambda p: math.exp(Lc(p, d) - base) * prior(p), 0.0, U, 0.0, rel_err)[0]
        try:
            if abs(cut) < 1e-5:  # cut_bl =~ 0. (ppatteries.ml:96-97)
                I = inner(cut / 2.0)
            else:
                I = qng(inner, 0.0, cut, 0.0, rel_err)[0] / cut
            info["upper"], info["evals"] = U, n_evals[0]
            return base + math.log(I), info
        except QngError as ex:
            if ex.code != "ETOL":
                raise
            info["exceptions"] += 1
            U = U / 2.0
