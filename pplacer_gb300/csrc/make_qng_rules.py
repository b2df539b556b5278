"""Writes qng_rules.h: the nested 10/21/43/87-point Gauss-Kronrod-Patterson
rules of the non-adaptive QNG integrator (Piessens, de Doncker-Kapenga,
Ueberhuber and Kahaner, QUADPACK, 1983; GSL's gsl_integration_qng, which
pplacer's posterior probabilities call through Gsl.Integration.qng,
pplacer_src/integration.ml:27-31).

The rules are computed here from their definition, in 120-digit arithmetic:
  * G10: the roots of the Legendre polynomial P10;
  * K21: G10 plus the 11 roots of the monic polynomial of degree 11
    orthogonal on [-1, 1] to every polynomial of lower degree with the weight
    P10 (Kronrod's extension);
  * P43, P87: each rule plus the roots of the monic polynomial of twice the
    previous extension's degree orthogonal to every lower-degree polynomial
    with the weight of the product of the rule's node polynomial (Patterson's
    extensions);
  * the weights of each rule: exact integration of the Legendre polynomials
    of degree below its node count.

Layout (the order the QNG algorithm consumes them; positive nodes, largest
first; "savfun" is the list of pair sums f(c + h x) + f(c - h x) of the
previous rules' nodes in the order x1, x2, x3):
  x1[5], w10[5]        G10 nodes and weights
  x2[5]                the Kronrod nodes other than 0
  w21a[5], w21b[6]     K21 weights at x1, and at x2 then the centre
  x3[11]               P43's new nodes
  w43a[10], w43b[12]   P43 weights at x1, x2, and at x3 then the centre
  x4[22]               P87's new nodes
  w87a[21], w87b[23]   P87 weights at x1, x2, x3, and at x4 then the centre

Run: python pplacer_gb300/csrc/make_qng_rules.py  (needs mpmath)
"""
import os

import mpmath as mp

mp.mp.dps = 120


def _poly_from_roots(roots):
    c = [mp.mpf(1)]
    for r in roots:
        n = [mp.mpf(0)] * (len(c) + 1)
        for i, a in enumerate(c):
            n[i] += a
            n[i + 1] -= a * r
        c = n
    return c  # highest degree first


def _weighted_moment(W, i):
    """int_{-1}^{1} W(x) x^i dx for W's coefficients, highest degree first."""
    deg = len(W) - 1
    s = mp.mpf(0)
    for j, a in enumerate(W):
        p = deg - j + i
        if p % 2 == 0:
            s += a * mp.mpf(2) / (p + 1)
    return s


def _extension(nodes, m):
    """Roots of the monic degree-m polynomial orthogonal to x^0..x^{m-1} with
    the weight prod (x - t), t in nodes."""
    W = _poly_from_roots(nodes)
    M = [_weighted_moment(W, i) for i in range(2 * m + 1)]
    A = mp.matrix(m, m)
    b = mp.matrix(m, 1)
    for k in range(m):
        for j in range(m):
            A[k, j] = M[k + j]
        b[k] = -M[k + m]
    c = mp.lu_solve(A, b)
    coeffs = [mp.mpf(1)] + [c[j] for j in range(m - 1, -1, -1)]
    return sorted(mp.re(x) for x in mp.polyroots(coeffs, maxsteps=500, extraprec=400))


def _weights(nodes):
    n = len(nodes)
    A = mp.matrix(n, n)
    b = mp.matrix(n, 1)
    for k in range(n):
        for j, t in enumerate(nodes):
            A[k, j] = mp.legendre(k, t)
        b[k] = 2 if k == 0 else 0
    w = mp.lu_solve(A, b)
    return {nodes[j]: w[j] for j in range(n)}


def rules():
    """The QNG tables as lists of Python floats (correctly rounded)."""
    p10 = mp.taylor(lambda x: mp.legendre(10, x), 0, 10)[::-1]
    g10 = sorted(mp.re(x) for x in mp.polyroots(p10, maxsteps=200, extraprec=200))
    k11 = _extension(g10, 11)
    p22 = _extension(g10 + k11, 22)
    p44 = _extension(g10 + k11 + p22, 44)

    def pos(v):  # positive nodes, largest first
        return sorted((x for x in v if x > mp.mpf(10) ** -60), reverse=True)
    x1, x2, x3, x4 = pos(g10), pos(k11), pos(p22), pos(p44)
    zero = [x for x in k11 if abs(x) < mp.mpf(10) ** -60][0]
    wg = _weights(sorted(g10))
    wk = _weights(sorted(g10 + k11))
    w43 = _weights(sorted(g10 + k11 + p22))
    w87 = _weights(sorted(g10 + k11 + p22 + p44))
    f = lambda v: [float(x) for x in v]
    return {
        "x1": f(x1), "w10": f(wg[x] for x in x1),
        "x2": f(x2), "w21a": f(wk[x] for x in x1), "w21b": f([wk[x] for x in x2] + [wk[zero]]),
        "x3": f(x3), "w43a": f(w43[x] for x in x1 + x2), "w43b": f([w43[x] for x in x3] + [w43[zero]]),
        "x4": f(x4), "w87a": f(w87[x] for x in x1 + x2 + x3), "w87b": f([w87[x] for x in x4] + [w87[zero]]),
    }


ORDER = ["x1", "w10", "x2", "w21a", "w21b", "x3", "w43a", "w43b", "x4", "w87a", "w87b"]


def write_header(path):
    r = rules()
    lines = ["// Generated by make_qng_rules.py: the nested 10/21/43/87-point Gauss-",
             "// Kronrod-Patterson rules of the QNG integrator, computed from their",
             "// definition (see that script for the layout); device constants of the",
             "// posterior-probability integral's QNG replica.",
             "#pragma once", "", "namespace pgb {", "namespace qng {", ""]
    for name in ORDER:
        vals = r[name]
        lines.append("__device__ const double %s[%d] = {" % (name, len(vals)))
        for i in range(0, len(vals), 3):
            lines.append("    " + ", ".join(repr(v) for v in vals[i:i + 3]) + ",")
        lines.append("};")
    lines += ["", "}  // namespace qng", "}  // namespace pgb", ""]
    with open(path, "w") as fh:
        fh.write("\n".join(lines))


if __name__ == "__main__":
    write_header(os.path.join(os.path.dirname(os.path.abspath(__file__)), "qng_rules.h"))
