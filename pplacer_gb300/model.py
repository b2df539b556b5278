"""Host-side model construction (FP64): what pplacer computes once before the
hot path and hands to the likelihood engine.

* ``diagd_normed`` -- Diagd.normed_of_exchangeable_pair (pplacer_src/diagd.ml:123-172):
  X diag(lambda) X^-1 = B D with B from the exchangeabilities and D = diag(pi),
  eigenvalues scaled to a mean rate of one.
* ``discrete_gamma`` -- Gamma.discrete_gamma (pplacer_src/gamma.ml:14-70).
* ``emper_freq`` -- Alignment.emper_freq (common_src/alignment.ml:186-215).
* ``premask`` -- Pplacer_run.premask (pplacer_src/pplacer_run.ml:59-144).
* ``dedup`` -- the query deduplication of pplacer_src/pplacer_run.ml:228-253.
"""
from dataclasses import dataclass

import numpy as np

NUC_CODES = "ACGTRYMKSWHBVDN-?X"
NUC_BITS = [1, 2, 4, 8, 5, 10, 3, 12, 6, 9, 11, 14, 7, 13, 15, 15, 15, 15]
PROT_CODES = "ARNDCQEGHILKMFPSTWYV"


def lv_of_char(c, K):
    """Likelihood vector of one character (nuc_models.ml:24-45, prot_models.ml:5-43)."""
    if K == 4:
        b = NUC_BITS[NUC_CODES.index(c)]
        return np.array([(b >> k) & 1 for k in range(4)], dtype=np.float64)
    v = np.zeros(K)
    if c in "-?X":
        v[:] = 1
    elif c == "B":
        v[[3, 2]] = 1
    elif c == "J":
        v[[9, 10]] = 1
    elif c == "Z":
        v[[6, 5]] = 1
    else:
        v[PROT_CODES.index(c)] = 1
    return v


def emper_freq(seqs, K):
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


def _safe_invert(x):
    return np.where(x == 0.0, 1.0, 1.0 / np.where(x == 0.0, 1.0, x))


def diagd_normed(exch, statd):
    """(x, lambda, xit) of the rate matrix for exchangeabilities ``exch`` and
    frequencies ``statd``, normalised to mean rate one."""
    r = np.asarray(exch, dtype=np.float64)
    pi = np.asarray(statd, dtype=np.float64)
    n = len(pi)
    b = r.copy()
    for i in range(n):  # b_ii = -(1/pi_i) sum_{k != i} r_ki pi_k  (diagd.ml:140-152)
        tot = sum(r[k, i] * pi[k] for k in range(n) if k != i)
        b[i, i] = -(tot * _safe_invert(pi[i]))
    if np.any(pi < 0):
        raise ValueError("negative element in the diagonal of a DB matrix!")
    d_root = np.sqrt(pi)
    sym = np.diag(d_root) @ (b @ np.diag(d_root))
    sym = 0.5 * (sym + sym.T)
    lam, u = np.linalg.eigh(sym)
    x = np.diag(_safe_invert(d_root)) @ u
    xit = np.diag(d_root) @ u
    q = (x * lam[None, :]) @ xit.T
    rate = -float(np.sum(np.diag(q) * pi))
    return x, lam / rate, xit


def discrete_gamma(n_cat, alpha):
    """Yang (1994) mean-of-category Gamma rates, normalised to mean one."""
    from scipy.special import gammainc, gammaincinv
    freq = [0.0]
    for i in range(1, n_cat):
        y = i / n_cat
        cut = 0.0 if y < gammainc(alpha, 1e-7) else float(gammaincinv(alpha, y))
        freq.append(float(gammainc(alpha + 1.0, cut)))
    freq.append(1.0)
    v = np.array([freq[i + 1] - freq[i] for i in range(n_cat)])
    return n_cat * v / v.sum()


@dataclass
class Model:
    """Gamma-mixture (site_cats None) or per-site CAT model."""
    K: int
    statd: np.ndarray
    x: np.ndarray
    lam: np.ndarray
    xit: np.ndarray
    rates: np.ndarray
    site_cats: np.ndarray = None

    @classmethod
    def from_exchangeabilities(cls, exch, statd, rates, site_cats=None):
        x, lam, xit = diagd_normed(exch, statd)
        sc = None if site_cats is None else np.ascontiguousarray(site_cats, dtype=np.int32)
        return cls(len(statd), np.asarray(statd, dtype=np.float64), x, lam, xit,
                   np.asarray(rates, dtype=np.float64), sc)

    @property
    def gcat(self):
        return self.site_cats is not None


def premask(ref_seqs, query_seqs):
    """Drop columns that are all-gap in the references or in the queries
    (pplacer_run.ml:59-144); returns the masked rows and the column mask.
    Queries that overlap no informative reference column are an error, as
    in the reference."""
    ref = np.frombuffer("".join(ref_seqs).encode(), dtype=np.uint8).reshape(len(ref_seqs), -1)
    qry = np.frombuffer("".join(query_seqs).encode(), dtype=np.uint8).reshape(len(query_seqs), -1)
    gap = np.frombuffer(b"-?", dtype=np.uint8)
    ref_inf = ~np.isin(ref, gap)
    qry_inf = ~np.isin(qry, gap)
    ref_mask = ref_inf.any(0)
    overlaps = (qry_inf & ref_mask[None, :]).any(1)
    if not overlaps.all():
        raise ValueError("query %d doesn't overlap any reference sequences" % int(np.argmin(overlaps)))
    mask = ref_mask & qry_inf.any(0)
    cut = lambda rows: [r[mask].tobytes().decode() for r in rows]
    return cut(ref), cut(qry), mask


def dedup(names, seqs):
    """Place identical query sequences once (pplacer_run.ml:228-253): returns
    (unique_seqs, name_lists), name_lists[i] holding every name whose
    sequence is unique_seqs[i], in input order.  Run it on pre-masked
    sequences, as the reference does.  Writing one pquery per unique sequence
    with each of its names at multiplicity 1 is Placerun.redup without
    ``as_mass`` (placerun.ml:95-112); ``jplace.to_jplace`` takes the name
    lists directly.  Unique sequences come in order of first appearance (the
    reference's order is its hash table's)."""
    if len(names) != len(seqs):
        raise ValueError("%d names for %d sequences" % (len(names), len(seqs)))
    index, uniq, namel = {}, [], []
    for n, s in zip(names, seqs):
        i = index.get(s)
        if i is None:
            index[s] = i = len(uniq)
            uniq.append(s)
            namel.append([])
        namel[i].append(n)
    return uniq, namel
