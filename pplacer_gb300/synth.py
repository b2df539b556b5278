"""Seeded synthetic placement workloads.

The reference publishes no benchmark data set for placement, so every workload
is generated here from a seed: a Yule-process topology with i.i.d.
exponential branch lengths, a random reversible rate matrix, Gamma or CAT
site rates, an alignment simulated down the tree, and query reads simulated
from random positions on random edges.  Node ids are post-order (children
before parents, children in increasing id order), which is how pplacer
numbers a Newick tree (pplacer_src/newick_parser.mly:50-59).

The five named workloads match the sizes and distributions of the benchmark
configurations:
  cpu_small   100 taxa, DNA GTR+G4, 1,000 sites, 200 queries of 150-400 sites
  dna_1k      1,000 taxa, DNA GTR+G4, 1,500 sites, 10,000 queries 100-1,500
  dna_2k      2,000 taxa, DNA GTR+G4, 3,000 sites, 50,000 queries 200-3,000
  aa_500      500 taxa, 20-state + G4, 400 sites, 5,000 queries 60-400
  cat_5k      5,000 taxa, DNA GTR + CAT(20), 1,500 sites, 100,000 queries
"""
from dataclasses import dataclass, field

import numpy as np

NUC = "ACGT"
AA = "ARNDCQEGHILKMFPSTWYV"


@dataclass
class Workload:
    name: str
    seed: int
    K: int
    exch: np.ndarray           # K x K symmetric exchangeabilities (diagonal 0)
    statd: np.ndarray          # K stationary frequencies
    rates: np.ndarray          # Gamma category rates, or CAT category rates
    site_cats: np.ndarray      # per-site CAT category (None for Gamma)
    parent: np.ndarray         # int32 [n_nodes], -1 at the root
    bl: np.ndarray             # float64 [n_nodes], 0 at the root
    leaf_row: np.ndarray       # int32 [n_nodes] alignment row of each leaf, -1 inside
    ref_seqs: list             # reference alignment rows (str)
    query_seqs: list           # query rows (str), same length
    prefs: dict = field(default_factory=dict)
    alpha: float = 0.0

    @property
    def n_nodes(self):
        return len(self.parent)

    @property
    def n_sites(self):
        return len(self.ref_seqs[0])


def yule_tree(rng, n_taxa, mean_bl):
    """Yule topology (uniformly random lineage splits), i.i.d. Exp(mean_bl)
    branch lengths, post-order ids."""
    # grow with temporary ids: node = (children list)
    children = {0: []}
    tips = [0]
    nxt = 1
    while len(tips) < n_taxa:
        i = rng.integers(len(tips))
        t = tips.pop(i)
        a, b = nxt, nxt + 1
        nxt += 2
        children[t] = [a, b]
        children[a] = []
        children[b] = []
        tips += [a, b]
    # post-order renumbering
    order = []
    stack = [(0, False)]
    while stack:
        n, done = stack.pop()
        if done:
            order.append(n)
            continue
        stack.append((n, True))
        for c in reversed(children[n]):
            stack.append((c, False))
    new_id = {old: i for i, old in enumerate(order)}
    n_nodes = len(order)
    parent = np.full(n_nodes, -1, dtype=np.int32)
    for old, kids in children.items():
        for c in kids:
            parent[new_id[c]] = new_id[old]
    bl = rng.exponential(mean_bl, size=n_nodes)
    bl[parent < 0] = 0.0
    return parent, bl


def random_gtr(rng, K, sigma, dir_alpha):
    ex = np.zeros((K, K))
    iu = np.triu_indices(K, 1)
    ex[iu] = rng.lognormal(0.0, sigma, size=len(iu[0]))
    ex = ex + ex.T
    statd = rng.dirichlet([dir_alpha] * K)
    return ex, statd


def rate_matrix(ex, statd):
    """Q_ij = r_ij pi_j, rows sum to zero, mean rate one (pplacer_src/diagd.ml:140-172)."""
    Q = ex * statd[None, :]
    np.fill_diagonal(Q, 0.0)
    np.fill_diagonal(Q, -Q.sum(1))
    return Q / -(np.diag(Q) @ statd)


def _expm(A):
    # scaling and squaring with a Pade(6) core; adequate for simulation
    n = A.shape[0]
    norm = np.abs(A).sum(1).max()
    s = max(0, int(np.ceil(np.log2(norm))) + 1) if norm > 0 else 0
    B = A / (2 ** s)
    # Pade (6,6) coefficients
    cc = [1.0, 1 / 2, 5 / 44, 1 / 66, 1 / 792, 1 / 15840, 1 / 665280]
    Bp = np.eye(n)
    N = np.zeros((n, n))
    D = np.zeros((n, n))
    for k, ck in enumerate(cc):
        N += ck * Bp
        D += ((-1) ** k) * ck * Bp
        Bp = Bp @ B
    E = np.linalg.solve(D, N)
    for _ in range(s):
        E = E @ E
    return E


def simulate(rng, parent, bl, Q, statd, site_rate, n_sites):
    """Simulate states down the tree; site_rate[s] scales the branch lengths."""
    n_nodes = len(parent)
    K = len(statd)
    root = int(np.where(parent < 0)[0][0])
    states = np.zeros((n_nodes, n_sites), dtype=np.int8)
    states[root] = rng.choice(K, size=n_sites, p=statd)
    uniq, inv = np.unique(site_rate, return_inverse=True)
    # children have smaller ids than parents: go from the root downwards
    for node in range(n_nodes - 1, -1, -1):
        p = parent[node]
        if p < 0:
            continue
        ps = states[p]
        out = np.empty(n_sites, dtype=np.int8)
        for ui, r in enumerate(uniq):
            sel = inv == ui
            P = _expm(Q * (bl[node] * r))
            cum = np.cumsum(P, axis=1)
            u = rng.random(sel.sum())
            out[sel] = (u[:, None] > cum[ps[sel]]).sum(1).clip(0, K - 1)
        states[node] = out
    return states


def _evolve_states(rng, Q, ps, t, rates_site):
    K = Q.shape[0]
    out = np.empty(len(ps), dtype=np.int8)
    uniq, inv = np.unique(rates_site, return_inverse=True)
    for ui, r in enumerate(uniq):
        sel = inv == ui
        P = _expm(Q * (t * r))
        cum = np.cumsum(P, axis=1)
        u = rng.random(sel.sum())
        out[sel] = (u[:, None] > cum[ps[sel]]).sum(1).clip(0, K - 1)
    return out


def make_queries(rng, parent, bl, states, Q, site_rate, n_queries, len_lo, len_hi, noise, gap_frac,
                 alphabet, pend_mean):
    n_nodes, n_sites = states.shape
    K = len(alphabet)
    nonroot = np.where(parent >= 0)[0]
    alpha = np.frombuffer(alphabet.encode(), dtype=np.uint8)
    out = []
    for _ in range(n_queries):
        e = int(rng.choice(nonroot))
        p = parent[e]
        frac = rng.random()
        attach = _evolve_states(rng, Q, states[p], bl[e] * (1 - frac), site_rate)
        seq = _evolve_states(rng, Q, attach, rng.exponential(pend_mean), site_rate)
        L = int(rng.integers(len_lo, len_hi + 1))
        L = min(L, n_sites)
        start = int(rng.integers(0, n_sites - L + 1))
        chars = np.full(n_sites, ord("-"), dtype=np.uint8)
        win = seq[start:start + L].copy()
        if noise > 0:
            flip = rng.random(L) < noise
            win[flip] = (win[flip] + rng.integers(1, K, size=flip.sum())) % K
        wc = alpha[win]
        if gap_frac > 0:
            wc[rng.random(L) < gap_frac] = ord("-")
        chars[start:start + L] = wc
        out.append(chars.tobytes().decode())
    return out


def make_workload(name, n_queries=None, **overrides):
    """Build one of the named workloads (n_queries overrides the query count;
    other keyword arguments override the spec, e.g. taxa=50, sites=200)."""
    specs = {
        "cpu_small": dict(seed=1000, taxa=100, mean_bl=0.05, K=4, sites=1000, Q=200, lo=150, hi=400,
                          noise=0.0, gaps=0.0, cat=False, alpha=0.7,
                          prefs=dict(max_strikes=0)),
        "dna_1k": dict(seed=1001, taxa=1000, mean_bl=0.05, K=4, sites=1500, Q=10000, lo=100, hi=1500,
                       noise=0.02, gaps=0.01, cat=False, alpha=0.7, prefs=dict(keep_at_most=7, max_strikes=6)),
        "dna_2k": dict(seed=1002, taxa=2000, mean_bl=0.04, K=4, sites=3000, Q=50000, lo=200, hi=3000,
                       noise=0.0, gaps=0.0, cat=False, alpha=0.7, prefs=dict()),
        "aa_500": dict(seed=1003, taxa=500, mean_bl=0.1, K=20, sites=400, Q=5000, lo=60, hi=400,
                       noise=0.0, gaps=0.0, cat=False, alpha=0.9, prefs=dict()),
        "cat_5k": dict(seed=1004, taxa=5000, mean_bl=0.03, K=4, sites=1500, Q=100000, lo=100, hi=1500,
                       noise=0.0, gaps=0.0, cat=True, alpha=0.0, prefs=dict()),
    }
    sp = dict(specs[name])
    sp.setdefault("n_rates", 4)
    sp.update(overrides)
    rng = np.random.default_rng(sp["seed"])
    K = sp["K"]
    parent, bl = yule_tree(rng, sp["taxa"], sp["mean_bl"])
    if K == 4:
        ex, statd = random_gtr(rng, 4, 0.5, 10.0)
        alphabet = NUC
    else:
        ex, statd = random_gtr(rng, 20, 1.0, 5.0)
        alphabet = AA
    Qm = rate_matrix(ex, statd)
    S = sp["sites"]
    if sp["cat"]:
        cat_rates = rng.gamma(0.5, 1.0, size=20)
        cat_rates = cat_rates / cat_rates.mean()
        site_cats = rng.integers(0, 20, size=S).astype(np.int32)
        rates = cat_rates
        site_rate = cat_rates[site_cats]
    else:
        from scipy.special import gammaincinv, gammainc
        a, nr = sp["alpha"], sp["n_rates"]
        # discrete Gamma(a, a) category means (Yang 1994), mean one
        cuts = [0.0] + [gammaincinv(a, i / nr) for i in range(1, nr)] + [np.inf]
        fr = [gammainc(a + 1, c) if np.isfinite(c) else 1.0 for c in cuts]
        rates = np.array([fr[i + 1] - fr[i] for i in range(nr)]) * nr
        site_cats = None
        site_rate = rates[rng.integers(0, nr, size=S)]
    states = simulate(rng, parent, bl, Qm, statd, site_rate, S)
    alpha_arr = np.frombuffer(alphabet.encode(), dtype=np.uint8)
    is_leaf = np.ones(len(parent), dtype=bool)
    is_leaf[parent[parent >= 0]] = False
    leaf_ids = np.where(is_leaf)[0]
    leaf_row = np.full(len(parent), -1, dtype=np.int32)
    leaf_row[leaf_ids] = np.arange(len(leaf_ids), dtype=np.int32)
    ref_seqs = [alpha_arr[states[i]].tobytes().decode() for i in leaf_ids]
    nq = sp["Q"] if n_queries is None else n_queries
    queries = make_queries(rng, parent, bl, states, Qm, site_rate, nq, sp["lo"], sp["hi"], sp["noise"],
                           sp["gaps"], alphabet, pend_mean=sp["mean_bl"])
    return Workload(name=name, seed=sp["seed"], K=K, exch=ex, statd=statd, rates=np.asarray(rates, dtype=np.float64),
                    site_cats=site_cats, parent=parent, bl=bl, leaf_row=leaf_row, ref_seqs=ref_seqs,
                    query_seqs=queries, prefs=sp["prefs"], alpha=sp["alpha"])
