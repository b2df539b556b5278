"""Host-side logic: model construction, synthetic workloads, pre-masking."""
import json
import os

import numpy as np
import pytest

from pplacer_gb300 import model as M
from pplacer_gb300 import synth

GOLD = os.path.join(os.path.dirname(__file__), "golden")


def test_discrete_gamma_kat():
    k = json.load(open(os.path.join(GOLD, "gamma_kat.json")))
    np.testing.assert_allclose(M.discrete_gamma(k["n_cat"], k["alpha"]), k["rates"], rtol=1e-10)


def test_diagd_matches_oracle(oracle_lib):
    """LAPACK-based Diagd (host) and the oracle's Jacobi Diagd give the same P(t)."""
    O = oracle_lib
    rng = np.random.default_rng(3)
    for K in (4, 20):
        ex, pi = synth.random_gtr(rng, K, 0.7, 5.0)
        x1, l1, xi1 = M.diagd_normed(ex, pi)
        x2, l2, xi2 = O.diagd_normed(ex, pi)
        for t in (1e-6, 0.03, 0.7, 3.0):
            P1 = (x1 * np.exp(l1 * t)[None, :]) @ xi1.T
            P2 = O.diagd_to_exp(x2, l2, xi2, t)
            np.testing.assert_allclose(P1, P2, rtol=1e-10, atol=1e-13)
            np.testing.assert_allclose(P1.sum(1), 1.0, atol=1e-12)


def test_emper_freq_matches_oracle(oracle_lib):
    fx = json.load(open(os.path.join(GOLD, "like_gtr.json")))
    np.testing.assert_allclose(M.emper_freq(fx["seqs"], 4), oracle_lib.emper_freq(fx["seqs"], 4), rtol=1e-15)


def test_synthetic_workload_shapes():
    w = synth.make_workload("cpu_small", n_queries=20)
    n = w.n_nodes
    assert n == 2 * 100 - 1
    root = np.where(w.parent < 0)[0]
    assert len(root) == 1 and root[0] == n - 1
    assert np.all(w.parent[:-1] > np.arange(n - 1))  # post-order
    assert w.n_sites == 1000 and len(w.ref_seqs) == 100
    np.testing.assert_allclose(w.rates, M.discrete_gamma(4, 0.7), rtol=1e-10)
    for q in w.query_seqs:
        L = len(q.strip("-"))
        assert 150 <= L <= 400 and len(q) == 1000


def test_premask_drops_all_gap_columns():
    refs = ["AC-T", "AG-T", "A--T"]
    qs = ["-CGT", "-C--"]
    r, q, mask = M.premask(refs, qs)
    assert list(mask) == [False, True, False, True]
    assert r == ["CT", "GT", "-T"] and q == ["CT", "C-"]
    with pytest.raises(ValueError):
        M.premask(refs, ["--G-"])  # only column 2, all-gap in the references
