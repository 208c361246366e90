"""Scratch reuse across pairs of different sizes. A persistent launch gives
each resident CTA one scratch slot and lets it take pairs in turn, so a slot
serves pairs of several sizes one after another. This batch has 1216
homography pairs, more than the engine's resident CTAs (the 64 KB
correspondence tile alone allows at most three per SM, 456 on 152 SMs).
Pair sizes are log-uniform over 300-6000 correspondences and inlier ratios
uniform over 5-60 %, on a 16^4 grid. Every pair must equal the oracle: masks,
statuses, iteration and graph-cut counts, models within 1e-6 relative
Frobenius error."""
import os

import numpy as np
import pytest

from pygcransac import _abi, synthetic as S

pytestmark = pytest.mark.gpu

MODEL_TOL = 1e-6
PAIRS = 1216


def test_mixed_sizes_with_slot_reuse_match_oracle(oracle, gcr):
    rng = np.random.default_rng(77)
    ns = np.exp(rng.uniform(np.log(300), np.log(6000), PAIRS)).astype(int)
    ratios = rng.uniform(0.05, 0.6, PAIRS)
    pairs = [S.homography_pair(900 + i, n=int(ns[i]), inlier_ratio=float(ratios[i])) for i in range(PAIRS)]
    p = _abi.Params(threshold=3.0, confidence=0.99, spatial_coherence_weight=0.975, neighborhood_size=16,
                    max_iterations=10000, min_iterations=50, sampler=0, neighborhood=0, lo_number=50, seed=0)
    seeds = np.arange(PAIRS, dtype=np.uint64) + np.uint64(5)
    models, masks, stats = gcr.find_batch(_abi.GCR_HOMOGRAPHY, [q["corr"] for q in pairs],
                                          [q["size"] for q in pairs], p, seeds=seeds)
    corr = np.concatenate([q["corr"] for q in pairs])
    offsets = np.zeros(PAIRS + 1, np.int64)
    offsets[1:] = np.cumsum([len(q["corr"]) for q in pairs])
    sz = np.zeros(PAIRS, _abi.SIZE_DTYPE)
    s = np.array([q["size"] for q in pairs])
    sz["h1"], sz["w1"], sz["h2"], sz["w2"] = s[:, 0], s[:, 1], s[:, 2], s[:, 3]
    m_o, k_o, st_o, _ = oracle.find_batch(_abi.GCR_HOMOGRAPHY, corr, offsets, sz, p, seeds=seeds,
                                          threads=os.cpu_count() or 1)
    assert np.array_equal(stats["status"], st_o["status"])
    assert np.array_equal(stats["iteration_number"], st_o["iteration_number"])
    assert np.array_equal(stats["graph_cut_number"], st_o["graph_cut_number"])
    for i in range(PAIRS):
        assert np.array_equal(masks[i], k_o[offsets[i]:offsets[i + 1]]), i
        if st_o["status"][i] == 0:
            a = models[i].ravel() / np.linalg.norm(models[i])
            b = m_o[i] / np.linalg.norm(m_o[i])
            assert min(np.linalg.norm(a - b), np.linalg.norm(a + b)) < MODEL_TOL, i
