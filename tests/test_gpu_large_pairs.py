"""Parity on pairs of 9000-40000 correspondences with a 16^4 grid: one batch per
model kind with pairs of different sizes (so a CTA's scratch may serve pairs
of several sizes), every pair checked against the oracle on exact masks,
statuses and iteration / graph-cut counts, models within 1e-6 relative
Frobenius error."""
import numpy as np
import pytest

from pygcransac import _abi, synthetic as S

pytestmark = pytest.mark.gpu

MODEL_TOL = 1e-6
SIZES = [(12000, 0.45), (9000, 0.3), (10500, 0.55)]
# the largest pairs of the mixed serving batch, inlier sets up to 12000 points
SIZES_XL = [(40000, 0.25), (24000, 0.5)]
CASES = [(SIZES, 0), (SIZES_XL, 100)]


def params(threshold, lam):
    return _abi.Params(threshold=threshold, confidence=0.99, spatial_coherence_weight=lam, neighborhood_size=16,
                       max_iterations=2000, min_iterations=50, sampler=0, neighborhood=0, lo_number=50, seed=0)


def rel_err(a, b):
    a = a / np.linalg.norm(a)
    b = b / np.linalg.norm(b)
    return min(np.linalg.norm(a - b), np.linalg.norm(a + b))


def check_batch(oracle, gcr, kind, pairs, p, K=None):
    seeds = [31 + i for i in range(len(pairs))]
    Kb = None if K is None else np.stack([np.concatenate([k.ravel(), k.ravel()]) for k in K])
    models, masks, stats = gcr.find_batch(kind, [q["corr"] for q in pairs], [q["size"] for q in pairs], p,
                                          seeds=seeds, K=Kb)
    for i, q in enumerate(pairs):
        kw = {} if K is None else dict(K1=K[i], K2=K[i])
        rc, M, m_o, st = oracle.find(kind, q["corr"], oracle.make_size(*q["size"]), p, seed=seeds[i], **kw)
        assert stats["status"][i] == rc, (i, stats["status"][i], rc)
        assert np.array_equal(masks[i], m_o), f"pair {i}: mask differs at {np.nonzero(masks[i] != m_o)[0][:10]}"
        if rc == 0:
            assert rel_err(models[i], M) < MODEL_TOL, i
        assert stats["iteration_number"][i] == st.iteration_number, i
        assert stats["graph_cut_number"][i] == st.graph_cut_number, i


@pytest.mark.parametrize("sizes,base", CASES)
def test_homography_large_pairs(oracle, gcr, sizes, base):
    pairs = [S.homography_pair(400 + base + i, n=n, inlier_ratio=r) for i, (n, r) in enumerate(sizes)]
    check_batch(oracle, gcr, _abi.GCR_HOMOGRAPHY, pairs, params(3.0, 0.975))


@pytest.mark.parametrize("sizes,base", CASES)
def test_fundamental_large_pairs(oracle, gcr, sizes, base):
    pairs = [S.two_view_pair(410 + base + i, n=n, inlier_ratio=r) for i, (n, r) in enumerate(sizes)]
    check_batch(oracle, gcr, _abi.GCR_FUNDAMENTAL, pairs, params(0.75, 0.975))


@pytest.mark.parametrize("sizes,base", CASES)
def test_essential_large_pairs(oracle, gcr, sizes, base):
    pairs = [S.two_view_pair(420 + base + i, n=n, inlier_ratio=r) for i, (n, r) in enumerate(sizes)]
    check_batch(oracle, gcr, _abi.GCR_ESSENTIAL, pairs, params(0.75, 0.1), K=[q["K"] for q in pairs])
