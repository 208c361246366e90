"""Grid cells above the flow solver's capacity (256 points per cell).

The labelling leaves such a cell to its unary terms and the pair ends with
GCR_CAPACITY. These tests hold the engine to three things there: the status is
reported, the run still returns a model and a mask of the pair's size, and the
result does not depend on what the context's scratch held before (the slots
are re-carved in place when the model kind changes, so an earlier batch of
another kind leaves its data where the labels of this pair are kept)."""
import numpy as np
import pytest

from pygcransac import _abi, synthetic as S

pytestmark = pytest.mark.gpu


def params(**kw):
    p = _abi.Params(threshold=3.0, confidence=0.99, spatial_coherence_weight=0.975, neighborhood_size=4,
                    max_iterations=10000, min_iterations=50, sampler=0, neighborhood=0, lo_number=50, seed=0)
    for k, v in kw.items():
        setattr(p, k, v)
    return p


def dirty_with_essential(gcr, seed):
    """One essential-matrix batch through the shared context, so the slots the
    next homography batch carves hold another kind's doubles and indices."""
    tv = S.two_view_pair(seed, n=6000, inlier_ratio=0.3)
    K = np.concatenate([tv["K"].ravel(), tv["K"].ravel()])[None]
    pe = params(threshold=0.75, neighborhood_size=8, max_iterations=300)
    gcr.find_batch(_abi.GCR_ESSENTIAL, [tv["corr"]], [tv["size"]], pe, seeds=[seed], K=K)


def test_oversize_cell_reported_and_independent_of_scratch(gcr):
    pr = S.homography_pair(41, n=900, inlier_ratio=0.4)
    p = params(neighborhood_size=1)  # one grid cell holding all 900 points
    dirty_with_essential(gcr, 5)
    m1, k1, s1 = gcr.find_batch(_abi.GCR_HOMOGRAPHY, [pr["corr"]], [pr["size"]], p, seeds=[7])
    # a different history: a larger homography batch, then the same pair again
    big = S.homography_pair(43, n=6000)
    gcr.find_batch(_abi.GCR_HOMOGRAPHY, [big["corr"]], [big["size"]], params(), seeds=[3])
    m2, k2, s2 = gcr.find_batch(_abi.GCR_HOMOGRAPHY, [pr["corr"]], [pr["size"]], p, seeds=[7])
    assert s1["status"][0] == _abi.GCR_CAPACITY
    assert len(k1[0]) == 900 and 4 < k1[0].sum() <= 900
    assert np.array_equal(k1[0], k2[0])
    assert np.array_equal(m1, m2)
    for f in ("status", "iteration_number", "graph_cut_number", "inlier_number", "models_scored", "flags"):
        assert s1[f][0] == s2[f][0], f
    H = m1[0] / m1[0][2, 2]
    assert S.homography_error(H, pr["H_gt"]) < 2.0


def test_ordinary_pairs_after_capacity_pairs_match_oracle(gcr, oracle):
    """Capacity pairs (one cell each) run first in slots dirtied by another
    kind; ordinary 8^4-grid pairs on the same slots then match the oracle
    exactly (masks, statuses, iteration counts)."""
    pairs = [S.homography_pair(60 + i, n=700 + 100 * i) for i in range(3)]
    dirty_with_essential(gcr, 6)
    _, k, s = gcr.find_batch(_abi.GCR_HOMOGRAPHY, [x["corr"] for x in pairs], [x["size"] for x in pairs],
                             params(neighborhood_size=1), seeds=[1, 2, 3])
    assert all(s["status"] == _abi.GCR_CAPACITY)
    assert all(len(k[i]) == len(x["corr"]) for i, x in enumerate(pairs))
    q = params(neighborhood_size=8)
    _, k, s = gcr.find_batch(_abi.GCR_HOMOGRAPHY, [x["corr"] for x in pairs], [x["size"] for x in pairs], q,
                             seeds=[1, 2, 3])
    for i, x in enumerate(pairs):
        rc, H_o, m_o, st_o = oracle.find(0, x["corr"], oracle.make_size(*x["size"]), q, seed=i + 1)
        assert s["status"][i] == rc
        assert np.array_equal(k[i], m_o), i
        assert s["iteration_number"][i] == st_o.iteration_number
        assert s["graph_cut_number"][i] == st_o.graph_cut_number
