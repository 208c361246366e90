"""Grid cells above the warp flow solver's 256 points.

Such a cell is cut by the whole CTA with the closed form of a clique's minimum
cut (the best source set of every size from one sort of the cell's points by
their distance term). These tests hold it to the oracle, whose labelling runs
Dinic's maximum flow on the whole graph with no cell limit: exact masks,
statuses, iteration and graph-cut counts and models within 1e-6, on pairs
with one 900-point cell, with a 1000-point cell among ordinary ones, with
cells of a few hundred to a few thousand points, and with a weak spatial term
that splits cells; and the results must not depend on what the context's
scratch held before (the slots are re-carved in place when the model kind
changes)."""
import numpy as np
import pytest

from pygcransac import _abi, synthetic as S

pytestmark = pytest.mark.gpu

MODEL_TOL = 1e-6


def params(**kw):
    p = _abi.Params(threshold=3.0, confidence=0.99, spatial_coherence_weight=0.975, neighborhood_size=4,
                    max_iterations=10000, min_iterations=50, sampler=0, neighborhood=0, lo_number=50, seed=0)
    for k, v in kw.items():
        setattr(p, k, v)
    return p


def rel_err(a, b):
    a = a / np.linalg.norm(a)
    b = b / np.linalg.norm(b)
    return min(np.linalg.norm(a - b), np.linalg.norm(a + b))


def dirty_with_essential(gcr, seed):
    """One essential-matrix batch through the shared context, so the slots the
    next homography batch carves hold another kind's doubles and indices."""
    tv = S.two_view_pair(seed, n=6000, inlier_ratio=0.3)
    K = np.concatenate([tv["K"].ravel(), tv["K"].ravel()])[None]
    pe = params(threshold=0.75, neighborhood_size=8, max_iterations=300)
    gcr.find_batch(_abi.GCR_ESSENTIAL, [tv["corr"]], [tv["size"]], pe, seeds=[seed], K=K)


def check_against_oracle(oracle, gcr, pairs, p, seeds, kind=_abi.GCR_HOMOGRAPHY):
    models, masks, stats = gcr.find_batch(kind, [x["corr"] for x in pairs], [x["size"] for x in pairs], p,
                                          seeds=seeds)
    for i, x in enumerate(pairs):
        rc, M_o, m_o, st_o = oracle.find(kind, x["corr"], oracle.make_size(*x["size"]), p, seed=seeds[i])
        assert stats["status"][i] == rc, (i, stats["status"][i], rc)
        assert np.array_equal(masks[i], m_o), f"pair {i}: mask differs at {np.nonzero(masks[i] != m_o)[0][:10]}"
        assert stats["iteration_number"][i] == st_o.iteration_number, i
        assert stats["graph_cut_number"][i] == st_o.graph_cut_number, i
        if rc == 0:
            assert rel_err(models[i], M_o) < MODEL_TOL, i
    return models, masks, stats


def test_one_cell_pair_matches_oracle_whatever_the_scratch_held(oracle, gcr):
    pr = S.homography_pair(41, n=900, inlier_ratio=0.4)
    p = params(neighborhood_size=1)  # one grid cell holding all 900 points
    dirty_with_essential(gcr, 5)
    m1, k1, s1 = check_against_oracle(oracle, gcr, [pr], p, [7])
    assert s1["status"][0] == _abi.GCR_OK
    # a different history: a larger homography batch, then the same pair again
    big = S.homography_pair(43, n=6000)
    gcr.find_batch(_abi.GCR_HOMOGRAPHY, [big["corr"]], [big["size"]], params(), seeds=[3])
    m2, k2, s2 = gcr.find_batch(_abi.GCR_HOMOGRAPHY, [pr["corr"]], [pr["size"]], p, seeds=[7])
    assert np.array_equal(k1[0], k2[0]) and np.array_equal(m1, m2) and np.array_equal(s1, s2)


@pytest.mark.parametrize("lam", [0.975, 0.02, 0.002])
def test_large_cells_match_oracle(oracle, gcr, lam):
    """2^4 and 1^4 grids over 1500-6000 points: cells of hundreds to thousands
    of points; a weak spatial term (0.02, 0.002) makes the cuts split cells."""
    pairs = [S.homography_pair(70 + i, n=n, inlier_ratio=r)
             for i, (n, r) in enumerate([(1500, 0.4), (3000, 0.3), (6000, 0.5)])]
    check_against_oracle(oracle, gcr, pairs, params(neighborhood_size=2, spatial_coherence_weight=lam), [1, 2, 3])
    check_against_oracle(oracle, gcr, pairs[:2], params(neighborhood_size=1, spatial_coherence_weight=lam), [4, 5])


def test_thousand_point_cell_among_ordinary_cells(oracle, gcr):
    """A pair whose inliers crowd one 8^4 cell: 1000 correspondences inside one
    cell of both images, plus uniform outliers in the other cells."""
    rng = np.random.default_rng(3)
    base = S.homography_pair(90, n=3000, inlier_ratio=0.0)
    # a small shear and shift keeps the inliers inside cell (0, 0) of both images
    H = np.array([[1.01, 0.02, 4.0], [-0.01, 0.99, 3.0], [0.0, 0.0, 1.0]])
    x1 = rng.uniform([10, 10], [70, 50], (1000, 2))
    x2 = S.project_h(H, x1) + rng.normal(0, 0.5, (1000, 2))
    keep = (x2[:, 0] > 0) & (x2[:, 0] < 80) & (x2[:, 1] > 0) & (x2[:, 1] < 60)
    assert keep.sum() > 950
    corr = np.r_[np.c_[x1[keep], x2[keep]], base["corr"][:2000]]
    corr = corr[rng.permutation(len(corr))]
    pr = dict(corr=np.ascontiguousarray(corr), size=base["size"])
    p = params(neighborhood_size=8, threshold=2.0)
    _, masks, stats = check_against_oracle(oracle, gcr, [pr], p, [11])
    assert stats["graph_cut_number"][0] >= 1


def test_fundamental_large_cells(oracle, gcr):
    pf = [S.two_view_pair(95 + i, n=2500, inlier_ratio=0.4) for i in range(2)]
    check_against_oracle(oracle, gcr, pf, params(threshold=0.75, neighborhood_size=2, max_iterations=1000), [1, 2],
                         kind=_abi.GCR_FUNDAMENTAL)
