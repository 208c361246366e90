"""GPU parity of the homography path: the device engine against the oracle on
the same seeded inputs, through the C-ABI. Masks must be identical, models
equal to 1e-6 relative Frobenius error after normalisation, and the run
statistics (iterations, graph-cuts) the same."""
import numpy as np
import pytest

from pygcransac import _abi, synthetic as S

pytestmark = pytest.mark.gpu

MODEL_TOL = 1e-6


def h_params(**kw):
    p = _abi.Params(threshold=3.0, confidence=0.99, spatial_coherence_weight=0.975, neighborhood_size=4,
                    max_iterations=10000, min_iterations=50, sampler=0, neighborhood=0, lo_number=50, seed=0)
    for k, v in kw.items():
        setattr(p, k, v)
    return p


def rel_model_err(a, b):
    a = a / np.linalg.norm(a)
    b = b / np.linalg.norm(b)
    return min(np.linalg.norm(a - b), np.linalg.norm(a + b))


def compare(oracle, gcr, corr, size, p, seed):
    rc_o, H_o, m_o, st_o = oracle.find(0, corr, oracle.make_size(*size), p, seed=seed)
    models, masks, stats = gcr.find_batch(_abi.GCR_HOMOGRAPHY, [corr], [size], p, seeds=[seed])
    assert stats["status"][0] == rc_o, (stats["status"][0], rc_o)
    assert np.array_equal(masks[0], m_o), f"mask differs at {np.nonzero(masks[0] != m_o)[0][:10]}"
    if rc_o == 0:
        assert rel_model_err(models[0], H_o) < MODEL_TOL
    assert stats["iteration_number"][0] == st_o.iteration_number
    assert stats["graph_cut_number"][0] == st_o.graph_cut_number
    assert stats["models_scored"][0] == st_o.models_scored
    assert stats["flags"][0] == st_o.flags
    return models[0], masks[0]


@pytest.mark.parametrize("seed", range(8))
def test_homography_config_pairs(oracle, gcr, seed):
    pr = S.homography_pair(seed)
    compare(oracle, gcr, pr["corr"], pr["size"], h_params(), seed)


@pytest.mark.parametrize("n,ratio", [(4, 1.0), (9, 0.6), (60, 0.3), (300, 0.15), (5000, 0.4)])
def test_homography_sizes(oracle, gcr, n, ratio):
    pr = S.homography_pair(100 + n, n=n, inlier_ratio=ratio)
    compare(oracle, gcr, pr["corr"], pr["size"], h_params(), 11)


def test_homography_prosac(oracle, gcr):
    pr = S.homography_pair(21)
    compare(oracle, gcr, pr["corr"], pr["size"], h_params(sampler=1), 3)


def test_homography_no_spatial_term(oracle, gcr):
    pr = S.homography_pair(22)
    compare(oracle, gcr, pr["corr"], pr["size"], h_params(spatial_coherence_weight=0.0), 4)


def test_homography_pure_outliers(oracle, gcr):
    rng = np.random.default_rng(5)
    corr = rng.uniform(0, 480, (40, 4))
    compare(oracle, gcr, corr, (480, 640, 480, 640), h_params(threshold=0.05), 1)


def test_homography_batch_matches_single(oracle, gcr):
    pairs = [S.homography_pair(200 + i, n=500 + 150 * i) for i in range(12)]
    p = h_params()
    seeds = list(range(12))
    models, masks, stats = gcr.find_batch(_abi.GCR_HOMOGRAPHY, [q["corr"] for q in pairs],
                                          [q["size"] for q in pairs], p, seeds=seeds)
    for i, q in enumerate(pairs):
        rc, H_o, m_o, st_o = oracle.find(0, q["corr"], oracle.make_size(*q["size"]), p, seed=seeds[i])
        assert stats["status"][i] == rc
        assert np.array_equal(masks[i], m_o), i
        assert rel_model_err(models[i], H_o) < MODEL_TOL


def test_drop_in_entry_point(oracle, gcr):
    pr = S.homography_pair(31)
    H, mask = gcr.findHomography(pr["corr"], 480, 640, 480, 640, threshold=3.0, use_sprt=False,
                                 use_space_partitioning=False, sampler=0, seed=9)
    rc, H_o, m_o, _ = oracle.find(0, pr["corr"], oracle.make_size(480, 640, 480, 640),
                                  h_params(spatial_coherence_weight=0.975), seed=9)
    assert H is not None and np.array_equal(mask, m_o)
    assert S.homography_error(H, pr["H_gt"]) < 1.0


def test_homography_pnapsac(oracle, gcr):
    pr = S.homography_pair(23)
    compare(oracle, gcr, pr["corr"], pr["size"], h_params(sampler=2), 6)
