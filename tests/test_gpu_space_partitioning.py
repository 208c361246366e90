"""GPU parity of the space-partitioning pre-selection of homography models
(SpacePartitioningRANSAC::runHomography) alone, with SPRT and with MAGSAC++,
against the oracle on the same seeded inputs."""
import numpy as np
import pytest

from pygcransac import _abi, synthetic as S

pytestmark = pytest.mark.gpu

MODEL_TOL = 1e-6


def rel_err(a, b):
    a = a / np.linalg.norm(a)
    b = b / np.linalg.norm(b)
    return min(np.linalg.norm(a - b), np.linalg.norm(a + b))


def params(**kw):
    p = _abi.Params(threshold=3.0, confidence=0.99, spatial_coherence_weight=0.975, neighborhood_size=4,
                    max_iterations=5000, min_iterations=50, sampler=0, neighborhood=0, lo_number=50, seed=0,
                    use_space_partitioning=1, min_inlier_ratio_for_sprt=1e-5)
    for k, v in kw.items():
        setattr(p, k, v)
    return p


def compare(oracle, gcr, pr, p, seed):
    rc_o, M_o, m_o, st_o = oracle.find(_abi.GCR_HOMOGRAPHY, pr["corr"], oracle.make_size(*pr["size"]), p, seed=seed)
    models, masks, stats = gcr.find_batch(_abi.GCR_HOMOGRAPHY, [pr["corr"]], [pr["size"]], p, seeds=[seed])
    assert stats["status"][0] == rc_o
    assert np.array_equal(masks[0], m_o), f"mask differs at {np.nonzero(masks[0] != m_o)[0][:10]}"
    if rc_o == 0:
        assert rel_err(models[0], M_o) < MODEL_TOL
    assert stats["iteration_number"][0] == st_o.iteration_number
    assert stats["graph_cut_number"][0] == st_o.graph_cut_number
    assert stats["models_scored"][0] == st_o.models_scored


@pytest.mark.parametrize("seed", range(4))
def test_space_partitioning(oracle, gcr, seed):
    pr = S.homography_pair(seed, n=2000)
    compare(oracle, gcr, pr, params(), seed)


@pytest.mark.parametrize("seed", range(3))
def test_space_partitioning_with_sprt(oracle, gcr, seed):
    pr = S.homography_pair(10 + seed, n=2000)
    compare(oracle, gcr, pr, params(use_sprt=1), seed)


def test_space_partitioning_with_magsac(oracle, gcr):
    pr = S.homography_pair(20, n=1500)
    compare(oracle, gcr, pr, params(scoring=_abi.GCR_SCORING_MAGSAC), 1)


def test_space_partitioning_low_inlier_ratio(oracle, gcr):
    pr = S.homography_pair(21, n=3000, inlier_ratio=0.15)
    compare(oracle, gcr, pr, params(), 2)


def test_drop_in_defaults(oracle, gcr):
    # the Python defaults: PROSAC, SPRT and space partitioning on
    pr = S.homography_pair(22, n=2000)
    H, mask = gcr.findHomography(pr["corr"], 480, 640, 480, 640, threshold=3.0, seed=4)
    assert H is not None and S.homography_error(H, pr["H_gt"]) < 3.0
