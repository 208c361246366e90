"""GPU parity of the fundamental-matrix path (7-point minimal solver, Sampson
scoring, symmetric-epipolar validity, DEGENSAC degeneracy test, 8-point + LM
non-minimal fits, graph-cut LO, IRLS and the driver's final bundle
adjustment) against the oracle on the same seeded inputs."""
import numpy as np
import pytest

from pygcransac import _abi, synthetic as S

pytestmark = pytest.mark.gpu

MODEL_TOL = 1e-6


def f_params(**kw):
    p = _abi.Params(threshold=0.75, confidence=0.99, spatial_coherence_weight=0.975, neighborhood_size=8,
                    max_iterations=3000, min_iterations=50, sampler=0, neighborhood=0, lo_number=50, seed=0)
    for k, v in kw.items():
        setattr(p, k, v)
    return p


def rel_err(a, b):
    a = a / np.linalg.norm(a)
    b = b / np.linalg.norm(b)
    return min(np.linalg.norm(a - b), np.linalg.norm(a + b))


def compare(oracle, gcr, pr, p, seed):
    rc_o, F_o, m_o, st_o = oracle.find(_abi.GCR_FUNDAMENTAL, pr["corr"], oracle.make_size(*pr["size"]), p,
                                       seed=seed)
    models, masks, stats = gcr.find_batch(_abi.GCR_FUNDAMENTAL, [pr["corr"]], [pr["size"]], p, seeds=[seed])
    assert (stats["flags"][0] & 8) == (st_o.flags & 8), "DEGENSAC inner runs differ"
    assert stats["status"][0] == rc_o
    assert np.array_equal(masks[0], m_o), f"mask differs at {np.nonzero(masks[0] != m_o)[0][:10]}"
    if rc_o == 0:
        assert rel_err(models[0], F_o) < MODEL_TOL
    assert stats["iteration_number"][0] == st_o.iteration_number
    assert stats["graph_cut_number"][0] == st_o.graph_cut_number
    assert stats["models_scored"][0] == st_o.models_scored


@pytest.mark.parametrize("seed", range(6))
def test_fundamental_pairs(oracle, gcr, seed):
    pr = S.two_view_pair(seed, n=1000, inlier_ratio=0.5)
    compare(oracle, gcr, pr, f_params(), seed)


def test_fundamental_no_spatial_term(oracle, gcr):
    pr = S.two_view_pair(11, n=800, inlier_ratio=0.6)
    compare(oracle, gcr, pr, f_params(spatial_coherence_weight=0.0), 2)


def test_fundamental_prosac(oracle, gcr):
    pr = S.two_view_pair(12, n=800, inlier_ratio=0.6)
    compare(oracle, gcr, pr, f_params(sampler=1), 3)


def test_fundamental_config_size(oracle, gcr):
    pr = S.two_view_pair(13, n=5000, inlier_ratio=0.25)
    compare(oracle, gcr, pr, f_params(max_iterations=2000), 5)


def test_fundamental_drop_in_defaults(gcr):
    pr = S.two_view_pair(14, n=1200, inlier_ratio=0.6)
    F, mask = gcr.findFundamentalMatrix(pr["corr"], 480, 640, 480, 640, threshold=0.75, seed=1)
    assert F is not None
    assert S.fundamental_error(F, pr) < 0.5


@pytest.mark.parametrize("seed", range(3))
def test_fundamental_pnapsac(oracle, gcr, seed):
    pr = S.two_view_pair(20 + seed, n=1500, inlier_ratio=0.4)
    compare(oracle, gcr, pr, f_params(sampler=2), seed)
