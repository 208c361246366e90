"""GPU parity of SPRT preemptive verification (preemption_sprt.h) for the
three model kinds: the device walks the same point order with the same
cursor, thresholds and history updates as the oracle, so masks, run
statistics and models must agree."""
import numpy as np
import pytest

from pygcransac import _abi, synthetic as S

pytestmark = pytest.mark.gpu

MODEL_TOL = 1e-6


def rel_err(a, b):
    a = a / np.linalg.norm(a)
    b = b / np.linalg.norm(b)
    return min(np.linalg.norm(a - b), np.linalg.norm(a + b))


def params(threshold, lam, grid, ratio, **kw):
    p = _abi.Params(threshold=threshold, confidence=0.99, spatial_coherence_weight=lam, neighborhood_size=grid,
                    max_iterations=2000, min_iterations=50, sampler=0, neighborhood=0, lo_number=50, seed=0,
                    use_sprt=1, min_inlier_ratio_for_sprt=ratio)
    for k, v in kw.items():
        setattr(p, k, v)
    return p


def compare(oracle, gcr, kind, pr, p, seed, K=None):
    rc_o, M_o, m_o, st_o = oracle.find(kind, pr["corr"], oracle.make_size(*pr["size"]), p, seed=seed,
                                       K1=K, K2=K)
    Kb = None if K is None else np.concatenate([K.ravel(), K.ravel()])[None, :]
    models, masks, stats = gcr.find_batch(kind, [pr["corr"]], [pr["size"]], p, seeds=[seed], K=Kb)
    assert stats["status"][0] == rc_o
    assert np.array_equal(masks[0], m_o), f"mask differs at {np.nonzero(masks[0] != m_o)[0][:10]}"
    if rc_o == 0:
        assert rel_err(models[0], M_o) < MODEL_TOL
    assert stats["iteration_number"][0] == st_o.iteration_number
    assert stats["graph_cut_number"][0] == st_o.graph_cut_number
    assert stats["models_scored"][0] == st_o.models_scored


@pytest.mark.parametrize("seed", range(3))
def test_sprt_homography(oracle, gcr, seed):
    pr = S.homography_pair(seed, n=2000)
    compare(oracle, gcr, _abi.GCR_HOMOGRAPHY, pr, params(3.0, 0.975, 4, 1e-5), seed)


@pytest.mark.parametrize("seed", range(3))
def test_sprt_fundamental(oracle, gcr, seed):
    pr = S.two_view_pair(seed, n=1500, inlier_ratio=0.4)
    compare(oracle, gcr, _abi.GCR_FUNDAMENTAL, pr, params(0.75, 0.975, 8, 1e-5), seed)


@pytest.mark.parametrize("seed", range(3))
def test_sprt_essential(oracle, gcr, seed):
    pr = S.two_view_pair(60 + seed, n=1500, inlier_ratio=0.4)
    compare(oracle, gcr, _abi.GCR_ESSENTIAL, pr, params(0.75, 0.1, 8, 0.01), seed, K=pr["K"])


def test_sprt_with_magsac(oracle, gcr):
    pr = S.homography_pair(7, n=1500)
    compare(oracle, gcr, _abi.GCR_HOMOGRAPHY, pr, params(3.0, 0.975, 4, 1e-5, scoring=_abi.GCR_SCORING_MAGSAC), 2)


def test_drop_in_defaults_use_sprt(gcr):
    pr = S.homography_pair(8, n=2000)
    H, mask = gcr.findHomography(pr["corr"], 480, 640, 480, 640, threshold=3.0, sampler=0, seed=3)
    assert H is not None
    assert S.homography_error(H, pr["H_gt"]) < 3.0
