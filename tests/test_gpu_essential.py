"""GPU parity of the essential-matrix path (K^-1 normalisation, Nister
five-point minimal solver with Sturm root isolation, Sampson scoring,
symmetric-epipolar validity, Stewenius non-minimal fits returning several
models in the graph-cut LO and IRLS, and the driver's pose-decomposition bundle
adjustment) against the oracle on the same seeded inputs."""
import numpy as np
import pytest

from pygcransac import _abi, synthetic as S

pytestmark = pytest.mark.gpu

MODEL_TOL = 1e-6


def e_params(**kw):
    p = _abi.Params(threshold=0.75, confidence=0.99, spatial_coherence_weight=0.1, neighborhood_size=8,
                    max_iterations=2000, min_iterations=50, sampler=0, neighborhood=0, lo_number=50, seed=0)
    for k, v in kw.items():
        setattr(p, k, v)
    return p


def rel_err(a, b):
    a = a / np.linalg.norm(a)
    b = b / np.linalg.norm(b)
    return min(np.linalg.norm(a - b), np.linalg.norm(a + b))


def compare(oracle, gcr, pr, p, seed):
    K = pr["K"]
    rc_o, E_o, m_o, st_o = oracle.find(_abi.GCR_ESSENTIAL, pr["corr"], oracle.make_size(*pr["size"]), p,
                                       seed=seed, K1=K, K2=K)
    Kb = np.concatenate([K.ravel(), K.ravel()])[None, :]
    models, masks, stats = gcr.find_batch(_abi.GCR_ESSENTIAL, [pr["corr"]], [pr["size"]], p, seeds=[seed], K=Kb)
    assert stats["status"][0] == rc_o
    assert np.array_equal(masks[0], m_o), f"mask differs at {np.nonzero(masks[0] != m_o)[0][:10]}"
    if rc_o == 0:
        assert rel_err(models[0], E_o) < MODEL_TOL
    assert stats["iteration_number"][0] == st_o.iteration_number
    assert stats["graph_cut_number"][0] == st_o.graph_cut_number
    assert stats["models_scored"][0] == st_o.models_scored
    return models[0], masks[0]


@pytest.mark.parametrize("seed", range(4))
def test_essential_pairs(oracle, gcr, seed):
    pr = S.two_view_pair(seed, n=1000, inlier_ratio=0.5)
    compare(oracle, gcr, pr, e_params(), seed)


def test_essential_low_inlier_ratio(oracle, gcr):
    pr = S.two_view_pair(31, n=2000, inlier_ratio=0.2)
    compare(oracle, gcr, pr, e_params(), 4)


def test_essential_no_spatial_term(oracle, gcr):
    pr = S.two_view_pair(32, n=800, inlier_ratio=0.6)
    compare(oracle, gcr, pr, e_params(spatial_coherence_weight=0.0), 2)


def test_essential_prosac(oracle, gcr):
    pr = S.two_view_pair(33, n=800, inlier_ratio=0.6)
    compare(oracle, gcr, pr, e_params(sampler=1), 3)


def test_essential_pnapsac(oracle, gcr):
    pr = S.two_view_pair(34, n=1500, inlier_ratio=0.4)
    compare(oracle, gcr, pr, e_params(sampler=2), 1)


@pytest.mark.parametrize("n", [5, 6, 40])
def test_essential_tiny_inputs(oracle, gcr, n):
    pr = S.two_view_pair(40 + n, n=n, inlier_ratio=1.0)
    compare(oracle, gcr, pr, e_params(), 0)


def test_essential_drop_in(gcr):
    pr = S.two_view_pair(35, n=1500, inlier_ratio=0.5)
    E, mask = gcr.findEssentialMatrix(pr["corr"], pr["K"], pr["K"], 480, 640, 480, 640, threshold=0.75, seed=1,
                                      sampler=0, neighborhood=0, neighborhood_size=8)
    assert E is not None
    assert S.essential_error(E, pr) < 2.0
