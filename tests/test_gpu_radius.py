"""GPU parity of the radius neighbourhood (neighborhood = 1, the reference's
FlannNeighborhoodGraph, restated with an exact ball search): the device builds
the same edges as the oracle, labels with a push-relabel maximum flow on the
sparse graph, and returns the oracle's masks, counts and models. Includes the
essential-matrix entry point called with the reference's default arguments
(radius graph of 20 px with spatial weight 0.1)."""
import numpy as np
import pytest

from pygcransac import _abi, synthetic as S

pytestmark = pytest.mark.gpu

MODEL_TOL = 1e-6


def rel_err(a, b):
    a = a / np.linalg.norm(a)
    b = b / np.linalg.norm(b)
    return min(np.linalg.norm(a - b), np.linalg.norm(a + b))


def compare(oracle, gcr, kind, pr, p, K=None):
    rc, M, mask, st = oracle.find(kind, pr["corr"], oracle.make_size(*pr["size"]), p, seed=p.seed, K1=K, K2=K)
    Kb = None if K is None else np.concatenate([K.ravel(), K.ravel()])[None, :]
    models, masks, stats = gcr.find_batch(kind, [pr["corr"]], [pr["size"]], p, seeds=[p.seed], K=Kb)
    assert stats["status"][0] == rc
    assert np.array_equal(masks[0], mask), f"mask differs at {np.nonzero(masks[0] != mask)[0][:10]}"
    assert (stats["iteration_number"][0], stats["graph_cut_number"][0], stats["local_optimization_number"][0]) == \
        (st.iteration_number, st.graph_cut_number, st.local_optimization_number)
    if rc == 0:
        assert rel_err(models[0], M) < MODEL_TOL


@pytest.mark.parametrize("seed", [0, 1])
def test_radius_graph_homography(oracle, gcr, seed):
    pr = S.homography_pair(500 + seed, n=1200, inlier_ratio=0.4)
    p = gcr.default_params(_abi.GCR_HOMOGRAPHY)
    p.threshold, p.use_sprt, p.use_space_partitioning, p.sampler = 3.0, 0, 0, 0
    p.neighborhood, p.neighborhood_size, p.max_iterations, p.seed = 1, 20.0, 2000, seed
    compare(oracle, gcr, _abi.GCR_HOMOGRAPHY, pr, p)


@pytest.mark.parametrize("seed", [0, 1])
def test_radius_graph_fundamental(oracle, gcr, seed):
    pr = S.two_view_pair(510 + seed, n=1500, inlier_ratio=0.35)
    p = gcr.default_params(_abi.GCR_FUNDAMENTAL)
    p.threshold, p.use_sprt, p.sampler, p.spatial_coherence_weight = 0.75, 0, 0, 0.975
    p.max_iterations, p.seed = 2000, seed
    compare(oracle, gcr, _abi.GCR_FUNDAMENTAL, pr, p)


@pytest.mark.parametrize("seed", [0, 1])
def test_radius_graph_essential_defaults(oracle, gcr, seed):
    """findEssentialMatrix with the reference's defaults: PROSAC, SPRT, radius
    graph (20 px), spatial weight 0.1."""
    pr = S.two_view_pair(520 + seed, n=1000, inlier_ratio=0.4)
    K = pr["K"]
    h1, w1, h2, w2 = pr["size"]
    E, mask, st = gcr.findEssentialMatrix(pr["corr"], K, K, h1, w1, h2, w2, None, threshold=0.75, seed=seed,
                                         return_stats=True)
    p = gcr.default_params(_abi.GCR_ESSENTIAL)
    p.threshold, p.seed = 0.75, seed
    rc, M, mref, sref = oracle.find(_abi.GCR_ESSENTIAL, pr["corr"], oracle.make_size(*pr["size"]), p, seed=seed,
                                    K1=K, K2=K)
    assert np.array_equal(mask, mref)
    assert (st.iteration_number, st.graph_cut_number) == (sref.iteration_number, sref.graph_cut_number)
    assert st.graph_cut_number > 0  # the labelling on the radius graph ran
    if rc == 0:
        assert rel_err(E, M) < MODEL_TOL
        assert S.essential_error(E, pr) < 2.0
