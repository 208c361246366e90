"""GPU parity of the planar-motion essential matrix
(findPlanarEssentialMatrix_, src/pygcransac/src/gcransac_python.cpp:
3531-3870; python findPlanarEssentialMatrix): the two-point planar minimal
solver, the bundle-adjustment non-minimal solver in the graph-cut LO (one
trial per thread), the CTA-wide reweighted fits (whose pose
refinement reads the point-indexed weights by row position, as the
reference's does), the SPRT branch's settings (100 graph cuts, no final
reweighted fit) and the driver's epilogue, against the oracle on the same
seeded inputs. Statuses, iteration and graph-cut counts and masks are
compared by batch_parity; models to 1e-6 where the masks agree."""
import numpy as np
import pytest

from pygcransac import _abi, synthetic as S

pytestmark = pytest.mark.gpu

MODEL_TOL = 1e-6


def planar_params(**kw):
    p = _abi.Params(threshold=0.75, confidence=0.99, spatial_coherence_weight=0.975, neighborhood_size=8,
                    max_iterations=2000, min_iterations=50, sampler=0, neighborhood=0, lo_number=50, seed=0,
                    min_inlier_ratio_for_sprt=1e-5)
    for k, v in kw.items():
        setattr(p, k, v)
    return p


def rel_err(a, b):
    a = a / np.linalg.norm(a)
    b = b / np.linalg.norm(b)
    return min(np.linalg.norm(a - b), np.linalg.norm(a + b))


def compare(oracle, batch_parity, gcr, pairs, p, seeds):
    kind = _abi.GCR_ESSENTIAL_PLANAR
    corr = np.concatenate([pr["corr"] for pr in pairs])
    offsets = np.zeros(len(pairs) + 1, np.int64)
    offsets[1:] = np.cumsum([len(pr["corr"]) for pr in pairs])
    sizes = np.array([pr["size"] for pr in pairs])
    K = np.stack([np.concatenate([pr["K"].ravel(), pr["K"].ravel()]) for pr in pairs])
    models, masks, stats = gcr.find_batch(kind, (corr, offsets), sizes, p, seeds=seeds, K=K)
    batch_parity(kind, corr, offsets, sizes, p, np.asarray(seeds, np.uint64), K, stats, np.concatenate(masks))
    for i, pr in enumerate(pairs):
        rc_o, E_o, m_o, st_o = oracle.find(kind, pr["corr"], oracle.make_size(*pr["size"]), p, seed=seeds[i],
                                           K1=pr["K"], K2=pr["K"])
        if np.array_equal(masks[i], m_o) and rc_o == 0:
            assert rel_err(models[i], E_o) < MODEL_TOL, i
    return models, masks, stats


@pytest.mark.parametrize("sampler,use_sprt", [(0, 0), (1, 0), (0, 1)])
def test_planar_batch(oracle, batch_parity, gcr, sampler, use_sprt):
    """Batches of planar-motion pairs (60-3000 correspondences, 20-70 %
    inliers): statuses, counts, masks and models equal the oracle's; the runs
    find the true motion."""
    pairs = [S.two_view_pair(200 + i, n=n, inlier_ratio=r, planar_motion=True)
             for i, (n, r) in enumerate([(600, 0.5), (1500, 0.3), (3000, 0.2), (60, 0.7), (1000, 0.4)])]
    models, masks, stats = compare(oracle, batch_parity, gcr, pairs, planar_params(sampler=sampler, use_sprt=use_sprt),
                                   seeds=[3, 4, 5, 6, 7])
    assert np.all(stats["status"] == 0)
    errs = [S.essential_error(models[i], pr) for i, pr in enumerate(pairs)]
    assert np.median(errs) < 1.0, errs


def test_planar_radius_graph_and_no_spatial_term(oracle, batch_parity, gcr):
    """The binding's default neighbourhood (the radius graph, radius 20 px)
    and a run without the spatial term."""
    pairs = [S.two_view_pair(210 + i, n=800, inlier_ratio=0.5, planar_motion=True) for i in range(2)]
    compare(oracle, batch_parity, gcr, pairs, planar_params(neighborhood=1, neighborhood_size=20.0), seeds=[1, 2])
    compare(oracle, batch_parity, gcr, pairs, planar_params(spatial_coherence_weight=0.0), seeds=[3, 4])


def test_planar_python_entry(oracle, gcr):
    """findPlanarEssentialMatrix equals the oracle's driver run and needs far
    fewer iterations than the five-point estimator on the same points."""
    pr = S.two_view_pair(220, n=1500, inlier_ratio=0.3, planar_motion=True)
    K = pr["K"]
    kw = dict(threshold=0.75, sampler=0, use_sprt=False, neighborhood=0, neighborhood_size=8, seed=5)
    E, mask, st = gcr.findPlanarEssentialMatrix(pr["corr"], K, K, 480, 640, 480, 640, return_stats=True, **kw)
    rc_o, E_o, m_o, st_o = oracle.find(_abi.GCR_ESSENTIAL_PLANAR, pr["corr"], oracle.make_size(*pr["size"]),
                                       planar_params(use_sprt=0, seed=5), seed=5, K1=K, K2=K)
    assert rc_o == 0
    if np.array_equal(mask, m_o):
        assert rel_err(E, E_o) < MODEL_TOL
    assert S.essential_error(E, pr) < 1.0
    E5, mask5, st5 = gcr.findEssentialMatrix(pr["corr"], K, K, 480, 640, 480, 640, return_stats=True,
                                             spatial_coherence_weight=0.975, **kw)
    assert st.iteration_number < st5.iteration_number
