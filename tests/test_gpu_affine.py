"""GPU parity of the kinds with rows of eight values through the C-ABI: the
homographies of findHomographyAC_ and findHomographySIFT_ and the fundamental
matrices of findFundamentalMatrixAC_ and findFundamentalMatrixSIFT_
(src/pygcransac/src/gcransac_python.cpp:4553-4811, 4813-5069, 1924-2221,
2222-2518; python findHomography / findFundamentalMatrix with solver = 2 and
with solver = 1), the device engine against the oracle
on the same seeded inputs of rows (x1, y1, x2, y2, a11, a12, a21, a22) or
(x1, y1, x2, y2, q1, q2, o1, o2). Statuses, iteration, graph-cut and
models-scored counts and masks must be identical, models equal to 1e-6
relative Frobenius error after normalisation."""
import numpy as np
import pytest

from pygcransac import _abi, synthetic as S

pytestmark = pytest.mark.gpu

MODEL_TOL = 1e-6


def ac_params(**kw):
    p = _abi.Params(threshold=3.0, confidence=0.99, spatial_coherence_weight=0.975, neighborhood_size=4,
                    max_iterations=10000, min_iterations=50, sampler=0, neighborhood=0, lo_number=50, seed=0,
                    min_inlier_ratio_for_sprt=1e-5)
    for k, v in kw.items():
        setattr(p, k, v)
    return p


def rel_model_err(a, b):
    a = a / np.linalg.norm(a)
    b = b / np.linalg.norm(b)
    return min(np.linalg.norm(a - b), np.linalg.norm(a + b))


def compare(oracle, gcr, pairs, p, seeds, tape=None):
    corr = [pr["corr"] for pr in pairs]
    sizes = [pr["size"] for pr in pairs]
    models, masks, stats = gcr.find_batch(_abi.GCR_HOMOGRAPHY_AFFINE, corr, sizes, p, seeds=seeds, sample_tape=tape)
    for i, pr in enumerate(pairs):
        rc_o, H_o, m_o, st_o = oracle.find(_abi.GCR_HOMOGRAPHY_AFFINE, pr["corr"], oracle.make_size(*pr["size"]), p,
                                           seed=seeds[i], sample_tape=None if tape is None else tape[i])
        assert stats["status"][i] == rc_o, (i, stats["status"][i], rc_o)
        assert np.array_equal(masks[i], m_o), f"pair {i}: mask differs at {np.nonzero(masks[i] != m_o)[0][:10]}"
        if rc_o == 0:
            assert rel_model_err(models[i], H_o) < MODEL_TOL
        for f in ("iteration_number", "graph_cut_number", "models_scored", "inlier_number"):
            assert stats[f][i] == getattr(st_o, f), (i, f, stats[f][i], getattr(st_o, f))
    return models, masks, stats


@pytest.mark.parametrize("sampler,use_sprt", [(0, 0), (1, 0), (0, 1)])
def test_affine_homography_batch(oracle, gcr, sampler, use_sprt):
    pairs = [S.homography_affine_pair(40 + i, n=n, inlier_ratio=r)
             for i, (n, r) in enumerate([(600, 0.5), (1500, 0.3), (3000, 0.4), (40, 0.8)])]
    compare(oracle, gcr, pairs, ac_params(sampler=sampler, use_sprt=use_sprt, max_iterations=2000),
            seeds=[3, 4, 5, 6])


def test_affine_homography_tape_of_inlier_samples(oracle, gcr):
    """A tape of all-inlier minimal samples drives device and oracle through
    the same minimal models, local optimisations and final fit."""
    pairs, tapes = [], []
    for i in range(3):
        pr = S.homography_affine_pair(70 + i, n=1200, inlier_ratio=0.35)
        inl = np.nonzero(pr["inlier_gt"])[0]
        rng = np.random.Generator(np.random.PCG64(i))
        tapes.append(np.stack([rng.choice(inl, 2, replace=False) for _ in range(300)]).astype(np.int32))
        pairs.append(pr)
    compare(oracle, gcr, pairs, ac_params(max_iterations=300, min_iterations=300), seeds=[1, 2, 3],
            tape=np.stack(tapes))


def test_affine_homography_python_entry(oracle, gcr):
    """findHomography(..., solver=2) runs the affine kind with the reference
    binding's shapes and returns (model or None, mask) like the oracle."""
    pr = S.homography_affine_pair(90, n=800, inlier_ratio=0.5)
    h, w = pr["size"][:2]
    H, mask = gcr.findHomography(pr["corr"], h, w, h, w, threshold=3.0, sampler=0, use_sprt=False,
                                 max_iters=1000, solver=2, seed=9)
    p = ac_params(max_iterations=1000, use_sprt=0, seed=9)
    rc_o, H_o, m_o, _ = oracle.find(_abi.GCR_HOMOGRAPHY_AFFINE, pr["corr"], oracle.make_size(*pr["size"]), p,
                                    seed=9)
    assert np.array_equal(mask, m_o)
    assert (H is None) == (rc_o != 0 or m_o.sum() == 0)
    if H is not None:
        assert rel_model_err(H, H_o) < MODEL_TOL


# ---- affine-correspondence fundamental matrix (findFundamentalMatrixAC_) ----

def fa_params(**kw):
    p = _abi.Params(threshold=0.75, confidence=0.99, spatial_coherence_weight=0.975, neighborhood_size=8,
                    max_iterations=10000, min_iterations=50, sampler=0, neighborhood=0, lo_number=50, seed=0,
                    min_inlier_ratio_for_sprt=1e-5)
    for k, v in kw.items():
        setattr(p, k, v)
    return p


def compare_f(oracle, batch_parity, gcr, pairs, p, seeds, kind=_abi.GCR_FUNDAMENTAL_AFFINE):
    corr = np.concatenate([pr["corr"] for pr in pairs])
    offsets = np.zeros(len(pairs) + 1, np.int64)
    offsets[1:] = np.cumsum([len(pr["corr"]) for pr in pairs])
    sizes = np.array([pr["size"] for pr in pairs])
    models, masks, stats = gcr.find_batch(kind, (corr, offsets), sizes, p, seeds=seeds)
    flat = np.concatenate(masks)
    batch_parity(kind, corr, offsets, sizes, p, np.asarray(seeds, np.uint64), None, stats, flat)
    for i, pr in enumerate(pairs):
        rc_o, F_o, m_o, st_o = oracle.find(kind, pr["corr"], oracle.make_size(*pr["size"]), p, seed=seeds[i])
        if np.array_equal(masks[i], m_o) and rc_o == 0:
            assert rel_model_err(models[i], F_o) < MODEL_TOL, i
            assert stats["models_scored"][i] == st_o.models_scored, i
    return models, masks, stats


@pytest.mark.parametrize("sampler,use_sprt", [(0, 0), (1, 0), (0, 1)])
def test_affine_fundamental_batch(oracle, batch_parity, gcr, sampler, use_sprt):
    """Batches of affine two-view pairs (200-4000 correspondences, 20-60 %
    inliers): statuses, iteration and graph-cut counts, masks and models equal
    the oracle's; the runs find the ground truth."""
    pairs = [S.two_view_affine_pair(80 + i, n=n, inlier_ratio=r)
             for i, (n, r) in enumerate([(200, 0.6), (1500, 0.3), (4000, 0.2), (900, 0.5), (2500, 0.4)])]
    models, masks, stats = compare_f(oracle, batch_parity, gcr, pairs,
                                     fa_params(sampler=sampler, use_sprt=use_sprt), seeds=[3, 4, 5, 6, 7])
    assert np.all(stats["status"] == 0)
    errs = [S.fundamental_error(models[i], pr) for i, pr in enumerate(pairs)]
    assert np.median(errs) < 1.0, errs


def test_affine_fundamental_large_and_no_spatial_term(oracle, batch_parity, gcr):
    """Pairs above the shared-memory tile (6000-9000 correspondences) and a run
    without the spatial term (no neighbourhood, as the driver builds none)."""
    pairs = [S.two_view_affine_pair(90 + i, n=n, inlier_ratio=0.3) for i, n in enumerate([6000, 9000])]
    compare_f(oracle, batch_parity, gcr, pairs, fa_params(), seeds=[1, 2])
    compare_f(oracle, batch_parity, gcr, pairs[:1], fa_params(spatial_coherence_weight=0.0), seeds=[5])


def test_affine_fundamental_python_entry(oracle, gcr):
    """findFundamentalMatrix(..., solver=2) equals the oracle's driver run and
    needs far fewer iterations than the seven-point form on the same points."""
    pr = S.two_view_affine_pair(95, n=1200, inlier_ratio=0.3)
    h, w = pr["size"][:2]
    kw = dict(threshold=0.75, sampler=0, use_sprt=False, neighborhood=0, neighborhood_size=8,
              spatial_coherence_weight=0.975, seed=4)
    F, mask, st = gcr.findFundamentalMatrix(pr["corr"], h, w, h, w, solver=2, return_stats=True, **kw)
    p = fa_params(seed=4)
    rc_o, F_o, m_o, st_o = oracle.find(_abi.GCR_FUNDAMENTAL_AFFINE, pr["corr"], oracle.make_size(*pr["size"]), p,
                                       seed=4)
    assert rc_o == 0 and np.array_equal(mask, m_o)
    assert rel_model_err(F, F_o) < MODEL_TOL
    F7, mask7, st7 = gcr.findFundamentalMatrix(pr["corr"][:, :4].copy(), h, w, h, w, return_stats=True, **kw)
    assert st.iteration_number < st7.iteration_number


# ---- SIFT-correspondence fundamental matrix (findFundamentalMatrixSIFT_) ----

@pytest.mark.parametrize("sampler,use_sprt", [(0, 0), (1, 0), (0, 1)])
def test_sift_fundamental_batch(oracle, batch_parity, gcr, sampler, use_sprt):
    """Batches of SIFT two-view pairs (scales and orientations): statuses,
    iteration and graph-cut counts, masks and models equal the oracle's; the
    runs find the ground truth."""
    pairs = [S.two_view_sift_pair(60 + i, n=n, inlier_ratio=r)
             for i, (n, r) in enumerate([(300, 0.6), (1500, 0.35), (5000, 0.3), (900, 0.5)])]
    models, masks, stats = compare_f(oracle, batch_parity, gcr, pairs, fa_params(sampler=sampler, use_sprt=use_sprt),
                                     seeds=[2, 3, 4, 5], kind=_abi.GCR_FUNDAMENTAL_SIFT)
    assert np.all(stats["status"] == 0)
    errs = [S.fundamental_error(models[i], pr) for i, pr in enumerate(pairs)]
    assert np.median(errs) < 1.0, errs


def test_sift_fundamental_python_entry(oracle, gcr):
    """findFundamentalMatrix(..., solver=1) equals the oracle's driver run."""
    pr = S.two_view_sift_pair(66, n=1200, inlier_ratio=0.4)
    h, w = pr["size"][:2]
    F, mask = gcr.findFundamentalMatrix(pr["corr"], h, w, h, w, solver=1, threshold=0.75, sampler=0, use_sprt=False,
                                        neighborhood=0, neighborhood_size=8, spatial_coherence_weight=0.975, seed=4)
    rc_o, F_o, m_o, _ = oracle.find(_abi.GCR_FUNDAMENTAL_SIFT, pr["corr"], oracle.make_size(*pr["size"]),
                                    fa_params(seed=4), seed=4)
    assert rc_o == 0 and np.array_equal(mask, m_o)
    assert rel_model_err(F, F_o) < MODEL_TOL


# ---- SIFT-correspondence homography (findHomographySIFT_) ----

def compare_hs(oracle, batch_parity, gcr, pairs, p, seeds, tape=None):
    """Device batch against the oracle pair by pair (batch_parity: statuses,
    iteration and graph-cut counts and masks, rounding-dependent pairs checked
    against the oracle's FMA-contracted build); models where the masks agree.
    The models-scored count may differ by a few: a sample whose two conics
    are nearly tangent has two real intersections in one rounding and none
    (or four) in the other. Such an extra model can start the local
    optimisation from another point, which may end on the same inliers with a
    slightly different least-squares model; models that differ by more than
    1e-6 must then agree to 0.5 px RMS transfer error over the image."""
    kind = _abi.GCR_HOMOGRAPHY_SIFT
    corr = np.concatenate([pr["corr"] for pr in pairs])
    offsets = np.zeros(len(pairs) + 1, np.int64)
    offsets[1:] = np.cumsum([len(pr["corr"]) for pr in pairs])
    sizes = np.array([pr["size"] for pr in pairs])
    models, masks, stats = gcr.find_batch(kind, (corr, offsets), sizes, p, seeds=seeds, sample_tape=tape)
    kw = {} if tape is None else dict(sample_tape=tape)
    batch_parity(kind, corr, offsets, sizes, p, np.asarray(seeds, np.uint64), None, stats, np.concatenate(masks), **kw)
    for i, pr in enumerate(pairs):
        rc_o, H_o, m_o, st_o = oracle.find(kind, pr["corr"], oracle.make_size(*pr["size"]), p, seed=seeds[i],
                                           sample_tape=None if tape is None else tape[i])
        if np.array_equal(masks[i], m_o) and rc_o == 0:
            if rel_model_err(models[i], H_o) >= MODEL_TOL:
                Hd = models[i].reshape(3, 3)
                assert S.homography_error(Hd / Hd[2, 2], H_o / H_o[2, 2]) < 0.5, i
            assert abs(int(stats["models_scored"][i]) - st_o.models_scored) <= max(4, st_o.models_scored // 100), i
    return models, masks, stats


@pytest.mark.parametrize("sampler,use_sprt", [(0, 0), (1, 0), (0, 1)])
def test_sift_homography_batch(oracle, batch_parity, gcr, sampler, use_sprt):
    """Batches of SIFT homography pairs (40-5000 correspondences, 20-80 %
    inliers, one pair above the shared-memory tile): statuses, iteration and
    graph-cut counts, masks and models equal the oracle's; the runs find the
    ground truth."""
    pairs = [S.homography_sift_pair(120 + i, n=n, inlier_ratio=r)
             for i, (n, r) in enumerate([(600, 0.5), (1500, 0.3), (5000, 0.2), (40, 0.8), (3000, 0.4)])]
    models, masks, stats = compare_hs(oracle, batch_parity, gcr, pairs,
                                      ac_params(sampler=sampler, use_sprt=use_sprt, max_iterations=2000),
                                      seeds=[3, 4, 5, 6, 7])
    assert np.all(stats["status"] == 0)
    errs = [S.homography_error(models[i].reshape(3, 3), pr["H_gt"]) for i, pr in enumerate(pairs)]
    assert np.median(errs) < 2.0, errs


def test_sift_homography_tape_and_no_spatial_term(oracle, batch_parity, gcr):
    """A tape of all-inlier minimal samples drives device and oracle through
    the same minimal models (up to four per sample), local optimisations and
    final fit; a run without the spatial term builds no neighbourhood."""
    pairs, tapes = [], []
    for i in range(3):
        pr = S.homography_sift_pair(130 + i, n=1200, inlier_ratio=0.35)
        inl = np.nonzero(pr["inlier_gt"])[0]
        rng = np.random.Generator(np.random.PCG64(i))
        tapes.append(np.stack([rng.choice(inl, 2, replace=False) for _ in range(200)]).astype(np.int32))
        pairs.append(pr)
    compare_hs(oracle, batch_parity, gcr, pairs, ac_params(max_iterations=200, min_iterations=200), seeds=[1, 2, 3],
               tape=np.stack(tapes))
    compare_hs(oracle, batch_parity, gcr, pairs[:2], ac_params(spatial_coherence_weight=0.0), seeds=[4, 5])


def test_sift_homography_python_entry(oracle, gcr):
    """findHomography(..., solver=1) equals the oracle's driver run and needs
    far fewer iterations than the four-point form on the same points."""
    pr = S.homography_sift_pair(140, n=1500, inlier_ratio=0.25)
    h, w = pr["size"][:2]
    kw = dict(threshold=3.0, sampler=0, use_sprt=False, seed=9, use_space_partitioning=False)
    H, mask, st = gcr.findHomography(pr["corr"], h, w, h, w, solver=1, return_stats=True, **kw)
    p = ac_params(use_sprt=0, seed=9)
    rc_o, H_o, m_o, st_o = oracle.find(_abi.GCR_HOMOGRAPHY_SIFT, pr["corr"], oracle.make_size(*pr["size"]), p,
                                       seed=9)
    assert rc_o == 0
    if np.array_equal(mask, m_o):
        assert rel_model_err(H, H_o) < MODEL_TOL
    else:  # a residual at the threshold decided differently by FMA rounding
        assert np.sum(mask != m_o) <= 2
    assert S.homography_error(H, pr["H_gt"]) < 2.0
    H4, mask4, st4 = gcr.findHomography(pr["corr"][:, :4].copy(), h, w, h, w, return_stats=True, **kw)
    assert st.iteration_number < st4.iteration_number
