"""CPU checks of the affine-correspondence homography (findHomographyAC_,
src/pygcransac/src/gcransac_python.cpp:4553-4811): the entry points' argument
checks run before any device work, and the oracle's restatement of the
minimal solver (solver_homography_two_affine.h:88-237) on its own terms."""
import ctypes

import numpy as np
import pytest

from pygcransac import _abi, synthetic as S


def ac_params(**kw):
    base = dict(threshold=3.0, confidence=0.99, spatial_coherence_weight=0.975, neighborhood_size=4,
                max_iterations=100, min_iterations=50, sampler=0, neighborhood=0, lo_number=50)
    base.update(kw)
    return _abi.Params(**base)


def test_affine_entry_checks_before_device_work(gcr):
    """P-NAPSAC (which the reference's driver refuses) and MAGSAC++ (which it
    does not offer) are refused; the python entry wants rows of 8 for
    solver=2 and at least 4 of them, like the reference binding."""
    lib = _abi.load()
    c = np.random.default_rng(1).uniform(0, 480, (50, 8))
    size = _abi.ImageSize(h1=480, w1=640, h2=480, w2=640)
    model, mask, st = np.zeros(9), np.zeros(50, np.uint8), _abi.Stats()
    for kw, want in ((dict(sampler=2), _abi.GCR_UNSUPPORTED), (dict(scoring=1), _abi.GCR_UNSUPPORTED),
                     (dict(threshold=0.0), _abi.GCR_INVALID_ARG)):
        p = ac_params(**kw)
        rc = lib.gcr_find_homography_affine(_abi.ptr(c), 50, ctypes.byref(size), None, ctypes.byref(p),
                                            _abi.ptr(model), _abi.ptr(mask), ctypes.byref(st))
        assert rc == want, (kw, rc)
    with pytest.raises(ValueError):
        gcr.findHomography(c[:, :4], 480, 640, 480, 640, solver=2)
    with pytest.raises(ValueError):
        gcr.findHomography(c[:3], 480, 640, 480, 640, solver=2)
    with pytest.raises(NotImplementedError):
        gcr.findHomography(c, 480, 640, 480, 640, solver=2, sampler=2)
    p = gcr.default_params(_abi.GCR_HOMOGRAPHY_AFFINE)
    assert (p.spatial_coherence_weight, p.neighborhood, p.neighborhood_size, p.use_space_partitioning) == \
        (0.975, 0, 4.0, 0)


def _minimal_rows(a, b):
    """The reference's minimal system: the point rows of both correspondences
    and the four affine rows of the first."""
    def pt(p):
        x1, y1, x2, y2 = p[:4]
        return [[-x1, -y1, -1, 0, 0, 0, x2 * x1, x2 * y1, x2], [0, 0, 0, -x1, -y1, -1, y2 * x1, y2 * y1, y2]]
    x1, y1, x2, y2, a11, a12, a21, a22 = a
    af = [[-1, 0, 0, 0, 0, 0, x2 + a11 * x1, a11 * y1, a11], [0, -1, 0, 0, 0, 0, a12 * x1, x2 + a12 * y1, a12],
          [0, 0, 0, -1, 0, 0, y2 + a21 * x1, a21 * y1, a21], [0, 0, 0, 0, -1, 0, a22 * x1, y2 + a22 * y1, a22]]
    return np.array(pt(a) + af + pt(b), np.float64)


def test_reference_minimal_system_is_rank_deficient():
    """The reference's minimal case (one affine and one point correspondence)
    gives only seven independent linear constraints on a homography: every
    homography that agrees with the first correspondence's point and local
    affine map moves the second point along the line through the first one,
    so its two point rows add one constraint. On exact data the 8 x 9 system
    has a two-dimensional null space holding the true homography, and the
    reference's SVD returns an arbitrary vector of it; on noisy data the
    system is regular and its null vector follows the noise. The restatement
    reproduces this behaviour (the same system, solved with h33 = 1)."""
    pr = S.homography_affine_pair(5, n=400, inlier_ratio=0.5, sigma=0.0, affine_sigma=0.0)
    c, g = pr["corr"], pr["inlier_gt"]
    H = pr["H_gt"] / pr["H_gt"][2, 2]
    for k in range(0, 20, 2):
        A = _minimal_rows(c[g][k], c[g][k + 1])
        sv = np.linalg.svd(A, compute_uv=False)
        assert sv[-1] / sv[0] < 1e-12  # rank 7
        assert np.abs(A @ H.ravel()).max() < 1e-9 * np.abs(A).max()
    # with both affine maps (two full correspondences) the system has rank 8
    af_b = _minimal_rows(c[g][1], c[g][0])[2:6]
    A12 = np.r_[_minimal_rows(c[g][0], c[g][1]), af_b]
    sv = np.linalg.svd(A12, compute_uv=False)
    assert sv[-2] / sv[0] > 1e-12


def test_oracle_affine_run_matches_its_minimal_solver(oracle):
    """A tape of one sample per call drives the oracle; a sample whose model
    the restated solver returns is scored (models_scored counts it), one the
    oriented-sample test rejects is not, and the run reports no model on
    noisy data, where the minimal models follow the noise."""
    pr = S.homography_affine_pair(11, n=600, inlier_ratio=0.5)
    inl = np.nonzero(pr["inlier_gt"])[0]
    tape = np.stack([inl[2 * k:2 * k + 2] for k in range(40)]).astype(np.int32)
    p = ac_params(max_iterations=40, min_iterations=40, use_sprt=0, lo_number=10)
    rc, H, m, st = oracle.find(_abi.GCR_HOMOGRAPHY_AFFINE, pr["corr"], oracle.make_size(*pr["size"]), p, seed=1,
                               sample_tape=tape)
    assert st.iteration_number >= 40
    assert 0 < st.models_scored <= 40
    assert rc in (0, 3)
