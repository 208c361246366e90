"""CPU checks of the planar-motion essential matrix
(findPlanarEssentialMatrix_, src/pygcransac/src/gcransac_python.cpp:
3531-3870): the entry points' argument checks before any device work, and
the oracle's restatement of the two-point planar solver
(solver_essential_matrix_two_points_planar.h:92-175) and of the run with the
bundle-adjustment non-minimal solver."""
import ctypes

import numpy as np
import pytest

from pygcransac import _abi, synthetic as S


def planar_params(**kw):
    base = dict(threshold=0.75, confidence=0.99, spatial_coherence_weight=0.975, neighborhood_size=8,
                max_iterations=200, min_iterations=50, sampler=0, neighborhood=0, lo_number=20)
    base.update(kw)
    return _abi.Params(**base)


def normalised(pr):
    Ki = np.linalg.inv(pr["K"])
    c = pr["corr"]
    x1 = np.c_[c[:, :2], np.ones(len(c))] @ Ki.T
    x2 = np.c_[c[:, 2:], np.ones(len(c))] @ Ki.T
    return np.ascontiguousarray(np.c_[x1[:, :2], x2[:, :2]])


def test_planar_entry_checks(gcr):
    """MAGSAC++ (which the planar driver does not offer) is refused, and so
    are missing intrinsics, before any device work; the python entry wants
    rows of 4 and at least 3 of them, like the reference binding; its
    defaults are the binding's."""
    lib = _abi.load()
    pr = S.two_view_pair(1, n=50, inlier_ratio=0.5, planar_motion=True)
    c = np.ascontiguousarray(pr["corr"])
    K = np.ascontiguousarray(pr["K"]).ravel()
    size = _abi.ImageSize(h1=480, w1=640, h2=480, w2=640)
    model, mask, st = np.zeros(9), np.zeros(50, np.uint8), _abi.Stats()
    p = planar_params(scoring=1)
    rc = lib.gcr_find_essential_planar(_abi.ptr(c), 50, _abi.ptr(K), _abi.ptr(K), ctypes.byref(size), None,
                                       ctypes.byref(p), _abi.ptr(model), _abi.ptr(mask), ctypes.byref(st))
    assert rc == _abi.GCR_UNSUPPORTED
    p = planar_params()
    rc = lib.gcr_find_essential_planar(_abi.ptr(c), 50, None, _abi.ptr(K), ctypes.byref(size), None,
                                       ctypes.byref(p), _abi.ptr(model), _abi.ptr(mask), ctypes.byref(st))
    assert rc == _abi.GCR_INVALID_ARG
    with pytest.raises(ValueError):
        gcr.findPlanarEssentialMatrix(c[:2], pr["K"], pr["K"], 480, 640, 480, 640)
    with pytest.raises(ValueError):
        gcr.findPlanarEssentialMatrix(np.c_[c, c], pr["K"], pr["K"], 480, 640, 480, 640)
    d = gcr.default_params(_abi.GCR_ESSENTIAL_PLANAR)
    assert (d.spatial_coherence_weight, d.neighborhood, d.neighborhood_size, d.sampler, d.use_sprt) == \
        (0.975, 1, 20.0, 1, 1)


def test_oracle_planar_solver_recovers_the_motion(oracle):
    """On exact correspondences of a planar motion the restated two-point
    solver returns the true essential matrix (up to sign and scale) among its
    models for every sample of 100 scenes, and every model has the planar
    structure (zeros at E11, E13, E22, E31, E33)."""
    lib = oracle.load()
    for seed in range(100):
        pr = S.two_view_pair(seed, n=60, inlier_ratio=1.0, sigma=0.0, planar_motion=True)
        nrm = normalised(pr)
        E = pr["E_gt"] / np.linalg.norm(pr["E_gt"])
        s = np.random.default_rng(seed).choice(60, 2, replace=False).astype(np.int64)
        out = np.zeros(90)
        k = lib.oracle_minimal(_abi.GCR_ESSENTIAL_PLANAR, oracle._p(nrm), 60, oracle._p(s), oracle._p(out))
        assert 1 <= k <= 4
        Ms = [out[9 * i:9 * i + 9].reshape(3, 3) for i in range(k)]
        for M in Ms:
            assert np.abs(M.ravel()[[0, 2, 4, 6, 8]]).max() == 0.0
        err = min(np.abs(M / np.linalg.norm(M) - sg * E).max() for M in Ms for sg in (1, -1))
        assert err < 1e-6, (seed, err)


@pytest.mark.parametrize("use_sprt", [0, 1])
def test_oracle_planar_run_recovers_the_scene(oracle, use_sprt):
    """The oracle's planar driver (bundle-adjustment non-minimal fits; with
    SPRT up to 100 graph cuts and no final reweighted fit) recovers a noisy
    planar-motion scene."""
    pr = S.two_view_pair(21, n=800, inlier_ratio=0.5, planar_motion=True)
    K = pr["K"]
    rc, E, m, st = oracle.find(_abi.GCR_ESSENTIAL_PLANAR, pr["corr"], oracle.make_size(*pr["size"]),
                               planar_params(use_sprt=use_sprt), seed=3, K1=K, K2=K)
    assert rc == 0
    assert S.essential_error(E, pr) < 1.0  # degrees
    assert m[pr["inlier_gt"]].mean() > 0.95


def test_oracle_planar_solver_degenerate_samples(oracle):
    """Degenerate two-point samples (a repeated point, points on the image
    row through the principal point, which zero the A2 rows) give no model
    or only finite ones: models with non-finite entries are dropped."""
    lib = oracle.load()
    pts = np.array([[0.1, 0.2, 0.15, 0.25], [0.1, 0.2, 0.15, 0.25],
                    [0.1, 0.0, 0.15, 0.0], [-0.2, 0.0, -0.1, 0.0]], np.float64)
    for s in ([0, 1], [2, 3]):
        out = np.full(90, np.nan)
        k = lib.oracle_minimal(_abi.GCR_ESSENTIAL_PLANAR, oracle._p(pts), 4, oracle._p(np.array(s, np.int64)),
                               oracle._p(out))
        assert 0 <= k <= 4
        assert np.all(np.isfinite(out[:9 * k]))


def _orientation_ok(E, pts):
    """isOrientationValid (essential_estimator.h:336-401) on the rows pts."""
    e = np.cross(E[0], E[2])
    if np.all(np.abs(e) <= 1.9984e-15):
        e = np.cross(E[1], E[2])
    sg = [(E[0, 0] * p[2] + E[1, 0] * p[3] + E[2, 0]) * (e[1] - e[2] * p[1]) for p in pts]
    return all(not (sg[0] * v < 0) for v in sg[1:])


def test_oracle_planar_solver_matches_a_numpy_restatement(oracle):
    """On noisy planar-motion samples the oracle's models equal a NumPy
    transliteration of the reference's steps (pseudo-inverse of A2, the
    quadratic in cos 2a, the four angles, atan2 of the mapped direction,
    solver_essential_matrix_two_points_planar.h:115-173) after the
    orientation test, in the same order."""
    lib = oracle.load()
    for seed in range(60):
        pr = S.two_view_pair(400 + seed, n=30, inlier_ratio=1.0, sigma=1.0, planar_motion=True)
        nrm = normalised(pr)
        s = np.random.default_rng(seed).choice(30, 2, replace=False)
        p = nrm[s]
        A1 = np.array([[q[1], -q[1] * q[2]] for q in p])
        A2 = np.array([[-q[3], q[0] * q[3]] for q in p])
        C = -np.linalg.inv(A2.T @ A2) @ A2.T @ A1
        C2 = C.T @ C
        a, b, c = C2[0, 0], C2[1, 0], C2[1, 1]
        cf1, cf2, cf3 = 4 * b * b + (a - c) ** 2, -2 * (a - c) * (2 - a - c), (2 - a - c) ** 2 - 4 * b * b
        with np.errstate(invalid="ignore"):
            d = np.sqrt(cf2 * cf2 - 4 * cf1 * cf3)
            r1, r2 = (-cf2 + d) / (2 * cf1), (-cf2 - d) / (2 * cf1)
            alphas = [np.arccos(r1) / 2, np.arccos(r2) / 2, -np.arccos(r1) / 2, -np.arccos(r2) / 2]
        ref = []
        for al in alphas:
            v1 = np.array([np.cos(al), np.sin(al)])
            v2 = C @ v1
            v2 = v2 / np.linalg.norm(v2)
            a1, amb = np.arctan2(v1[1], v1[0]), np.arctan2(v2[1], v2[0])
            E = np.array([[0, -np.sin(a1), 0], [np.sin(amb), 0, -np.cos(amb)], [0, np.cos(a1), 0]])
            if np.all(np.isfinite(E)) and _orientation_ok(E, p):
                ref.append(E.ravel())
        out = np.zeros(90)
        k = lib.oracle_minimal(_abi.GCR_ESSENTIAL_PLANAR, oracle._p(nrm), 30, oracle._p(s.astype(np.int64)),
                               oracle._p(out))
        assert k == len(ref), (seed, k, len(ref))
        for i in range(k):
            assert np.abs(out[9 * i:9 * i + 9] - ref[i]).max() < 1e-9, (seed, i)
