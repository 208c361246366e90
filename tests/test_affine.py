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


def test_affine_fundamental_entry_checks(gcr):
    """The affine fundamental kind refuses P-NAPSAC and MAGSAC++ (not offered
    by findFundamentalMatrixAC_) before any device work; the python entry wants
    rows of 8 and at least 7 of them, like the reference binding."""
    lib = _abi.load()
    c = np.random.default_rng(3).uniform(0, 480, (50, 8))
    size = _abi.ImageSize(h1=480, w1=640, h2=480, w2=640)
    model, mask, st = np.zeros(9), np.zeros(50, np.uint8), _abi.Stats()
    for kw in (dict(sampler=2), dict(scoring=1)):
        p = ac_params(**kw)
        rc = lib.gcr_find_fundamental_affine(_abi.ptr(c), 50, ctypes.byref(size), None, ctypes.byref(p),
                                             _abi.ptr(model), _abi.ptr(mask), ctypes.byref(st))
        assert rc == _abi.GCR_UNSUPPORTED, kw
    with pytest.raises(ValueError):
        gcr.findFundamentalMatrix(c[:, :4], 480, 640, 480, 640, solver=2)
    with pytest.raises(ValueError):
        gcr.findFundamentalMatrix(c[:6], 480, 640, 480, 640, solver=2)


def test_oracle_three_affine_solver_recovers_the_scene(oracle):
    """On exact affine correspondences of a two-view scene the three-affine
    system (solver_fundamental_matrix_three_affine.h:84-250) has a
    two-dimensional null space holding the true fundamental matrix, and a tape
    of inlier triples drives the oracle's run to it."""
    pr = S.two_view_affine_pair(4, n=600, inlier_ratio=0.5, sigma=0.0, affine_sigma=0.0)
    c, g, F = pr["corr"], pr["inlier_gt"], pr["F_gt"]

    def rows(p):
        x0, y0, x1, y1, a11, a12, a21, a22 = p
        return [[x1 * x0, x1 * y0, x1, y1 * x0, y1 * y0, y1, x0, y0, 1],
                [x1 + a11 * x0, a11 * y0, a11, y1 + a21 * x0, a21 * y0, a21, 1, 0, 0],
                [a12 * x0, x1 + a12 * y0, a12, a22 * x0, y1 + a22 * y0, a22, 0, 1, 0]]
    inl = c[g]
    A = np.array(rows(inl[0]) + rows(inl[1]) + rows(inl[2])[:1])
    sv = np.linalg.svd(A, compute_uv=False)
    assert sv[-1] / sv[0] > 1e-12  # rank 7: a pencil of matrices
    assert np.abs(A @ F.ravel()).max() < 1e-9 * np.abs(A).max()
    idx = np.nonzero(g)[0]
    tape = np.stack([idx[3 * k:3 * k + 3] for k in range(30)]).astype(np.int32)
    p = _abi.Params(threshold=0.75, confidence=0.99, spatial_coherence_weight=0.975, neighborhood_size=8,
                    max_iterations=30, min_iterations=30, sampler=0, neighborhood=0, lo_number=20)
    rc, Fo, m, st = oracle.find(_abi.GCR_FUNDAMENTAL_AFFINE, c, oracle.make_size(*pr["size"]), p, seed=1,
                                sample_tape=tape)
    assert rc == 0
    assert S.fundamental_error(Fo, pr) < 0.05  # px, after the local optimisation and final fits
    assert np.all(m[g])  # every true inlier (outliers near an epipolar line can pass the threshold too)


def test_sift_fundamental_entry_checks(gcr):
    """The SIFT fundamental kind refuses P-NAPSAC before any device work; the
    python entry wants rows of 8 for solver=1."""
    lib = _abi.load()
    c = np.random.default_rng(4).uniform(0, 480, (50, 8))
    size = _abi.ImageSize(h1=480, w1=640, h2=480, w2=640)
    model, mask, st = np.zeros(9), np.zeros(50, np.uint8), _abi.Stats()
    p = ac_params(sampler=2)
    rc = lib.gcr_find_fundamental_sift(_abi.ptr(c), 50, ctypes.byref(size), None, ctypes.byref(p), _abi.ptr(model),
                                       _abi.ptr(mask), ctypes.byref(st))
    assert rc == _abi.GCR_UNSUPPORTED
    with pytest.raises(ValueError):
        gcr.findFundamentalMatrix(c[:, :4], 480, 640, 480, 640, solver=1)


def test_oracle_four_sift_solver_recovers_the_scene(oracle):
    """On exact SIFT correspondences of a two-view scene the true fundamental
    matrix satisfies every row of the four-SIFT system
    (solver_fundamental_matrix_four_sift.h:111-150), and a tape of inlier
    quadruples drives the oracle's run to it."""
    pr = S.two_view_sift_pair(7, n=600, inlier_ratio=0.5, sigma=0.0, angle_sigma=0.0, scale_sigma=0.0)
    c, g, F = pr["corr"], pr["inlier_gt"], pr["F_gt"]
    u1, v1, u2, v2, q1, q2, o1, o2 = c[g][:20].T
    s1, c1, s2, c2 = np.sin(o1), np.cos(o1), np.sin(o2), np.cos(o2)
    rows = np.stack([s2 * s2 * q2 * u1 - c1 * c2 * q1 * u2 - q2 * u1, s2 * s2 * q2 * v1 - s1 * c2 * q1 * u2 - q2 * v1,
                     s2 * s2 * q2 - q2, -c2 * s2 * q2 * u1 - c1 * c2 * q1 * v2, -c2 * s2 * q2 * v1 - s1 * c2 * q1 * v2,
                     -c2 * s2 * q2, -c1 * c2 * q1, -s1 * c2 * q1, 0 * u1], 1)
    assert np.abs(rows @ F.ravel()).max() < 1e-9 * np.abs(rows).max()
    idx = np.nonzero(g)[0]
    tape = np.stack([idx[4 * k:4 * k + 4] for k in range(30)]).astype(np.int32)
    p = _abi.Params(threshold=0.75, confidence=0.99, spatial_coherence_weight=0.975, neighborhood_size=8,
                    max_iterations=30, min_iterations=30, sampler=0, neighborhood=0, lo_number=20)
    rc, Fo, m, st = oracle.find(_abi.GCR_FUNDAMENTAL_SIFT, c, oracle.make_size(*pr["size"]), p, seed=1,
                                sample_tape=tape)
    assert rc == 0
    assert S.fundamental_error(Fo, pr) < 0.05
    assert np.all(m[g])


def test_sift_homography_entry_checks(gcr):
    """The SIFT homography kind (findHomographySIFT_,
    gcransac_python.cpp:4813-5069) refuses P-NAPSAC and MAGSAC++ before any
    device work; the python entry wants rows of 8 for solver=1; its defaults
    are the homography entry's without space partitioning."""
    lib = _abi.load()
    c = np.random.default_rng(5).uniform(0, 480, (50, 8))
    size = _abi.ImageSize(h1=480, w1=640, h2=480, w2=640)
    model, mask, st = np.zeros(9), np.zeros(50, np.uint8), _abi.Stats()
    for kw in (dict(sampler=2), dict(scoring=1)):
        p = ac_params(**kw)
        rc = lib.gcr_find_homography_sift(_abi.ptr(c), 50, ctypes.byref(size), None, ctypes.byref(p),
                                          _abi.ptr(model), _abi.ptr(mask), ctypes.byref(st))
        assert rc == _abi.GCR_UNSUPPORTED, kw
    with pytest.raises(ValueError):
        gcr.findHomography(c[:, :4], 480, 640, 480, 640, solver=1)
    with pytest.raises(NotImplementedError):
        gcr.findHomography(c, 480, 640, 480, 640, solver=3)
    p = gcr.default_params(_abi.GCR_HOMOGRAPHY_SIFT)
    assert (p.spatial_coherence_weight, p.neighborhood, p.neighborhood_size, p.use_space_partitioning) == \
        (0.975, 0, 4.0, 0)


def _sift_h_rows(p):
    """The reference's three rows of one SIFT correspondence
    (solver_homography_two_sift.h:150-185)."""
    u1, v1, u2, v2, q1, q2, a1, a2 = p
    s1, c1, s2, c2 = np.sin(a1), np.cos(a1), np.sin(a2), np.cos(a2)
    return [[0, 0, 0, u1, v1, 1, -u1 * v2, -v1 * v2, -v2], [u1, v1, 1, 0, 0, 0, -u1 * u2, -v1 * u2, -u2],
            [-c1 * s2, -s1 * s2, 0, c1 * c2, s1 * c2, 0, u2 * c1 * s2 - v2 * c1 * c2, u2 * s1 * s2 - v2 * s1 * c2, 0]]


def test_oracle_two_sift_homography_solver(oracle):
    """On exact SIFT correspondences of a homography the true homography
    satisfies the reference's six linear rows and both scale equations
    (q2 w^2 = q1 (w^2 det J), the coefficient expressions of
    solver_homography_two_sift.h:226-355), and the restated solver (null space
    by elimination, resultant quartic, bisection) returns it among its models
    for every sample of 200 scenes."""
    lib = oracle.load()
    for seed in range(200):
        pr = S.homography_sift_pair(seed, n=50, inlier_ratio=1.0, sigma=0.0, angle_sigma=0.0, scale_sigma=0.0)
        c = np.ascontiguousarray(pr["corr"])
        H = pr["H_gt"] / pr["H_gt"][2, 2]
        s = np.random.default_rng(seed).choice(50, 2, replace=False).astype(np.int64)
        if seed < 20:
            A = np.array(_sift_h_rows(c[s[0]]) + _sift_h_rows(c[s[1]]))
            assert np.abs(A @ H.ravel()).max() < 1e-9 * np.abs(A).max()
            for r in c[s]:
                u1, v1, u2, v2, q1, q2 = r[:6]
                h = H.ravel()
                w = h[6] * u1 + h[7] * v1 + h[8]
                D = (h[0] * h[4] - h[1] * h[3]) + u2 * (h[3] * h[7] - h[4] * h[6]) + v2 * (h[1] * h[6] - h[0] * h[7])
                assert abs(q2 * w * w - q1 * D) < 1e-9 * q2 * w * w
        out = np.zeros(90)
        k = lib.oracle_minimal(_abi.GCR_HOMOGRAPHY_SIFT, oracle._p(c), 50, oracle._p(s), oracle._p(out))
        assert 1 <= k <= 4
        err = min(np.abs(out[9 * i:9 * i + 9].reshape(3, 3) - H).max() / np.abs(H).max() for i in range(k))
        assert err < 1e-6, (seed, err)


def test_oracle_sift_homography_run_recovers_the_scene(oracle):
    """A tape of inlier pairs drives the oracle's SIFT-homography run to the
    true homography on a noisy scene (the local optimisation's 4-point fits
    average the noise), with every true inlier in the mask."""
    pr = S.homography_sift_pair(13, n=600, inlier_ratio=0.5, sigma=0.5)
    g = pr["inlier_gt"]
    idx = np.nonzero(g)[0]
    tape = np.stack([idx[2 * k:2 * k + 2] for k in range(30)]).astype(np.int32)
    p = ac_params(max_iterations=30, min_iterations=30, lo_number=20)
    rc, H, m, st = oracle.find(_abi.GCR_HOMOGRAPHY_SIFT, pr["corr"], oracle.make_size(*pr["size"]), p, seed=1,
                               sample_tape=tape)
    assert rc == 0
    assert S.homography_error(H, pr["H_gt"]) < 1.0  # px RMS over the image
    assert m[g].mean() > 0.97


def test_oracle_two_sift_homography_degenerate_samples(oracle):
    """A repeated SIFT correspondence (rank-deficient 6 x 9 system) and a
    pair with zero scales give no model or only finite ones."""
    lib = oracle.load()
    c = np.array([[100.0, 120.0, 110.0, 130.0, 2.0, 2.2, 0.3, 0.35],
                  [100.0, 120.0, 110.0, 130.0, 2.0, 2.2, 0.3, 0.35],
                  [300.0, 220.0, 310.0, 240.0, 0.0, 0.0, 1.0, 1.1],
                  [200.0, 320.0, 205.0, 335.0, 0.0, 0.0, -1.0, -0.9]], np.float64)
    for s in ([0, 1], [2, 3]):
        out = np.full(90, np.nan)
        k = lib.oracle_minimal(_abi.GCR_HOMOGRAPHY_SIFT, oracle._p(c), 4, oracle._p(np.array(s, np.int64)),
                               oracle._p(out))
        assert 0 <= k <= 4
        assert np.all(np.isfinite(out[:9 * k]))


def test_oracle_two_sift_homography_matches_an_svd_restatement(oracle):
    """On noisy SIFT correspondences (where the minimal models are not the
    true homography) the oracle's models equal those of an independent
    restatement of the reference's steps: the null space of the six rows by
    SVD (solver_homography_two_sift.h:187-190), h = a n1 + b n2 + n3, the two
    scale equations as conics in (a, b), their real intersections from
    NumPy's polynomial roots, each model divided by h33 (:469). Samples whose
    resultant has nearly double roots are skipped (their real-root count is
    decided by rounding); the models agree to 1e-3 relative, most to 1e-5
    (ill-conditioned samples lose digits on either route)."""
    lib = oracle.load()
    checked = 0
    rel = []
    for seed in range(60):
        pr = S.homography_sift_pair(300 + seed, n=40, inlier_ratio=1.0, sigma=1.0, angle_sigma=0.05,
                                    scale_sigma=0.05)
        c = np.ascontiguousarray(pr["corr"])
        s = np.random.default_rng(seed).choice(40, 2, replace=False)
        A = np.array(_sift_h_rows(c[s[0]]) + _sift_h_rows(c[s[1]]))
        N = np.linalg.svd(A)[2][-3:]

        def conic(r):
            u1, v1, u2, v2, q1, q2 = r[:6]

            def g(h):
                w = h[6] * u1 + h[7] * v1 + h[8]
                D = (h[0] * h[4] - h[1] * h[3]) + u2 * (h[3] * h[7] - h[4] * h[6]) + v2 * (h[1] * h[6] - h[0] * h[7])
                return q2 * w * w - q1 * D
            # quadratic form coefficients by polarisation
            f = lambda a, b: g(a * N[0] + b * N[1] + N[2])  # noqa: E731
            c5 = f(0, 0)
            c0 = (f(1, 0) + f(-1, 0)) / 2 - c5
            c3 = (f(1, 0) - f(-1, 0)) / 2
            c2 = (f(0, 1) + f(0, -1)) / 2 - c5
            c4 = (f(0, 1) - f(0, -1)) / 2
            c1 = f(1, 1) - c0 - c2 - c3 - c4 - c5
            return c0, c1, c2, c3, c4, c5
        K1, K2 = conic(c[s[0]]), conic(c[s[1]])
        # resultant in b of the two quadratics in a
        A1, A2 = float(K1[0]), float(K2[0])
        B1, B2 = np.poly1d([K1[1], K1[3]]), np.poly1d([K2[1], K2[3]])
        C1, C2 = np.poly1d([K1[2], K1[4], K1[5]]), np.poly1d([K2[2], K2[4], K2[5]])
        P = A1 * C2 - A2 * C1
        L = A1 * B2 - A2 * B1
        R = P * P - L * (B1 * C2 - B2 * C1)
        roots = np.roots(R.coeffs)
        if np.any(np.abs(roots.imag) < 1e-3 * (1 + np.abs(roots.real))) and \
                np.any((np.abs(roots.imag) > 0) & (np.abs(roots.imag) < 1e-3 * (1 + np.abs(roots.real)))):
            continue
        ref = []
        for b in roots[np.abs(roots.imag) == 0].real:
            a = -P(b) / L(b)
            h = a * N[0] + b * N[1] + N[2]
            ref.append(h / h[8])
        out = np.zeros(90)
        k = lib.oracle_minimal(_abi.GCR_HOMOGRAPHY_SIFT, oracle._p(c), 40, oracle._p(s.astype(np.int64)),
                               oracle._p(out))
        assert k == len(ref), (seed, k, len(ref))
        for i in range(k):
            h = out[9 * i:9 * i + 9]
            # two independent numerical routes on raw pixel coordinates (rows
            # with entries up to 1e5): every model within 1e-3 relative of one
            # of the other route's, most within 1e-5
            rel.append(min(np.abs(h - r).max() / np.abs(r).max() for r in ref))
            assert rel[-1] < 1e-3, (seed, i, rel[-1])
        checked += 1
    assert checked >= 40
    assert np.mean(np.array(rel) < 1e-5) > 0.9, np.sort(rel)[-5:]


def _orientation_ok(F, pts):
    """isOrientationValid (fundamental_estimator.h) on the rows pts."""
    e = np.cross(F[0], F[2])
    if np.all(np.abs(e) <= 1.9984e-15):
        e = np.cross(F[1], F[2])
    sg = [(F[0, 0] * p[2] + F[1, 0] * p[3] + F[2, 0]) * (e[1] - e[2] * p[1]) for p in pts]
    return all(not (sg[0] * v < 0) for v in sg[1:])


def _epipolar_row(p):
    x0, y0, x1, y1 = p[:4]
    return [x1 * x0, x1 * y0, x1, y1 * x0, y1 * y0, y1, x0, y0, 1.0]


def _affine_rows(p):
    x0, y0, x1, y1, a11, a12, a21, a22 = p
    return [[x1 + a11 * x0, a11 * y0, a11, y1 + a21 * x0, a21 * y0, a21, 1, 0, 0],
            [a12 * x0, x1 + a12 * y0, a12, a22 * x0, y1 + a22 * y0, a22, 0, 1, 0]]


def _sift_row(p):
    u1, v1, u2, v2, q1, q2, o1, o2 = p
    s1, c1, s2, c2 = np.sin(o1), np.cos(o1), np.sin(o2), np.cos(o2)
    return [s2 * s2 * q2 * u1 - c1 * c2 * q1 * u2 - q2 * u1, s2 * s2 * q2 * v1 - s1 * c2 * q1 * u2 - q2 * v1,
            s2 * s2 * q2 - q2, -c2 * s2 * q2 * u1 - c1 * c2 * q1 * v2, -c2 * s2 * q2 * v1 - s1 * c2 * q1 * v2,
            -c2 * s2 * q2, -c1 * c2 * q1, -s1 * c2 * q1, 0.0]


@pytest.mark.parametrize("kind", ["affine", "sift"])
def test_oracle_fundamental_rows8_solvers_match_an_svd_restatement(oracle, kind):
    """On noisy affine / SIFT correspondences the oracle's minimal models equal
    an independent restatement: the reference's seven rows (three-affine:
    epipolar rows of all three and affine rows of the first two,
    solver_fundamental_matrix_three_affine.h:118-170; four-SIFT: epipolar
    rows of all four and the orientation-scale rows of the first three,
    solver_fundamental_matrix_four_sift.h:111-150), their two-dimensional
    null space by SVD, det(x F1 + (1 - x) F2) = 0 by NumPy's roots, the
    oriented constraint on the sample. Compared as sets of unit-norm models
    up to sign; samples with nearly double roots are skipped."""
    lib = oracle.load()
    gen = S.two_view_affine_pair if kind == "affine" else S.two_view_sift_pair
    code = _abi.GCR_FUNDAMENTAL_AFFINE if kind == "affine" else _abi.GCR_FUNDAMENTAL_SIFT
    m = 3 if kind == "affine" else 4
    checked = 0
    for seed in range(40):
        pr = gen(500 + seed, n=40, inlier_ratio=1.0)
        c = np.ascontiguousarray(pr["corr"])
        s = np.random.default_rng(seed).choice(40, m, replace=False)
        p = c[s]
        if kind == "affine":
            A = np.array([_epipolar_row(q) for q in p] + _affine_rows(p[0]) + _affine_rows(p[1]))
        else:
            A = np.array([_epipolar_row(q) for q in p] + [_sift_row(q) for q in p[:3]])
        V = np.linalg.svd(A)[2]
        F1, F2 = V[-2].reshape(3, 3), V[-1].reshape(3, 3)
        xs = np.linspace(-2, 2, 4)
        dets = [np.linalg.det(x * F1 + (1 - x) * F2) for x in xs]
        cub = np.polyfit(xs, dets, 3)
        roots = np.roots(cub)
        near = (np.abs(roots.imag) > 0) & (np.abs(roots.imag) < 1e-4 * (1 + np.abs(roots.real)))
        if np.any(near):
            continue
        ref = []
        for x in roots[roots.imag == 0].real:
            F = x * F1 + (1 - x) * F2
            if _orientation_ok(F, p):
                ref.append(F.ravel() / np.linalg.norm(F))
        out = np.zeros(90)
        k = lib.oracle_minimal(code, oracle._p(c), 40, oracle._p(s.astype(np.int64)), oracle._p(out))
        assert k == len(ref), (seed, k, len(ref))
        for i in range(k):
            f = out[9 * i:9 * i + 9] / np.linalg.norm(out[9 * i:9 * i + 9])
            err = min(min(np.abs(f - r).max(), np.abs(f + r).max()) for r in ref)
            assert err < 1e-6, (seed, i, err)
        checked += 1
    assert checked >= 30
