"""Seeded synthetic image pairs with known ground truth.

These stand in for the reference's real SIFT-matched image pairs (which need
OpenCV to produce). Shapes, sizes and value distributions follow the benchmark
workloads of this engine:

* ``homography_pair``: N=2000 in 640x480, H = T(c) [s R(theta) | t] T(-c) with a
  perspective row, theta ~ U(+-15 deg), s ~ U(0.8, 1.2), t ~ U(+-50 px),
  p ~ U(+-1e-4); 40 % inliers with sigma = 1 px, uniform outliers.
* ``two_view_pair``: points uniform in camera 1's frustum at depth 2-10 m,
  focal 800 px, 640x480, camera 2 rotated by U(+-30 deg) about a random axis
  and translated by a unit vector; inliers with sigma = 0.5 px, uniform
  outliers. Used for both the fundamental (pixels) and essential (K known)
  workloads. With ``smooth_depth=True`` the inliers' depth is a smooth field
  over the first image (three random plane waves, 0.5-2 cycles per image,
  2-10 m) instead of independent per point: the piecewise-smooth scenes real
  image pairs show, in which neighbouring inliers move alike (the hard
  fundamental-matrix workload of the learned proposal, 5-10 % inliers).

All generators use numpy ``Generator(PCG64(seed))``.
"""
import numpy as np

W, H = 640, 480


def _rng(seed):
    return np.random.Generator(np.random.PCG64(seed))


def _rot(axis, ang):
    axis = axis / np.linalg.norm(axis)
    K = np.array([[0, -axis[2], axis[1]], [axis[2], 0, -axis[0]], [-axis[1], axis[0], 0]])
    return np.eye(3) + np.sin(ang) * K + (1 - np.cos(ang)) * K @ K


def random_homography(rng, w=W, h=H):
    th = np.deg2rad(rng.uniform(-15, 15))
    s = rng.uniform(0.8, 1.2)
    t = rng.uniform(-50, 50, 2)
    p = rng.uniform(-1e-4, 1e-4, 2)
    c = np.array([w / 2, h / 2])
    A = np.eye(3)
    A[:2, :2] = s * np.array([[np.cos(th), -np.sin(th)], [np.sin(th), np.cos(th)]])
    A[:2, 2] = t
    A[2, :2] = p
    Tc = np.array([[1, 0, c[0]], [0, 1, c[1]], [0, 0, 1.0]])
    Tm = np.array([[1, 0, -c[0]], [0, 1, -c[1]], [0, 0, 1.0]])
    Hm = Tc @ A @ Tm
    return Hm / Hm[2, 2]


def project_h(Hm, x):
    xh = np.c_[x, np.ones(len(x))] @ Hm.T
    return xh[:, :2] / xh[:, 2:3]


def homography_pair(seed, n=2000, inlier_ratio=0.4, sigma=1.0, w=W, h=H):
    """Returns dict(corr [n,4] f64, H_gt, inlier_gt bool[n], size (h1,w1,h2,w2))."""
    rng = _rng(seed)
    Hm = random_homography(rng, w, h)
    ni = int(round(n * inlier_ratio))
    pts1 = np.zeros((0, 2))
    pts2 = np.zeros((0, 2))
    while len(pts1) < ni:
        x1 = rng.uniform([0, 0], [w, h], size=(2 * ni, 2))
        x2 = project_h(Hm, x1) + rng.normal(0, sigma, size=(2 * ni, 2))
        ok = (x2[:, 0] >= 0) & (x2[:, 0] < w) & (x2[:, 1] >= 0) & (x2[:, 1] < h)
        pts1 = np.r_[pts1, x1[ok]]
        pts2 = np.r_[pts2, x2[ok]]
    inl = np.c_[pts1[:ni], pts2[:ni]]
    no = n - ni
    out = np.c_[rng.uniform([0, 0], [w, h], size=(no, 2)), rng.uniform([0, 0], [w, h], size=(no, 2))]
    corr = np.r_[inl, out]
    gt = np.r_[np.ones(ni, bool), np.zeros(no, bool)]
    perm = rng.permutation(n)
    return dict(corr=corr[perm], H_gt=Hm, inlier_gt=gt[perm], size=(h, w, h, w))


def homography_jacobian(Hm, x):
    """[n, 4] row-major 2x2 Jacobians (a11, a12, a21, a22) of x -> H x at the
    points x [n, 2]: the local affine map of an affine correspondence."""
    X = np.c_[x, np.ones(len(x))] @ Hm.T
    s = X[:, 2]
    u, v = X[:, 0] / s, X[:, 1] / s
    a11 = (Hm[0, 0] - u * Hm[2, 0]) / s
    a12 = (Hm[0, 1] - u * Hm[2, 1]) / s
    a21 = (Hm[1, 0] - v * Hm[2, 0]) / s
    a22 = (Hm[1, 1] - v * Hm[2, 1]) / s
    return np.c_[a11, a12, a21, a22]


def homography_affine_pair(seed, n=2000, inlier_ratio=0.4, sigma=1.0, affine_sigma=0.02, w=W, h=H):
    """Affine correspondences of a homography: the point pairs of
    homography_pair and, per row, the local affine map (a11, a12, a21, a22) —
    the Jacobian of the true homography at x1 plus N(0, affine_sigma) noise
    for inliers, a random map (rotation by U(-pi, pi), scales U(0.5, 2)) for
    outliers. Returns dict(corr [n, 8], H_gt, inlier_gt, size)."""
    pr = homography_pair(seed, n=n, inlier_ratio=inlier_ratio, sigma=sigma, w=w, h=h)
    rng = _rng(seed + 7919)
    corr = pr["corr"]
    A = homography_jacobian(pr["H_gt"], corr[:, :2]) + rng.normal(0, affine_sigma, size=(n, 4))
    out = ~pr["inlier_gt"]
    k = int(out.sum())
    ang = rng.uniform(-np.pi, np.pi, k)
    sc = rng.uniform(0.5, 2.0, (k, 2))
    c, si = np.cos(ang), np.sin(ang)
    A[out] = np.c_[c * sc[:, 0], -si * sc[:, 1], si * sc[:, 0], c * sc[:, 1]]
    return dict(corr=np.ascontiguousarray(np.c_[corr, A]), H_gt=pr["H_gt"], inlier_gt=pr["inlier_gt"],
                size=pr["size"])


def homography_sift_pair(seed, n=2000, inlier_ratio=0.4, sigma=1.0, angle_sigma=0.01, scale_sigma=0.01, w=W, h=H):
    """SIFT-like correspondences of a homography: the point pairs of
    homography_pair and, per row, the features' scales and orientations
    (q1, q2, o1, o2). For an inlier, o1 ~ U(-pi, pi) and q1 ~ U(1, 5); the
    Jacobian J of the true homography at x1 gives o2 = the direction of
    J (cos o1, sin o1) and q2 = q1 det J (the scale equation of the
    two-SIFT homography solver); o2 and q2 then get N(0, angle_sigma) and
    relative N(0, scale_sigma) noise. Outliers have independent q ~ U(1, 5)
    and o ~ U(-pi, pi). Returns dict(corr [n, 8], H_gt, inlier_gt, size)."""
    pr = homography_pair(seed, n=n, inlier_ratio=inlier_ratio, sigma=sigma, w=w, h=h)
    rng = _rng(seed + 15485863)
    corr = pr["corr"]
    J = homography_jacobian(pr["H_gt"], corr[:, :2])
    o1 = rng.uniform(-np.pi, np.pi, n)
    q1 = rng.uniform(1.0, 5.0, n)
    vx = J[:, 0] * np.cos(o1) + J[:, 1] * np.sin(o1)
    vy = J[:, 2] * np.cos(o1) + J[:, 3] * np.sin(o1)
    o2 = np.arctan2(vy, vx) + rng.normal(0, angle_sigma, n)
    q2 = q1 * (J[:, 0] * J[:, 3] - J[:, 1] * J[:, 2]) * (1.0 + rng.normal(0, scale_sigma, n))
    out = ~pr["inlier_gt"]
    k = int(out.sum())
    o1[out] = rng.uniform(-np.pi, np.pi, k)
    o2[out] = rng.uniform(-np.pi, np.pi, k)
    q1[out] = rng.uniform(1.0, 5.0, k)
    q2[out] = rng.uniform(1.0, 5.0, k)
    return dict(pr, corr=np.ascontiguousarray(np.c_[corr, q1, q2, o1, o2]))


def intrinsics(f=800.0, w=W, h=H):
    return np.array([[f, 0, w / 2], [0, f, h / 2], [0, 0, 1.0]])


def skew(t):
    return np.array([[0, -t[2], t[1]], [t[2], 0, -t[0]], [-t[1], t[0], 0]])


def depth_field(rng, w=W, h=H):
    """Smooth depth (2-10 m) over the first image: 6 + 4 * (0.5 s1 + 0.3 s2 +
    0.2 s3) with s_i = sin(2 pi f_i (cos a_i u/w + sin a_i v/h) + phi_i),
    f_i ~ U(0.5, 2) cycles per image, a_i, phi_i ~ U(0, 2 pi)."""
    fr = rng.uniform(0.5, 2.0, 3)
    ang = rng.uniform(0, 2 * np.pi, 3)
    ph = rng.uniform(0, 2 * np.pi, 3)
    amp = np.array([0.5, 0.3, 0.2])

    def Z(uv):
        u, v = uv[:, 0] / w, uv[:, 1] / h
        s = sum(amp[i] * np.sin(2 * np.pi * fr[i] * (np.cos(ang[i]) * u + np.sin(ang[i]) * v) + ph[i])
                for i in range(3))
        return 6.0 + 4.0 * s
    return Z


def two_view_pair(seed, n=5000, inlier_ratio=0.25, sigma=0.5, f=800.0, w=W, h=H, max_angle_deg=30.0,
                  smooth_depth=False, planar_motion=False):
    """Returns dict(corr [n,4] pixels, K, R, t, F_gt, E_gt, inlier_gt, size).
    planar_motion: rotation about the camera's y axis by up to max_angle_deg
    and a unit translation in its x-z plane (the motion model of the planar
    essential-matrix solver)."""
    rng = _rng(seed)
    Zf = depth_field(rng, w, h) if smooth_depth else None
    K = intrinsics(f, w, h)
    Ki = np.linalg.inv(K)
    ni = int(round(n * inlier_ratio))
    for _attempt in range(100):
        if planar_motion:
            R = _rot(np.array([0.0, 1.0, 0.0]), np.deg2rad(rng.uniform(-max_angle_deg, max_angle_deg)))
            phi = rng.uniform(-np.pi, np.pi)
            t = np.array([np.sin(phi), 0.0, np.cos(phi)])
        else:
            R = _rot(rng.normal(size=3), np.deg2rad(rng.uniform(-max_angle_deg, max_angle_deg)))
            t = rng.normal(size=3)
            t /= np.linalg.norm(t)
        pts1 = np.zeros((0, 2))
        pts2 = np.zeros((0, 2))
        tries = 0
        while len(pts1) < ni and tries < 200:
            tries += 1
            m = 4 * ni
            uv = rng.uniform([0, 0], [w, h], size=(m, 2))
            depth = rng.uniform(2, 10, size=m) if Zf is None else Zf(uv)
            X = (np.c_[uv, np.ones(m)] @ Ki.T) * depth[:, None]
            X2 = X @ R.T + t
            front = X2[:, 2] > 0.1
            x2 = (X2 @ K.T)
            x2 = x2[:, :2] / x2[:, 2:3]
            x1n = uv + rng.normal(0, sigma, size=(m, 2))
            x2n = x2 + rng.normal(0, sigma, size=(m, 2))
            ok = front & (x2n[:, 0] >= 0) & (x2n[:, 0] < w) & (x2n[:, 1] >= 0) & (x2n[:, 1] < h) & \
                (x1n[:, 0] >= 0) & (x1n[:, 0] < w) & (x1n[:, 1] >= 0) & (x1n[:, 1] < h)
            pts1 = np.r_[pts1, x1n[ok]]
            pts2 = np.r_[pts2, x2n[ok]]
        if len(pts1) >= ni:
            break
    inl = np.c_[pts1[:ni], pts2[:ni]]
    no = n - ni
    out = np.c_[rng.uniform([0, 0], [w, h], size=(no, 2)), rng.uniform([0, 0], [w, h], size=(no, 2))]
    corr = np.r_[inl, out]
    gt = np.r_[np.ones(ni, bool), np.zeros(no, bool)]
    perm = rng.permutation(n)
    E = skew(t) @ R
    F = Ki.T @ E @ Ki
    return dict(corr=corr[perm], K=K, R=R, t=t, E_gt=E / np.linalg.norm(E), F_gt=F / np.linalg.norm(F),
                inlier_gt=gt[perm], size=(h, w, h, w))


def two_view_affine_pair(seed, n=2000, inlier_ratio=0.4, sigma=0.5, affine_sigma=0.01, f=800.0, w=W, h=H,
                         max_angle_deg=30.0):
    """Affine correspondences of a two-view scene (the scene of two_view_pair):
    each inlier is a 3D point on a local plane whose normal is the viewing ray
    turned by up to about 30 degrees; its local affine map (a11, a12, a21, a22)
    is the Jacobian at x1 of the plane's homography K (R + t n^T / d) K^-1 plus
    N(0, affine_sigma) noise, and the points carry N(0, sigma) pixel noise.
    Outliers are random point pairs with random maps (rotation by U(-pi, pi),
    scales U(0.5, 2)). Returns dict(corr [n, 8], K, R, t, F_gt, E_gt,
    inlier_gt, size)."""
    rng = _rng(seed)
    K = intrinsics(f, w, h)
    Ki = np.linalg.inv(K)
    ni = int(round(n * inlier_ratio))
    rows = np.zeros((0, 8))
    for _attempt in range(100):
        R = _rot(rng.normal(size=3), np.deg2rad(rng.uniform(-max_angle_deg, max_angle_deg)))
        t = rng.normal(size=3)
        t /= np.linalg.norm(t)
        rows = np.zeros((0, 8))
        tries = 0
        while len(rows) < ni and tries < 200:
            tries += 1
            m = 4 * ni
            uv = rng.uniform([0, 0], [w, h], size=(m, 2))
            depth = rng.uniform(2, 10, size=m)
            X = (np.c_[uv, np.ones(m)] @ Ki.T) * depth[:, None]
            X2 = X @ R.T + t
            front = X2[:, 2] > 0.1
            nrm = -X / np.linalg.norm(X, axis=1, keepdims=True) + rng.normal(0, 0.3, size=(m, 3))
            nrm /= np.linalg.norm(nrm, axis=1, keepdims=True)
            d = np.sum(nrm * X, axis=1)
            Hs = np.einsum("ij,njk,kl->nil", K, R[None] + t[None, :, None] * (nrm / d[:, None])[:, None, :], Ki)
            Xh = np.einsum("nij,nj->ni", Hs, np.c_[uv, np.ones(m)])
            sc = Xh[:, 2]
            u2, v2 = Xh[:, 0] / sc, Xh[:, 1] / sc
            A = np.c_[(Hs[:, 0, 0] - u2 * Hs[:, 2, 0]) / sc, (Hs[:, 0, 1] - u2 * Hs[:, 2, 1]) / sc,
                      (Hs[:, 1, 0] - v2 * Hs[:, 2, 0]) / sc, (Hs[:, 1, 1] - v2 * Hs[:, 2, 1]) / sc]
            x2 = X2 @ K.T
            x2 = x2[:, :2] / x2[:, 2:3]
            x1n = uv + rng.normal(0, sigma, size=(m, 2))
            x2n = x2 + rng.normal(0, sigma, size=(m, 2))
            An = A + rng.normal(0, affine_sigma, size=(m, 4))
            ok = front & (x2n[:, 0] >= 0) & (x2n[:, 0] < w) & (x2n[:, 1] >= 0) & (x2n[:, 1] < h) & \
                (x1n[:, 0] >= 0) & (x1n[:, 0] < w) & (x1n[:, 1] >= 0) & (x1n[:, 1] < h) & \
                (np.abs(A).max(axis=1) < 10.0)
            rows = np.r_[rows, np.c_[x1n, x2n, An][ok]]
        if len(rows) >= ni:
            break
    no = n - ni
    ang = rng.uniform(-np.pi, np.pi, no)
    sc = rng.uniform(0.5, 2.0, (no, 2))
    c, si = np.cos(ang), np.sin(ang)
    out = np.c_[rng.uniform([0, 0], [w, h], size=(no, 2)), rng.uniform([0, 0], [w, h], size=(no, 2)),
                c * sc[:, 0], -si * sc[:, 1], si * sc[:, 0], c * sc[:, 1]]
    corr = np.r_[rows[:ni], out]
    gt = np.r_[np.ones(ni, bool), np.zeros(no, bool)]
    perm = rng.permutation(n)
    E = skew(t) @ R
    F = Ki.T @ E @ Ki
    return dict(corr=np.ascontiguousarray(corr[perm]), K=K, R=R, t=t, E_gt=E / np.linalg.norm(E),
                F_gt=F / np.linalg.norm(F), inlier_gt=gt[perm], size=(h, w, h, w))


def two_view_sift_pair(seed, n=2000, inlier_ratio=0.4, sigma=0.5, angle_sigma=0.01, scale_sigma=0.01, **kw):
    """SIFT-like correspondences of the scene of two_view_affine_pair: rows
    (x1, y1, x2, y2, q1, q2, o1, o2), a feature's scale q and orientation o
    in each image. For an inlier, o1 ~ U(-pi, pi) and q1 ~ U(1, 5), and the
    local affine map A of its plane gives q2 (cos o2, sin o2) = A q1 (cos o1,
    sin o1); o2 and q2 then get N(0, angle_sigma) and relative N(0,
    scale_sigma) noise. Outliers have independent q ~ U(1, 5) and o ~ U(-pi,
    pi). Returns dict(corr [n, 8], K, R, t, F_gt, E_gt, inlier_gt, size)."""
    pr = two_view_affine_pair(seed, n=n, inlier_ratio=inlier_ratio, sigma=sigma, affine_sigma=0.0, **kw)
    rng = _rng(seed + 104729)
    c = pr["corr"]
    a11, a12, a21, a22 = c[:, 4], c[:, 5], c[:, 6], c[:, 7]
    o1 = rng.uniform(-np.pi, np.pi, n)
    q1 = rng.uniform(1.0, 5.0, n)
    vx = q1 * (a11 * np.cos(o1) + a12 * np.sin(o1))
    vy = q1 * (a21 * np.cos(o1) + a22 * np.sin(o1))
    o2 = np.arctan2(vy, vx) + rng.normal(0, angle_sigma, n)
    q2 = np.hypot(vx, vy) * (1.0 + rng.normal(0, scale_sigma, n))
    out = ~pr["inlier_gt"]
    k = int(out.sum())
    o1[out] = rng.uniform(-np.pi, np.pi, k)
    o2[out] = rng.uniform(-np.pi, np.pi, k)
    q1[out] = rng.uniform(1.0, 5.0, k)
    q2[out] = rng.uniform(1.0, 5.0, k)
    corr = np.ascontiguousarray(np.c_[c[:, :4], q1, q2, o1, o2])
    return dict(pr, corr=corr)


# --- model error against ground truth -------------------------------------

def homography_error(H_est, H_gt, w=W, h=H):
    """RMS transfer error (px) of a 1000-point grid under H_est vs H_gt."""
    if H_est is None:
        return np.inf
    gx, gy = np.meshgrid(np.linspace(0, w, 40), np.linspace(0, h, 25))
    x = np.c_[gx.ravel(), gy.ravel()]
    d = project_h(H_est, x) - project_h(H_gt, x)
    return float(np.sqrt(np.mean(np.sum(d * d, axis=1))))


def sampson_sq(F, corr):
    x1 = np.c_[corr[:, :2], np.ones(len(corr))]
    x2 = np.c_[corr[:, 2:4], np.ones(len(corr))]
    Fx1 = x1 @ F.T
    Ftx2 = x2 @ F
    num = np.sum(x2 * Fx1, axis=1) ** 2
    den = Fx1[:, 0] ** 2 + Fx1[:, 1] ** 2 + Ftx2[:, 0] ** 2 + Ftx2[:, 1] ** 2
    return num / den


def fundamental_error(F_est, pair, n=1000, seed=12345):
    """Mean Sampson distance (px) of noise-free ground-truth correspondences."""
    if F_est is None or not np.any(F_est):
        return np.inf
    clean = two_view_pair_clean(pair, n, seed)
    with np.errstate(invalid="ignore", divide="ignore"):
        e = float(np.mean(np.sqrt(sampson_sq(F_est, clean))))
    return e if np.isfinite(e) else np.inf


def two_view_pair_clean(pair, n, seed):
    rng = _rng(seed)
    K, R, t = pair["K"], pair["R"], pair["t"]
    Ki = np.linalg.inv(K)
    h, w = pair["size"][0], pair["size"][1]
    out = np.zeros((0, 4))
    while len(out) < n:
        m = 4 * n
        uv = rng.uniform([0, 0], [w, h], size=(m, 2))
        depth = rng.uniform(2, 10, size=m)
        X = (np.c_[uv, np.ones(m)] @ Ki.T) * depth[:, None]
        X2 = X @ R.T + t
        x2 = X2 @ K.T
        x2 = x2[:, :2] / x2[:, 2:3]
        ok = (X2[:, 2] > 0.1) & (x2[:, 0] >= 0) & (x2[:, 0] < w) & (x2[:, 1] >= 0) & (x2[:, 1] < h)
        out = np.r_[out, np.c_[uv[ok], x2[ok]]]
    return out[:n]


def essential_error(E_est, pair):
    """max(rotation error, translation-direction error) in degrees over the
    four decompositions of E_est (best one), like a cheirality-free pose check."""
    if E_est is None:
        return np.inf
    U, _, Vt = np.linalg.svd(E_est)
    if np.linalg.det(U) < 0:
        U = -U
    if np.linalg.det(Vt) < 0:
        Vt = -Vt
    Wm = np.array([[0, -1, 0], [1, 0, 0], [0, 0, 1.0]])
    best = np.inf
    for Rc in (U @ Wm @ Vt, U @ Wm.T @ Vt):
        for tc in (U[:, 2], -U[:, 2]):
            cr = np.clip((np.trace(Rc.T @ pair["R"]) - 1) / 2, -1, 1)
            er = np.degrees(np.arccos(cr))
            ct = np.clip(np.dot(tc, pair["t"]) / np.linalg.norm(tc) / np.linalg.norm(pair["t"]), -1, 1)
            et = np.degrees(np.arccos(ct))
            best = min(best, max(er, et))
    return float(best)
