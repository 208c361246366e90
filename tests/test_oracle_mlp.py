"""CPU checks of the learned proposal's NumPy oracle (oracle/oracle_mlp.py):
its analytic gradient against central finite differences, the feature
definition on a hand-made pair, the ordering rule, and the checkpoint format
of pygcransac.learned (header and payload layout, no device needed)."""
import json
import struct

import numpy as np

import oracle_mlp as M


def test_gradient_matches_finite_differences():
    rng = np.random.Generator(np.random.PCG64(0))
    P = rng.normal(scale=0.2, size=M.OFF["count"])
    X = rng.normal(size=(12, M.IN))
    X[:, M.FEAT:] = 0
    y = (rng.uniform(size=12) < 0.5).astype(float)
    w = rng.uniform(0.5, 2.0, 12)
    _, G = M.loss_and_grad(X, P, y, w, rounding=False)
    idx = np.r_[rng.integers(0, M.OFF["count"], 200), M.OFF["b4"], M.OFF["W4"] + 3]
    h = 1e-6
    for i in idx:
        Pp, Pm = P.copy(), P.copy()
        Pp[i] += h
        Pm[i] -= h
        fd = (M.loss_and_grad(X, Pp, y, w, rounding=False)[0] - M.loss_and_grad(X, Pm, y, w, rounding=False)[0]) / (2 * h)
        assert abs(fd - G[i]) <= 1e-6 + 1e-5 * abs(fd), (i, fd, G[i])


def test_features_of_a_hand_made_pair():
    # three points moving by (+10, 0), one outlier moving by (-200, +100)
    corr = np.array([[100, 100, 110, 100], [103, 100, 113, 100], [100, 104, 110, 104], [102, 102, -98, 202.0]])
    X = M.features(corr, (480, 640, 480, 640))
    assert X.shape == (4, M.IN) and np.all(X[:, M.FEAT:] == 0)
    np.testing.assert_allclose(X[0, :4], [100 / 640 - 0.5, 100 / 480 - 0.5, 110 / 640 - 0.5, 100 / 480 - 0.5],
                               rtol=1e-6)
    # point 0: the two agreeing neighbours first (difference 0, distances 3
    # and 4 px), then the outlier (difference |(-210, 100)|, distance sqrt 8),
    # then five missing neighbours
    q = lambda v: 0.25 * np.sqrt(v)  # noqa: E731
    np.testing.assert_allclose(X[0, 4:10], [0, q(3), 0, q(4), q(np.hypot(210, 100)), q(np.sqrt(8))], rtol=1e-6)
    np.testing.assert_allclose(X[0, 10:20], 4.0)
    # the outlier disagrees with every neighbour
    assert np.all(X[3, 4:10:2] > 3.5)


def test_order_rule():
    z = np.array([0.5, np.nan, 2.0, 0.5, -np.inf, 2.0], np.float32)
    np.testing.assert_array_equal(M.order(z), [2, 5, 0, 3, 1, 4])


def test_bf16_round_is_nearest_even():
    x = np.array([1.0, 1.0 + 2 ** -8, 1.0 + 3 * 2 ** -8, -3.14159, 1e-30], np.float32)
    r = M.bf16_round(x)
    assert r[0] == 1.0 and r[1] == 1.0 and r[2] == 1.0 + 2 ** -6
    assert abs(r[3] + 3.14159) < 2 ** -7 * 4


def test_checkpoint_layout(tmp_path):
    from pygcransac import learned
    hdr = json.dumps({"count": M.OFF["count"], "feature_width": M.IN, "step": 7}).encode()
    body = np.arange(3 * M.OFF["count"], dtype="<f4").tobytes()
    p = tmp_path / "x.gcrl"
    p.write_bytes(learned.MAGIC + struct.pack("<I", len(hdr)) + hdr + body)
    blob = p.read_bytes()
    (hl,) = struct.unpack("<I", blob[4:8])
    assert json.loads(blob[8:8 + hl])["step"] == 7
    assert len(blob) - 8 - hl == 12 * M.OFF["count"]
