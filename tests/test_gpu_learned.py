"""GPU checks of the learned proposal (csrc/gcr_learned.cu) against the NumPy
oracle (oracle/oracle_mlp.py): neighbour features bit-exact, tensor-core
forward logits and the backward gradient within FP32-accumulation tolerance of
the FP64 restatement on the same BF16 weights and roundings, the Adam step, the per-pair ordering and
mask mapping exact; the learned batch equals the plain engine run on the same
order; and a trained network's gain over the uniform sampler on hard pairs."""
import numpy as np
import pytest

import oracle_mlp as M
from pygcransac import _abi, synthetic as S

pytestmark = pytest.mark.gpu

# FP32 accumulation of BF16-weighted sums over <= 128 terms against FP64
LOGIT_RTOL = 1e-3
GRAD_RTOL = 2e-4


@pytest.fixture(scope="module")
def torch():
    import torch
    assert torch.cuda.is_available()
    return torch


@pytest.fixture(scope="module")
def net(torch):
    from pygcransac.learned import LearnedProposal
    return LearnedProposal(seed=3)


def _pairs(sizes_n, seed0=0):
    out = []
    for k, n in enumerate(sizes_n):
        if n >= 20:
            pr = S.two_view_pair(seed0 + k, n=n, inlier_ratio=0.3)
            out.append((pr["corr"], pr["size"]))
        else:
            rng = np.random.Generator(np.random.PCG64(seed0 + k))
            out.append((rng.uniform(0, 480, (n, 4)), (480, 640, 480, 640)))
    return out


def test_features_bit_exact(net):
    """Grid search (pairs up to 8192) and all-pairs scan (larger pairs) give
    the oracle's features bit for bit, including duplicate points (distance
    ties broken by index), a zero-width bounding box and points outside the
    image."""
    pairs = _pairs([300, 1, 2, 8, 9, 2500, 129, 8500])
    rng = np.random.Generator(np.random.PCG64(21))
    dup = rng.integers(0, 12, (600, 4)).astype(np.float64)  # many identical first-image points
    line = np.c_[np.full(300, 17.0), rng.uniform(0, 480, 300), rng.uniform(0, 640, (300, 2))]
    outside = rng.uniform(-200, 900, (700, 4))
    pairs += [(dup, (480, 640, 480, 640)), (line, (480, 640, 480, 640)), (outside, (480, 640, 480, 640))]
    feat, offsets = net.host_features([c for c, _ in pairs], [z for _, z in pairs])
    F = feat.cpu().numpy()
    for i, (c, z) in enumerate(pairs):
        ref = M.features(c, z)
        got = F[offsets[i]:offsets[i + 1]]
        assert np.array_equal(got, ref), f"pair {i} (n={len(c)}): rows {np.nonzero((got != ref).any(1))[0][:8]}"


def _device_forward(torch, net, X):
    n = len(X)
    a = [torch.empty((n, 128), dtype=torch.float32, device="cuda") for _ in range(3)]
    z = torch.empty(n, dtype=torch.float32, device="cuda")
    d_x = torch.from_numpy(X).cuda()
    import ctypes
    vp = lambda t: ctypes.c_void_p(t.data_ptr())  # noqa: E731
    assert net.lib.gcr_learned_forward(vp(d_x), n, vp(net.bf16), vp(a[0]), vp(a[1]), vp(a[2]), vp(z), None) == 0
    return d_x, [t.cpu().numpy().astype(np.float64) for t in a], z


def test_forward_matches_oracle(torch, net):
    """Tensor-core forward vs the FP64 restatement with the same BF16
    roundings: the two accumulate in different orders, so an activation close
    to a BF16 rounding boundary can round to the neighbouring value (one BF16
    ulp); such flips are rare and move a logit by far less than its scale."""
    c, z = _pairs([3000], 11)[0]
    X = M.features(c, z)
    Pb = net.bf16_parameters()
    _, (a1, a2, a3), zd = _device_forward(torch, net, X)
    A1, A2, A3, ref = M.forward(X, Pb)
    got = zd.cpu().numpy()
    scale = np.abs(ref).max()
    d = np.abs(got - ref)
    assert np.percentile(d, 99) <= LOGIT_RTOL * scale, (np.percentile(d, 99), scale)
    assert d.max() <= 1e-2 * scale
    for dev, orc in ((a1, A1), (a2, A2)):
        assert np.mean(dev != orc) < 2e-3  # BF16 values: equal unless a rounding flipped
    np.testing.assert_allclose(a3, A3, rtol=1e-2, atol=1e-2 * np.abs(A3).max())


@pytest.mark.parametrize("n", [1, 127, 128, 129, 383, 20000])
def test_forward_tile_edges(torch, net, n):
    """The forward kernel works on tiles of 128 rows (one tensor-core MMA of
    M = 128 per layer); partial tiles, single rows and more tiles than
    resident CTAs give the oracle's logits, and every row is written."""
    rng = np.random.Generator(np.random.PCG64(100 + n))
    X = np.zeros((n, 32), np.float32)
    X[:, :20] = rng.uniform(-0.5, 2.0, (n, 20)).astype(np.float32)
    _, (a1, a2, a3), zd = _device_forward(torch, net, X)
    A1, A2, A3, ref = M.forward(X, net.bf16_parameters())
    got = zd.cpu().numpy()
    assert np.isfinite(got).all()
    scale = max(np.abs(ref).max(), 1e-3)
    d = np.abs(got - ref)
    assert np.percentile(d, 99) <= LOGIT_RTOL * scale, (np.percentile(d, 99), scale)
    assert d.max() <= 1e-2 * scale
    for dev, orc in ((a1, A1), (a2, A2)):
        assert np.mean(dev != orc) < 2e-3
    # logits without the activation outputs equal those with them
    d_x = torch.from_numpy(X).cuda()
    z2 = torch.empty(n, dtype=torch.float32, device="cuda")
    import ctypes
    assert net.lib.gcr_learned_forward(ctypes.c_void_p(d_x.data_ptr()), n, ctypes.c_void_p(net.bf16.data_ptr()),
                                       None, None, None, ctypes.c_void_p(z2.data_ptr()), None) == 0
    assert np.array_equal(z2.cpu().numpy(), got)


def test_backward_matches_oracle(torch, net):
    """Gradient of the device backward pass vs the FP64 restatement on the
    device forward's own layer inputs (so only the backward arithmetic is
    compared)."""
    c, z = _pairs([1000], 12)[0]
    X = M.features(c, z)
    rng = np.random.Generator(np.random.PCG64(5))
    y = (rng.uniform(size=len(X)) < 0.3).astype(np.float32)
    w = np.where(y > 0, 2.5, 1.0).astype(np.float32)
    loss, G = net.loss_and_grad(torch.from_numpy(X).cuda(), torch.from_numpy(y).cuda(), torch.from_numpy(w).cuda())
    G = G.cpu().numpy().astype(np.float64)
    _, (a1, a2, a3), zd = _device_forward(torch, net, X)
    loss_ref, G_ref = M.grad_from(M.bf16_round(X), a1, a2, a3, zd.cpu().numpy(), net.bf16_parameters(),
                                  y.astype(np.float64), w.astype(np.float64))
    assert abs(loss - loss_ref) <= 1e-5 * max(1.0, abs(loss_ref))
    for name, a, b in [("W1", "W1", "b1"), ("b1", "b1", "W2"), ("W2", "W2", "b2"), ("b2", "b2", "W3"),
                       ("W3", "W3", "b3"), ("b3", "b3", "W4"), ("W4", "W4", "b4")]:
        g, r = G[M.OFF[a]:M.OFF[b]], G_ref[M.OFF[a]:M.OFF[b]]
        err = np.linalg.norm(g - r) / max(np.linalg.norm(r), 1e-30)
        assert err < GRAD_RTOL, f"{name}: relative error {err:.2e}"
    assert abs(G[M.OFF["b4"]] - G_ref[M.OFF["b4"]]) <= GRAD_RTOL * max(1e-6, abs(G_ref[M.OFF["b4"]]))


def test_adam_step_matches_oracle(torch):
    from pygcransac.learned import LearnedProposal
    a = LearnedProposal(seed=9)
    P0 = a.parameters().astype(np.float64)
    rng = np.random.Generator(np.random.PCG64(2))
    m = v = np.zeros_like(P0)
    P = P0
    for step in (1, 2, 3):
        g = rng.normal(scale=1e-2, size=len(P0)).astype(np.float32)
        a.grad.copy_(torch.from_numpy(g))
        a.adam(1e-3)
        m, v, P = M.adam(m, v, P, g.astype(np.float64), 1e-3, step)
    got = a.parameters().astype(np.float64)
    np.testing.assert_allclose(got, P, rtol=0, atol=2e-6)
    np.testing.assert_array_equal(a.bf16_parameters(), M.bf16_round(got.astype(np.float32)))


def test_order_and_unpermute_exact(torch, net):
    lib = _abi.load()
    from pygcransac.learned import layout
    rng = np.random.Generator(np.random.PCG64(4))
    lens = [5, 1, 3000, 257, 64, 8500]  # the last uses the counting kernel, the others the bitonic sort
    corr = [rng.uniform(0, 640, (n, 4)) for n in lens]
    offsets, max_n, por = layout(lens)
    z = np.round(rng.normal(size=int(offsets[-1])), 1).astype(np.float32)  # many ties
    z[[3, 10, 400, 4000]] = np.nan
    z[[11, 12, 4001]] = -np.inf
    z[[13, 14]] = [0.0, -0.0]
    d_corr = torch.from_numpy(np.concatenate(corr)).cuda()
    d_off = torch.from_numpy(offsets).cuda()
    d_z = torch.from_numpy(z).cuda()
    d_sorted = torch.empty_like(d_corr)
    d_perm = torch.empty(int(offsets[-1]), dtype=torch.int32, device="cuda")
    P = _abi.ptr
    import ctypes
    vp = lambda t: ctypes.c_void_p(t.data_ptr())  # noqa: E731
    assert lib.gcr_learned_order(vp(d_corr), vp(d_off), len(lens), max_n, vp(d_z), vp(d_sorted), vp(d_perm),
                                 None) == 0, _abi.last_error()
    perm = d_perm.cpu().numpy()
    srt = d_sorted.cpu().numpy()
    mask_sorted = (rng.uniform(size=int(offsets[-1])) < 0.4).astype(np.uint8)
    d_ms = torch.from_numpy(mask_sorted).cuda()
    d_por = torch.from_numpy(por).cuda()
    d_mask = torch.zeros_like(d_ms)
    assert lib.gcr_learned_unpermute_mask(vp(d_ms), vp(d_perm), vp(d_off), vp(d_por), int(offsets[-1]), vp(d_mask),
                                          None) == 0, _abi.last_error()
    mask = d_mask.cpu().numpy()
    for i in range(len(lens)):
        o0, o1 = offsets[i], offsets[i + 1]
        ref = M.order(z[o0:o1])
        np.testing.assert_array_equal(perm[o0:o1], ref)
        np.testing.assert_array_equal(srt[o0:o1], corr[i][ref])
        back = np.zeros(o1 - o0, np.uint8)
        back[ref] = mask_sorted[o0:o1]
        np.testing.assert_array_equal(mask[o0:o1], back)
    del P


def f_params(max_iters, sampler=0, seed=0):
    return _abi.Params(threshold=0.75, confidence=0.99, spatial_coherence_weight=0.975, neighborhood_size=8,
                       max_iterations=max_iters, min_iterations=min(50, max_iters), sampler=sampler, neighborhood=0,
                       lo_number=50, seed=seed)


def test_learned_batch_equals_engine_on_same_order(torch, net, gcr):
    """The device pipeline (order -> PROSAC -> mask back) is the plain engine
    run on the learned order: models and masks bit-identical."""
    from pygcransac.learned import find_batch_learned
    prs = [S.two_view_pair(40 + k, n=n, inlier_ratio=r) for k, (n, r) in enumerate([(900, 0.2), (1500, 0.08),
                                                                                       (400, 0.5)])]
    corr = [p["corr"] for p in prs]
    sizes = [p["size"] for p in prs]
    p = f_params(300, sampler=1)
    models, masks, stats = find_batch_learned(_abi.GCR_FUNDAMENTAL, corr, sizes, p, net, seeds=[7, 8, 9])
    probs = net.predict(corr, sizes)
    for i in range(len(prs)):
        # the device sorts on the FP32 logits; sigmoid is monotone, so the
        # probabilities give the same order except where it rounds two logits to one value
        z = net.logits(net.host_features([corr[i]], [sizes[i]])[0]).cpu().numpy()
        order = M.order(z)
        assert np.all(np.diff(probs[i][order]) <= 0)
        m2, k2, s2 = gcr.find_batch(_abi.GCR_FUNDAMENTAL, [corr[i][order]], [sizes[i]], p, seeds=[7 + i])
        assert stats["status"][i] == s2["status"][0]
        back = np.zeros(len(order), bool)
        back[order] = k2[0]
        np.testing.assert_array_equal(masks[i], back)
        np.testing.assert_array_equal(models[i], m2[0])


def test_trained_network_beats_uniform_sampler(torch, gcr):
    """Trained on plain-method masks of 15-50 % inlier scenes, the network's
    order lets PROSAC reach a lower median F error on unseen 5-10 % inlier
    pairs than the plain uniform sampler with the same iteration budget, and its
    top-ranked correspondences are mostly inliers."""
    from pygcransac.learned import LearnedProposal, find_batch_learned
    from pygcransac.train_proposal import label
    n = 4000
    rng = np.random.Generator(np.random.PCG64(77))
    train = [S.two_view_pair(900000 + k, n=n, inlier_ratio=float(rng.uniform(0.15, 0.5))) for k in range(48)]
    corr = [p["corr"] for p in train]
    sizes = np.array([p["size"] for p in train])
    masks, ok = label(corr, sizes, 0)
    assert ok.mean() > 0.9
    net = LearnedProposal(seed=1)
    feat, _ = net.host_features(corr, sizes)
    y = torch.from_numpy(np.concatenate(masks).astype(np.float32)).cuda()
    hist = net.train_rows(feat, y, epochs=8, lr=2e-3, batch_rows=4096)
    assert np.mean(hist[-10:]) < 0.8 * np.mean(hist[:3])

    test = [S.two_view_pair(950000 + k, n=n, inlier_ratio=float(rng.uniform(0.05, 0.10))) for k in range(24)]
    tc = [p["corr"] for p in test]
    ts = [p["size"] for p in test]
    probs = net.predict(tc, ts)
    prec = [p["inlier_gt"][np.argsort(-q, kind="stable")[:50]].mean() for p, q in zip(test, probs)]
    base = np.mean([p["inlier_gt"].mean() for p in test])
    assert np.median(prec) > 4 * base, (np.median(prec), base)

    budget = 200
    m_l, _, _ = find_batch_learned(_abi.GCR_FUNDAMENTAL, tc, ts, f_params(budget, 1), net)
    m_u, _, _ = gcr.find_batch(_abi.GCR_FUNDAMENTAL, tc, ts, f_params(budget, 0))
    e_l = np.median([S.fundamental_error(m, p, n=200) for m, p in zip(m_l, test)])
    e_u = np.median([S.fundamental_error(m, p, n=200) for m, p in zip(m_u, test)])
    assert e_l < 0.5 * e_u, (e_l, e_u)
