"""GPU test of the prepared batch launch recorded into a CUDA graph:
gcr_batch_prepare + gcr_batch_launch captured with torch.cuda.graph and
replayed must give the results of gcr_batch_run_device, also after new
correspondences are written into the same device buffer."""
import ctypes

import numpy as np
import pytest

from pygcransac import _abi, synthetic as S

pytestmark = pytest.mark.gpu


def run_kind(kind, pairs, p, K=None):
    torch = pytest.importorskip("torch")
    lib = _abi.load()
    corr = np.concatenate([pr["corr"] for pr in pairs])
    offsets = np.zeros(len(pairs) + 1, np.int64)
    offsets[1:] = np.cumsum([len(pr["corr"]) for pr in pairs])
    sizes = np.zeros(len(pairs), _abi.SIZE_DTYPE)
    for i, pr in enumerate(pairs):
        sizes[i] = pr["size"]
    P = len(pairs)
    seeds = np.arange(P, dtype=np.uint64) + np.uint64(5)
    d_corr = torch.from_numpy(np.ascontiguousarray(corr)).cuda()
    outs = []
    for _ in range(2):
        outs.append((torch.zeros(P * 9, dtype=torch.float64, device="cuda"),
                     torch.zeros(len(corr), dtype=torch.uint8, device="cuda"),
                     torch.zeros(P * _abi.STATS_DTYPE.itemsize, dtype=torch.uint8, device="cuda")))
    ctx = ctypes.c_void_p()
    assert lib.gcr_context_create(ctypes.byref(ctx)) == 0
    ptr = lambda t: ctypes.c_void_p(t.data_ptr())  # noqa: E731
    Kp = _abi.ptr(K)
    # reference: the one-call form
    rc = lib.gcr_batch_run_device(ctx, kind, P, ptr(d_corr), _abi.ptr(offsets), Kp, _abi.ptr(sizes),
                                  ctypes.byref(p), _abi.ptr(seeds), ptr(outs[0][0]), ptr(outs[0][1]),
                                  ptr(outs[0][2]), ctypes.c_void_p(torch.cuda.current_stream().cuda_stream))
    assert rc == 0, _abi.last_error()
    torch.cuda.synchronize()
    # prepared + captured
    rc = lib.gcr_batch_prepare(ctx, kind, P, ptr(d_corr), _abi.ptr(offsets), Kp, _abi.ptr(sizes), ctypes.byref(p),
                               _abi.ptr(seeds), ptr(outs[1][0]), ptr(outs[1][1]), ptr(outs[1][2]))
    assert rc == 0, _abi.last_error()
    g = torch.cuda.CUDAGraph()
    s = torch.cuda.Stream()
    with torch.cuda.stream(s):
        with torch.cuda.graph(g, stream=s):
            rc = lib.gcr_batch_launch(ctx, ctypes.c_void_p(s.cuda_stream))
    assert rc == 0, _abi.last_error()
    for _ in range(2):
        outs[1][2].zero_()
        g.replay()
        torch.cuda.synchronize()
        assert torch.equal(outs[0][1], outs[1][1])
        assert torch.equal(outs[0][2], outs[1][2])
        assert torch.allclose(outs[0][0], outs[1][0], rtol=0, atol=1e-12)
    # new correspondences in the same buffer: the replay follows them
    d_corr.copy_(torch.from_numpy(np.ascontiguousarray(corr[::-1].copy())))
    g.replay()
    torch.cuda.synchronize()
    assert not torch.equal(outs[0][1], outs[1][1])
    lib.gcr_context_destroy(ctx)


def test_graph_replay_homography():
    pairs = [S.homography_pair(s, n=1000 + 200 * s) for s in range(6)]
    p = _abi.Params(threshold=3.0, confidence=0.99, spatial_coherence_weight=0.975, neighborhood_size=4,
                    max_iterations=2000, min_iterations=50, sampler=0, neighborhood=0, lo_number=50, seed=0)
    run_kind(_abi.GCR_HOMOGRAPHY, pairs, p)


def test_graph_replay_essential():
    pairs = [S.two_view_pair(s, n=600 + 100 * s, inlier_ratio=0.5) for s in range(4)]
    K = np.stack([np.concatenate([pr["K"].ravel(), pr["K"].ravel()]) for pr in pairs])
    p = _abi.Params(threshold=0.75, confidence=0.99, spatial_coherence_weight=0.1, neighborhood_size=8,
                    max_iterations=500, min_iterations=50, sampler=0, neighborhood=0, lo_number=20, seed=0,
                    scoring=_abi.GCR_SCORING_MAGSAC)
    run_kind(_abi.GCR_ESSENTIAL, pairs, p, K=K)


def test_pair_times_stamp_every_pair():
    """gcr_context_set_pair_times: every pair of a batch gets a start and an
    end stamp from the GPU's global timer, end >= start, and the results are
    those of a run without stamps."""
    import ctypes

    import numpy as np
    import torch

    from pygcransac import _abi, synthetic as S
    lib = _abi.load()
    prs = [S.homography_pair(60 + k, n=500 + 100 * k) for k in range(5)]
    corr = np.ascontiguousarray(np.concatenate([p["corr"] for p in prs]))
    offsets = np.zeros(6, np.int64)
    offsets[1:] = np.cumsum([len(p["corr"]) for p in prs])
    sizes = np.zeros(5, _abi.SIZE_DTYPE)
    for i, p in enumerate(prs):
        sizes[i] = tuple(p["size"])
    prm = _abi.Params(threshold=3.0, confidence=0.99, spatial_coherence_weight=0.975, neighborhood_size=4,
                      max_iterations=1000, min_iterations=50, sampler=0, neighborhood=0, lo_number=50, seed=0)
    vp = lambda t: ctypes.c_void_p(t.data_ptr())  # noqa: E731
    d_corr = torch.from_numpy(corr).cuda()
    outs = []
    for stamped in (False, True):
        d_models = torch.zeros(45, dtype=torch.float64, device="cuda")
        d_masks = torch.zeros(int(offsets[-1]), dtype=torch.uint8, device="cuda")
        d_stats = torch.zeros(5 * _abi.STATS_DTYPE.itemsize, dtype=torch.uint8, device="cuda")
        times = torch.zeros(10, dtype=torch.int64, device="cuda")
        ctx = ctypes.c_void_p()
        assert lib.gcr_context_create(ctypes.byref(ctx)) == 0
        try:
            if stamped:
                assert lib.gcr_context_set_pair_times(ctx, vp(times)) == 0
            assert lib.gcr_batch_run_device(ctx, _abi.GCR_HOMOGRAPHY, 5, vp(d_corr), _abi.ptr(offsets), None,
                                            _abi.ptr(sizes), ctypes.byref(prm), None, vp(d_models), vp(d_masks),
                                            vp(d_stats), None) == 0, _abi.last_error()
            torch.cuda.synchronize()
        finally:
            lib.gcr_context_destroy(ctx)
        outs.append((d_models.cpu().numpy(), d_masks.cpu().numpy(), times.cpu().numpy().reshape(5, 2)))
    (m0, k0, t0), (m1, k1, t1) = outs
    assert np.array_equal(m0, m1) and np.array_equal(k0, k1)
    assert np.all(t0 == 0)
    assert np.all(t1 > 0) and np.all(t1[:, 1] >= t1[:, 0])


def test_non_positive_image_sizes_are_rejected(gcr):
    pr = S.homography_pair(3, n=300)
    p = gcr.default_params(_abi.GCR_HOMOGRAPHY)
    for bad in [(0, 640, 480, 640), (480, -1, 480, 640), (480, 640, 480, 0)]:
        with pytest.raises(ValueError, match="image sizes must be positive"):
            gcr.find_batch(_abi.GCR_HOMOGRAPHY, [pr["corr"]], [bad], p, seeds=[1])


def test_context_destroy_releases_every_scratch_buffer():
    """Create / run / destroy with the radius graph and the AR sampler (their
    per-CTA scratch is the largest) several times: free device memory returns
    to where it started."""
    torch = pytest.importorskip("torch")
    lib = _abi.load()
    pr = S.two_view_pair(41, n=1500, inlier_ratio=0.4)
    corr = np.ascontiguousarray(pr["corr"])
    n = len(corr)
    offsets = np.array([0, n], np.int64)
    sizes = np.zeros(1, _abi.SIZE_DTYPE)
    sizes[0] = tuple(pr["size"])
    prm = _abi.Params(threshold=0.75, confidence=0.99, spatial_coherence_weight=0.975, neighborhood_size=20.0,
                      max_iterations=300, min_iterations=50, sampler=_abi.GCR_SAMPLER_AR, neighborhood=1,
                      lo_number=50, seed=0, sampler_variance=0.1)
    vp = lambda t: ctypes.c_void_p(t.data_ptr())  # noqa: E731
    d_corr = torch.from_numpy(corr).cuda()
    d_prob = torch.from_numpy(0.1 + pr["inlier_gt"].astype(np.float64)).cuda()
    d_models = torch.zeros(9, dtype=torch.float64, device="cuda")
    d_masks = torch.zeros(n, dtype=torch.uint8, device="cuda")
    d_stats = torch.zeros(_abi.STATS_DTYPE.itemsize, dtype=torch.uint8, device="cuda")
    torch.cuda.synchronize()

    def cycle():
        ctx = ctypes.c_void_p()
        assert lib.gcr_context_create(ctypes.byref(ctx)) == 0
        try:
            assert lib.gcr_context_set_probabilities(ctx, vp(d_prob)) == 0
            assert lib.gcr_batch_run_device(ctx, _abi.GCR_FUNDAMENTAL, 1, vp(d_corr), _abi.ptr(offsets), None,
                                            _abi.ptr(sizes), ctypes.byref(prm), None, vp(d_models), vp(d_masks),
                                            vp(d_stats), None) == 0, _abi.last_error()
            torch.cuda.synchronize()
        finally:
            assert lib.gcr_context_destroy(ctx) == 0

    cycle()  # first use: module loading and the runtime's own allocations
    free0 = torch.cuda.mem_get_info()[0]
    for _ in range(3):
        cycle()
    free1 = torch.cuda.mem_get_info()[0]
    assert free0 - free1 < (64 << 20), f"{(free0 - free1) >> 20} MiB not returned"
