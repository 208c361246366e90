"""GPU test of the launch-shape autotuner: every candidate shape (hypotheses
per batch 64 / 128 / 256, one or two CTAs per SM, caller's or largest-first
pair order) gives bit-identical masks, statistics and models on a ragged
calibration batch (autotune.tune raises otherwise); the fastest shape,
recorded in a cache and installed on a context, is the one
gcr_batch_prepare selects, and the tuned run equals the oracle (a pair on a
rounding-level tie equals the oracle's FMA-contracted build)."""
import ctypes

import numpy as np
import pytest

from pygcransac import _abi, autotune as A, synthetic as S

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("kind,sampler", [(_abi.GCR_FUNDAMENTAL, 1), (_abi.GCR_HOMOGRAPHY, 2),
                                          (_abi.GCR_ESSENTIAL, 0)])
def test_shapes_agree_and_tuned_run_matches_oracle(batch_parity, kind, sampler, tmp_path):
    torch = pytest.importorskip("torch")
    rng = np.random.default_rng(5)
    P = 40
    ns = np.exp(rng.uniform(np.log(300), np.log(5000), P)).astype(int)
    if kind == _abi.GCR_HOMOGRAPHY:
        pairs = [S.homography_pair(500 + i, n=int(ns[i]), inlier_ratio=0.4) for i in range(P)]
        p = _abi.Params(threshold=3.0, confidence=0.99, spatial_coherence_weight=0.975, neighborhood_size=8,
                        max_iterations=2000, min_iterations=50, sampler=sampler, neighborhood=0, lo_number=20)
        K = None
    else:
        pairs = [S.two_view_pair(500 + i, n=int(ns[i]), inlier_ratio=0.4) for i in range(P)]
        p = _abi.Params(threshold=0.75, confidence=0.99, spatial_coherence_weight=0.975, neighborhood_size=8,
                        max_iterations=2000 if kind == _abi.GCR_ESSENTIAL else 300, min_iterations=50,
                        sampler=sampler, neighborhood=0, lo_number=20)
        K = None if kind != _abi.GCR_ESSENTIAL else np.stack(
            [np.concatenate([q["K"].ravel(), q["K"].ravel()]) for q in pairs])
    corr = np.ascontiguousarray(np.concatenate([q["corr"] for q in pairs]))
    off = np.zeros(P + 1, np.int64)
    off[1:] = np.cumsum([len(q["corr"]) for q in pairs])
    sizes = np.array([q["size"] for q in pairs])
    seeds = np.arange(P, dtype=np.uint64) + np.uint64(17)
    d_corr = torch.from_numpy(corr).cuda()
    best, timings = A.tune(kind, d_corr, off, sizes, p, seeds, K, repeats=1)
    assert set(timings) == set(A.CANDIDATES)
    cache = A.record({}, "this-gpu", kind, int(np.diff(off).max()), best, timings)
    path = str(tmp_path / "tuning.json")
    A.save_cache(cache, path)

    lib = _abi.load()
    ctx = ctypes.c_void_p()
    assert lib.gcr_context_create(ctypes.byref(ctx)) == 0
    try:
        rows = A.apply(ctx, gpu="this-gpu", path=path)
        assert len(rows) == 1
        sz = np.zeros(P, _abi.SIZE_DTYPE)
        sz["h1"], sz["w1"], sz["h2"], sz["w2"] = sizes[:, 0], sizes[:, 1], sizes[:, 2], sizes[:, 3]
        pm = torch.zeros(P * 9, dtype=torch.float64, device="cuda")
        pk = torch.zeros(len(corr), dtype=torch.uint8, device="cuda")
        ps = torch.zeros(P * _abi.STATS_DTYPE.itemsize, dtype=torch.uint8, device="cuda")
        vp = lambda t: ctypes.c_void_p(t.data_ptr())  # noqa: E731
        rc = lib.gcr_batch_run_device(ctx, kind, P, vp(d_corr), _abi.ptr(off), _abi.ptr(K), _abi.ptr(sz),
                                      ctypes.byref(p), _abi.ptr(seeds), vp(pm), vp(pk), vp(ps), None)
        assert rc == 0, _abi.last_error()
        torch.cuda.synchronize()
        used = A.last_tuning(ctx)
        assert (used["batch_calls"], used["ctas_per_sm"], used["order"]) == tuple(best)
    finally:
        lib.gcr_context_destroy(ctx)
    stats = np.frombuffer(ps.cpu().numpy().tobytes(), _abi.STATS_DTYPE)
    masks = pk.cpu().numpy().astype(bool)
    batch_parity(kind, corr, off, sz, p, seeds, K, stats, masks)
