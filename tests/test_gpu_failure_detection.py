"""Failure detection without a GPU fault.

* A runaway flow: the labelling's maximum-flow step limit set tiny through
  gcr_context_set_flow_step_limit makes the flow solvers stop; the pair
  reports GCR_TIMEOUT, the kernel returns, every pair's outputs are written,
  and the same context runs the same batch to the untouched result once the
  limit is restored. Grid cells (warp solver) and the radius graph.
* Bad input injected on the host: a pair with a NaN or an infinite coordinate
  reports GCR_INVALID_ARG and is not run while the other pairs of its batch
  run unchanged; a pair whose correspondences all coincide and an essential
  pair with singular intrinsics end with a status, never a device fault.
"""
import ctypes

import numpy as np
import pytest

from pygcransac import _abi, synthetic as S

pytestmark = pytest.mark.gpu


def batch_arrays(pairs, K=None):
    corr = np.ascontiguousarray(np.concatenate([q["corr"] for q in pairs]), np.float64)
    off = np.zeros(len(pairs) + 1, np.int64)
    off[1:] = np.cumsum([len(q["corr"]) for q in pairs])
    sz = np.zeros(len(pairs), _abi.SIZE_DTYPE)
    for i, q in enumerate(pairs):
        sz[i] = q["size"]
    return corr, off, sz


def run_device(lib, ctx, kind, pairs, p, seeds, K=None):
    torch = pytest.importorskip("torch")
    corr, off, sz = batch_arrays(pairs)
    P = len(pairs)
    d_corr = torch.from_numpy(corr).cuda()
    pm = torch.full((P * 9,), -7.0, dtype=torch.float64, device="cuda")
    pk = torch.full((len(corr),), 9, dtype=torch.uint8, device="cuda")
    ps = torch.full((P * _abi.STATS_DTYPE.itemsize,), 0xAB, dtype=torch.uint8, device="cuda")
    ptr = lambda t: ctypes.c_void_p(t.data_ptr())  # noqa: E731
    rc = lib.gcr_batch_run_device(ctx, kind, P, ptr(d_corr), _abi.ptr(off), _abi.ptr(K), _abi.ptr(sz),
                                  ctypes.byref(p), _abi.ptr(seeds), ptr(pm), ptr(pk), ptr(ps), None)
    assert rc == _abi.GCR_OK, _abi.last_error()
    torch.cuda.synchronize()
    stats = np.frombuffer(ps.cpu().numpy().tobytes(), _abi.STATS_DTYPE)
    return pm.cpu().numpy().reshape(P, 3, 3), pk.cpu().numpy(), stats


def h_params(**kw):
    base = dict(threshold=3.0, confidence=0.99, spatial_coherence_weight=0.975, neighborhood_size=4,
                max_iterations=2000, min_iterations=50, sampler=0, neighborhood=0, lo_number=20, seed=0)
    base.update(kw)
    return _abi.Params(**base)


@pytest.mark.parametrize("graph", ["grid", "radius"])
def test_flow_step_limit_reports_timeout_and_context_recovers(graph):
    lib = _abi.load()
    if graph == "grid":
        kind = _abi.GCR_HOMOGRAPHY
        pairs = [S.homography_pair(60 + i, n=1500, inlier_ratio=0.5) for i in range(4)]
        p = h_params()  # a 4^4 grid: cells of a few to a few dozen points
    else:
        kind = _abi.GCR_FUNDAMENTAL
        pairs = [S.two_view_pair(70 + i, n=900, inlier_ratio=0.5) for i in range(3)]
        p = h_params(threshold=0.75, neighborhood=1, neighborhood_size=20.0, spatial_coherence_weight=0.975)
    seeds = np.arange(len(pairs), dtype=np.uint64) + np.uint64(3)
    ctx = ctypes.c_void_p()
    assert lib.gcr_context_create(ctypes.byref(ctx)) == 0
    try:
        _, mask0, st0 = run_device(lib, ctx, kind, pairs, p, seeds)
        assert np.all(st0["status"] == 0)
        assert lib.gcr_context_set_flow_step_limit(ctx, -1) == _abi.GCR_INVALID_ARG
        # one step: a flow that needs a second push or relabel anywhere stops
        assert lib.gcr_context_set_flow_step_limit(ctx, 1) == _abi.GCR_OK
        models, mask, st = run_device(lib, ctx, kind, pairs, p, seeds)
        assert np.all(st["status"] == _abi.GCR_TIMEOUT), st["status"]
        assert np.all(st["graph_cut_number"] >= 1)
        assert set(np.unique(mask)) <= {0, 1}  # every mask byte written
        assert np.all(np.isfinite(models))
        assert lib.gcr_context_set_flow_step_limit(ctx, 0) == _abi.GCR_OK
        _, mask1, st1 = run_device(lib, ctx, kind, pairs, p, seeds)
        assert np.array_equal(st1, st0) and np.array_equal(mask1, mask0)
    finally:
        lib.gcr_context_destroy(ctx)


def test_non_finite_coordinates_are_rejected_per_pair(gcr):
    lib = _abi.load()
    pairs = [S.homography_pair(80 + i, n=800) for i in range(4)]
    pairs[1]["corr"] = pairs[1]["corr"].copy()
    pairs[1]["corr"][17, 2] = np.nan
    pairs[3]["corr"] = pairs[3]["corr"].copy()
    pairs[3]["corr"][0, 0] = np.inf
    p = h_params(neighborhood_size=4)
    seeds = np.arange(4, dtype=np.uint64) + np.uint64(1)
    ctx = ctypes.c_void_p()
    assert lib.gcr_context_create(ctypes.byref(ctx)) == 0
    try:
        models, mask, st = run_device(lib, ctx, _abi.GCR_HOMOGRAPHY, pairs, p, seeds)
    finally:
        lib.gcr_context_destroy(ctx)
    assert list(st["status"]) == [0, _abi.GCR_INVALID_ARG, 0, _abi.GCR_INVALID_ARG]
    _, off, _ = batch_arrays(pairs)
    for i in (1, 3):
        assert not mask[off[i]:off[i + 1]].any()
        assert not models[i].any()
        assert st["iteration_number"][i] == 0
    # the clean pairs are untouched by their neighbours
    for i in (0, 2):
        m1, k1, s1 = gcr.find_batch(_abi.GCR_HOMOGRAPHY, [pairs[i]["corr"]], [pairs[i]["size"]], p, seeds=[seeds[i]])
        assert s1["status"][0] == 0 and np.array_equal(k1[0], mask[off[i]:off[i + 1]].astype(bool))
    # the single-pair entry returns the status; the Python entry raises ValueError
    with pytest.raises(ValueError):
        gcr.findHomography(pairs[1]["corr"], 480, 640, 480, 640, None, threshold=3.0)


def test_degenerate_inputs_end_with_a_status(gcr):
    # every correspondence the same point: no minimal sample is usable
    same = np.tile(np.array([[100.0, 120.0, 130.0, 90.0]]), (300, 1))
    for kind in (_abi.GCR_HOMOGRAPHY, _abi.GCR_FUNDAMENTAL):
        p = h_params(threshold=1.0, max_iterations=500)
        models, masks, st = gcr.find_batch(kind, [same], [(480, 640, 480, 640)], p, seeds=[5])
        assert st["status"][0] in (_abi.GCR_OK, _abi.GCR_NO_MODEL, _abi.GCR_CAPACITY), st["status"][0]
        if st["status"][0] == _abi.GCR_NO_MODEL:
            assert not masks[0].any()
    K = np.array([[800.0, 0, 320], [0, 800.0, 240], [0, 0, 1]])
    Ks = np.array([[800.0, 0, 320], [1600.0, 0, 640], [0, 0, 1]])  # rank 2
    pr = S.two_view_pair(90, n=500, inlier_ratio=0.5)
    with pytest.raises(ValueError):
        gcr.findEssentialMatrix(pr["corr"], K, Ks, 480, 640, 480, 640, None, threshold=0.75)
    E, mask = gcr.findEssentialMatrix(pr["corr"], K, K, 480, 640, 480, 640, None, threshold=0.75)
    assert E is not None and mask.sum() > 100
