"""GPU parity of the samplers fed by per-correspondence probabilities for the
three model kinds: the importance sampler (3, samplers/importance_sampler.h:
the same cumulative table as the oracle and the same multinomial draws from
the shared Philox streams) and the AR sampler (4, adaptive_reordering_sampler.h:
the same heap replay and jitter draws), so masks, counts and models agree.
Covers the single-pair entry points (host probabilities) and the device batch
entry (gcr_context_set_probabilities)."""
import ctypes

import numpy as np
import pytest

from pygcransac import _abi, synthetic as S

pytestmark = pytest.mark.gpu

MODEL_TOL = 1e-6


def rel_err(a, b):
    a = a / np.linalg.norm(a)
    b = b / np.linalg.norm(b)
    return min(np.linalg.norm(a - b), np.linalg.norm(a + b))


def weights(pr, seed):
    """Positive weights that favour the inliers, as a learned proposal would."""
    rng = np.random.Generator(np.random.PCG64(seed))
    return 0.05 + 0.9 * pr["inlier_gt"] * rng.uniform(0.3, 1.0, len(pr["corr"])) + rng.uniform(0, 0.1, len(pr["corr"]))


CASES = [
    ("homography", _abi.GCR_HOMOGRAPHY, 3.0, 0.975, 4),
    ("fundamental", _abi.GCR_FUNDAMENTAL, 0.75, 0.975, 8),
    ("essential", _abi.GCR_ESSENTIAL, 0.75, 0.1, 8),
]


def make(name, seed):
    if name == "homography":
        return S.homography_pair(seed, n=1500, inlier_ratio=0.3)
    return S.two_view_pair(seed, n=1500, inlier_ratio=0.3)


@pytest.mark.parametrize("sampler", [3, 4])
@pytest.mark.parametrize("case", range(3))
def test_weighted_sampler_single_pair(oracle, gcr, case, sampler):
    name, kind, thr, lam, grid = CASES[case]
    pr = make(name, 300 + case)
    prob = weights(pr, case)
    p = gcr._params(kind, thr, 0.99, lam, 2000, 50, False, sampler, 0, grid, 50, False, 11, sampler_variance=0.1)
    K = pr.get("K")
    rc, M, mask, st = oracle.find(kind, pr["corr"], oracle.make_size(*pr["size"]), p, seed=11, K1=K, K2=K,
                                  probabilities=prob)
    h1, w1, h2, w2 = pr["size"]
    kw = dict(probabilities=prob, threshold=thr, spatial_coherence_weight=lam, max_iters=2000, min_iters=50,
              use_sprt=False, sampler=sampler, neighborhood=0, neighborhood_size=grid, seed=11, return_stats=True,
              sampler_variance=0.1)
    if kind == _abi.GCR_HOMOGRAPHY:
        model, m, sd = gcr.findHomography(pr["corr"], h1, w1, h2, w2, use_space_partitioning=False, **kw)
    elif kind == _abi.GCR_FUNDAMENTAL:
        model, m, sd = gcr.findFundamentalMatrix(pr["corr"], h1, w1, h2, w2, **kw)
    else:
        model, m, sd = gcr.findEssentialMatrix(pr["corr"], K, K, h1, w1, h2, w2, **kw)
    assert np.array_equal(m, mask), f"{name}: mask differs at {np.nonzero(m != mask)[0][:10]}"
    assert (sd.iteration_number, sd.graph_cut_number, sd.local_optimization_number) == \
        (st.iteration_number, st.graph_cut_number, st.local_optimization_number)
    if rc == 0:
        assert rel_err(model, M) < MODEL_TOL


@pytest.mark.parametrize("sampler", [3, 4])
def test_weighted_sampler_device_batch(oracle, sampler):
    import torch
    lib = _abi.load()
    prs = [S.two_view_pair(400 + k, n=n, inlier_ratio=0.35) for k, n in enumerate((900, 1700))]
    probs = [weights(pr, 40 + k) for k, pr in enumerate(prs)]
    corr = np.ascontiguousarray(np.concatenate([pr["corr"] for pr in prs]))
    offsets = np.array([0, 900, 2600], np.int64)
    sizes = np.zeros(2, _abi.SIZE_DTYPE)
    for i, pr in enumerate(prs):
        sizes[i] = tuple(pr["size"])
    p = _abi.Params(threshold=0.75, confidence=0.99, spatial_coherence_weight=0.975, neighborhood_size=8,
                    max_iterations=1500, min_iterations=50, sampler=sampler, neighborhood=0, lo_number=50, seed=0,
                    sampler_variance=0.1)
    seeds = np.array([5, 6], np.uint64)
    d_corr = torch.from_numpy(corr).cuda()
    d_prob = torch.from_numpy(np.concatenate(probs)).cuda()
    d_models = torch.zeros(18, dtype=torch.float64, device="cuda")
    d_masks = torch.zeros(2600, dtype=torch.uint8, device="cuda")
    d_stats = torch.zeros(2 * _abi.STATS_DTYPE.itemsize, dtype=torch.uint8, device="cuda")
    vp = lambda t: ctypes.c_void_p(t.data_ptr())  # noqa: E731
    ctx = ctypes.c_void_p()
    assert lib.gcr_context_create(ctypes.byref(ctx)) == 0
    try:
        assert lib.gcr_context_set_probabilities(ctx, vp(d_prob)) == 0
        rc = lib.gcr_batch_run_device(ctx, _abi.GCR_FUNDAMENTAL, 2, vp(d_corr), _abi.ptr(offsets), None,
                                      _abi.ptr(sizes), ctypes.byref(p), _abi.ptr(seeds), vp(d_models), vp(d_masks),
                                      vp(d_stats), None)
        assert rc == 0, _abi.last_error()
        torch.cuda.synchronize()
    finally:
        lib.gcr_context_destroy(ctx)
    models = d_models.cpu().numpy().reshape(2, 3, 3)
    masks = d_masks.cpu().numpy().astype(bool)
    stats = np.frombuffer(d_stats.cpu().numpy().tobytes(), _abi.STATS_DTYPE)
    for i, pr in enumerate(prs):
        rc, M, mask, st = oracle.find(_abi.GCR_FUNDAMENTAL, pr["corr"], oracle.make_size(*pr["size"]), p,
                                      seed=int(seeds[i]), probabilities=probs[i])
        assert stats["status"][i] == rc
        assert np.array_equal(masks[offsets[i]:offsets[i + 1]], mask)
        assert stats["iteration_number"][i] == st.iteration_number
        if rc == 0:
            assert rel_err(models[i], M) < MODEL_TOL
