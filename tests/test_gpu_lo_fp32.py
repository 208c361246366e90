"""The FP32 fits (gcr_context_set_lo_precision(GCR_LO_FP32)): every
fundamental-matrix fit after the minimal solver (local-optimisation trials,
iteratively reweighted fits, final refit, the drivers' bundle adjustment) in
FP32.
It is a throughput mode, judged on model error rather than mask parity:

* on hard pairs (4000 correspondences, 5-10 % inliers, the learned proposal's
  workload) the learned form's median model error with FP32 fits is within 5 %
  (or 0.05 px) of the FP64 fits' and every pair still ends with a model;
* on easier pairs run by the plain form, the median model error matches the
  FP64 run's and no pair loses more than 2 % of the FP64 run's inliers (the
  FP32 iteratively reweighted fits may converge to a larger consensus);
* GCR_LO_FP64 stays the default and keeps the oracle's results.
"""
import ctypes
import os

import numpy as np
import pytest

from pygcransac import _abi, synthetic as S

pytestmark = pytest.mark.gpu

CKPT = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "graph-cut-ransac_gb300",
                    "pygcransac", "weights", "proposal_fundamental.gcrl")


def f_params(iters, sampler=0):
    return _abi.Params(threshold=0.75, confidence=0.99, spatial_coherence_weight=0.975, neighborhood_size=8,
                       max_iterations=iters, min_iterations=min(50, iters), sampler=sampler, neighborhood=0,
                       lo_number=50, seed=0)


def test_fp32_lo_keeps_the_learned_forms_error():
    pytest.importorskip("torch")
    from pygcransac.learned import LearnedProposal, find_batch_learned
    net = LearnedProposal.load(CKPT)
    rng = np.random.default_rng(8)
    pairs = [S.two_view_pair(20000 + i, n=4000, inlier_ratio=float(rng.uniform(0.05, 0.10))) for i in range(96)]
    corr = [q["corr"] for q in pairs]
    sizes = [q["size"] for q in pairs]
    seeds = np.arange(96, dtype=np.uint64) + np.uint64(3)
    out = {}
    for prec in (_abi.GCR_LO_FP64, _abi.GCR_LO_FP32):
        models, masks, stats = find_batch_learned(_abi.GCR_FUNDAMENTAL, corr, sizes, f_params(50, 1), net, seeds=seeds,
                                                  lo_precision=prec)
        err = [S.fundamental_error(m, q, n=100) for m, q in zip(models, pairs)]
        out[prec] = (float(np.median(err)), stats)
    e64, st64 = out[_abi.GCR_LO_FP64]
    e32, st32 = out[_abi.GCR_LO_FP32]
    assert np.all(st32["status"] == 0) and np.all(st64["status"] == 0)
    assert e32 <= e64 * 1.05 or e32 <= e64 + 0.05, (e32, e64)


def test_fp32_lo_models_agree_on_plain_runs(gcr):
    lib = _abi.load()
    import torch
    pairs = [S.two_view_pair(21000 + i, n=1500, inlier_ratio=0.3) for i in range(24)]
    corr = np.ascontiguousarray(np.concatenate([q["corr"] for q in pairs]))
    off = np.zeros(len(pairs) + 1, np.int64)
    off[1:] = np.cumsum([len(q["corr"]) for q in pairs])
    sz = np.zeros(len(pairs), _abi.SIZE_DTYPE)
    for i, q in enumerate(pairs):
        sz[i] = q["size"]
    P = len(pairs)
    seeds = np.arange(P, dtype=np.uint64) + np.uint64(7)
    d_corr = torch.from_numpy(corr).cuda()
    vp = lambda t: ctypes.c_void_p(t.data_ptr())  # noqa: E731
    res = {}
    for prec in (None, _abi.GCR_LO_FP64, _abi.GCR_LO_FP32):
        ctx = ctypes.c_void_p()
        assert lib.gcr_context_create(ctypes.byref(ctx)) == 0
        pm = torch.zeros(P * 9, dtype=torch.float64, device="cuda")
        pk = torch.zeros(len(corr), dtype=torch.uint8, device="cuda")
        ps = torch.zeros(P * _abi.STATS_DTYPE.itemsize, dtype=torch.uint8, device="cuda")
        try:
            if prec is not None:
                assert lib.gcr_context_set_lo_precision(ctx, prec) == 0
            p = f_params(2000)
            rc = lib.gcr_batch_run_device(ctx, _abi.GCR_FUNDAMENTAL, P, vp(d_corr), _abi.ptr(off), None, _abi.ptr(sz),
                                          ctypes.byref(p), _abi.ptr(seeds), vp(pm), vp(pk), vp(ps), None)
            assert rc == 0, _abi.last_error()
            torch.cuda.synchronize()
        finally:
            lib.gcr_context_destroy(ctx)
        res[prec] = (pm.cpu().numpy().reshape(P, 3, 3), pk.cpu().numpy(),
                     np.frombuffer(ps.cpu().numpy().tobytes(), _abi.STATS_DTYPE))
    # the default is the FP64 arithmetic
    assert np.array_equal(res[None][1], res[_abi.GCR_LO_FP64][1])
    assert np.array_equal(res[None][2], res[_abi.GCR_LO_FP64][2])
    m64, k64, s64 = res[_abi.GCR_LO_FP64]
    m32, k32, s32 = res[_abi.GCR_LO_FP32]
    assert np.all(s32["status"] == 0)
    e64 = np.array([S.fundamental_error(m, q, n=200) for m, q in zip(m64, pairs)])
    e32 = np.array([S.fundamental_error(m, q, n=200) for m, q in zip(m32, pairs)])
    assert np.median(e32) <= np.median(e64) * 1.05 + 0.02, (np.median(e32), np.median(e64))
    assert np.all(s32["inlier_number"] >= s64["inlier_number"] - np.maximum(2, 0.02 * s64["inlier_number"]))
    assert lib.gcr_context_set_lo_precision(None, 1) == _abi.GCR_INVALID_ARG
