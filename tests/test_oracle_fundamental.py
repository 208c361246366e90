"""CPU known-answer tests of the oracle's fundamental-matrix path."""
import numpy as np

from pygcransac import _abi, synthetic as S


def f_params(**kw):
    p = _abi.Params(threshold=0.75, confidence=0.99, spatial_coherence_weight=0.975, neighborhood_size=8,
                    max_iterations=3000, min_iterations=50, sampler=0, neighborhood=0, lo_number=50, seed=0)
    for k, v in kw.items():
        setattr(p, k, v)
    return p


def norm_f(F):
    F = F / np.linalg.norm(F)
    return F if F[2, 2] >= 0 else -F


def test_seven_point_recovers_exact_model(oracle):
    pr = S.two_view_pair(3, n=200, inlier_ratio=1.0, sigma=0.0)
    corr = pr["corr"]
    k, Fs = oracle.minimal(_abi.GCR_FUNDAMENTAL, corr, np.arange(7))
    assert k >= 1
    errs = [min(np.linalg.norm(norm_f(F) - pr["F_gt"]), np.linalg.norm(norm_f(F) + pr["F_gt"])) for F in Fs]
    assert min(errs) < 1e-6
    # every returned model satisfies the epipolar constraint on the sample
    x1 = np.c_[corr[:7, :2], np.ones(7)]
    x2 = np.c_[corr[:7, 2:], np.ones(7)]
    for F in Fs:
        assert np.abs(np.einsum("ij,jk,ik->i", x2, F, x1)).max() < 1e-6 * np.abs(F).max() * 640 * 640


def test_fundamental_exact_recovery(oracle):
    # noise-free and outlier-free: every stage must return the true model
    # (with outliers near the epipolar lines, the final weighted bundle
    # adjustment legitimately trades exactness for a higher MSAC score)
    pr = S.two_view_pair(5, n=300, inlier_ratio=1.0, sigma=0.0)
    rc, F, mask, st = oracle.find(_abi.GCR_FUNDAMENTAL, pr["corr"], oracle.make_size(*pr["size"]),
                                  f_params(threshold=0.5))
    assert rc == 0
    assert mask.all()
    assert S.fundamental_error(F, pr) < 1e-6


def test_fundamental_noisy_pair(oracle):
    pr = S.two_view_pair(1, n=1000, inlier_ratio=0.5)
    rc, F, mask, st = oracle.find(_abi.GCR_FUNDAMENTAL, pr["corr"], oracle.make_size(*pr["size"]), f_params())
    assert rc == 0
    assert (mask & pr["inlier_gt"]).sum() >= 0.95 * pr["inlier_gt"].sum()
    assert S.fundamental_error(F, pr) < 0.3
