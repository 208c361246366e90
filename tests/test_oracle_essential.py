"""CPU known-answer tests of the oracle's essential-matrix path: the Sturm
root isolation, the Nister minimal solver, the Stewenius non-minimal solver
and the findEssentialMatrix driver on exact and noisy synthetic pairs."""
import numpy as np
import pytest

from pygcransac import _abi, synthetic as S


def e_params(**kw):
    p = _abi.Params(threshold=0.75, confidence=0.99, spatial_coherence_weight=0.1, neighborhood_size=8,
                    max_iterations=1000, min_iterations=50, sampler=0, neighborhood=0, lo_number=50, seed=0)
    for k, v in kw.items():
        setattr(p, k, v)
    return p


def normalised(pr):
    Ki = np.linalg.inv(pr["K"])
    c = pr["corr"]
    x1 = np.c_[c[:, :2], np.ones(len(c))] @ Ki.T
    x2 = np.c_[c[:, 2:], np.ones(len(c))] @ Ki.T
    return np.c_[x1[:, :2], x2[:, :2]]


def e_dist(E, E_gt):
    E = E / np.linalg.norm(E)
    return min(np.linalg.norm(E - E_gt), np.linalg.norm(E + E_gt))


def test_sturm_finds_known_roots(oracle):
    # six real roots and two complex pairs: degree 10
    roots = np.array([-2.5, -1.0, -0.3, 0.2, 0.7, 1.9])
    p = np.poly1d(np.poly(roots)) * np.poly1d([1.0, 0.0, 1.0]) * np.poly1d([1.0, 0.4, 2.0])
    assert p.order == 10
    got = oracle.sturm10(p.coeffs[::-1])
    np.testing.assert_allclose(got, roots, atol=1e-8)


def test_sturm_degree10_real_roots(oracle):
    roots = np.array([-3.1, -2.2, -1.4, -0.9, -0.2, 0.1, 0.55, 1.3, 2.4, 4.0])
    coeffs = np.poly(roots)[::-1] * 3.7
    got = oracle.sturm10(coeffs)
    np.testing.assert_allclose(got, roots, atol=1e-8)


@pytest.mark.parametrize("seed", [3, 4, 5])
def test_nister_recovers_exact_model(oracle, seed):
    pr = S.two_view_pair(seed, n=100, inlier_ratio=1.0, sigma=0.0)
    xn = normalised(pr)
    k, Es = oracle.minimal(_abi.GCR_ESSENTIAL, xn, np.arange(5))
    assert k >= 1
    assert min(e_dist(E, pr["E_gt"]) for E in Es) < 1e-8
    x1 = np.c_[xn[:5, :2], np.ones(5)]
    x2 = np.c_[xn[:5, 2:], np.ones(5)]
    for E in Es:
        assert np.abs(np.einsum("ij,jk,ik->i", x2, E, x1)).max() < 1e-9 * np.abs(E).max()
        # essential: two equal singular values, one zero
        sv = np.linalg.svd(E, compute_uv=False)
        assert sv[2] < 1e-9 * sv[0] and abs(sv[0] - sv[1]) < 1e-7 * sv[0]


@pytest.mark.parametrize("n", [5, 6, 12, 35])
def test_stewenius_recovers_exact_model(oracle, n):
    pr = S.two_view_pair(7, n=100, inlier_ratio=1.0, sigma=0.0)
    xn = normalised(pr)
    Es = oracle.nonminimal_essential(xn, np.arange(n))
    assert len(Es) >= 1
    assert min(e_dist(E, pr["E_gt"]) for E in Es) < 1e-7
    for E in Es:
        assert abs(np.linalg.norm(E) - 1) < 1e-12 and E[2, 2] >= 0


def test_stewenius_weights_by_point_index(oracle):
    pr = S.two_view_pair(8, n=60, inlier_ratio=1.0, sigma=0.0)
    xn = normalised(pr)
    w = np.zeros(60)
    w[10:45] = np.linspace(0.2, 1.0, 35)
    Es = oracle.nonminimal_essential(xn, np.arange(10, 45), w)
    assert min(e_dist(E, pr["E_gt"]) for E in Es) < 1e-7


def test_essential_exact_recovery(oracle):
    pr = S.two_view_pair(5, n=300, inlier_ratio=1.0, sigma=0.0)
    K = pr["K"]
    rc, E, mask, st = oracle.find(_abi.GCR_ESSENTIAL, pr["corr"], oracle.make_size(*pr["size"]), e_params(),
                                  K1=K, K2=K)
    assert rc == 0
    assert mask.all()
    assert e_dist(E, pr["E_gt"]) < 1e-6


@pytest.mark.parametrize("seed,ratio", [(1, 0.5), (2, 0.3)])
def test_essential_noisy_pair(oracle, seed, ratio):
    pr = S.two_view_pair(seed, n=1000, inlier_ratio=ratio)
    K = pr["K"]
    rc, E, mask, st = oracle.find(_abi.GCR_ESSENTIAL, pr["corr"], oracle.make_size(*pr["size"]), e_params(),
                                  K1=K, K2=K)
    assert rc == 0
    assert (mask & pr["inlier_gt"]).sum() >= 0.95 * pr["inlier_gt"].sum()
    assert S.essential_error(E, pr) < 2.0
    assert st.iteration_number >= 50


def test_essential_too_few_points(oracle):
    pr = S.two_view_pair(1, n=10, inlier_ratio=1.0)
    rc, E, mask, st = oracle.find(_abi.GCR_ESSENTIAL, pr["corr"][:4], oracle.make_size(*pr["size"]), e_params(),
                                  K1=pr["K"], K2=pr["K"])
    assert rc == _abi.GCR_TOO_FEW_POINTS
