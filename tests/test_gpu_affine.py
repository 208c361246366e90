"""GPU parity of the affine-correspondence homography (findHomographyAC_,
src/pygcransac/src/gcransac_python.cpp:4553-4811; python findHomography with
solver = 2): the device engine against the oracle on the same seeded inputs
of rows (x1, y1, x2, y2, a11, a12, a21, a22), through the C-ABI. Statuses,
iteration, graph-cut and models-scored counts and masks must be identical,
models equal to 1e-6 relative Frobenius error after normalisation."""
import numpy as np
import pytest

from pygcransac import _abi, synthetic as S

pytestmark = pytest.mark.gpu

MODEL_TOL = 1e-6


def ac_params(**kw):
    p = _abi.Params(threshold=3.0, confidence=0.99, spatial_coherence_weight=0.975, neighborhood_size=4,
                    max_iterations=10000, min_iterations=50, sampler=0, neighborhood=0, lo_number=50, seed=0,
                    min_inlier_ratio_for_sprt=1e-5)
    for k, v in kw.items():
        setattr(p, k, v)
    return p


def rel_model_err(a, b):
    a = a / np.linalg.norm(a)
    b = b / np.linalg.norm(b)
    return min(np.linalg.norm(a - b), np.linalg.norm(a + b))


def compare(oracle, gcr, pairs, p, seeds, tape=None):
    corr = [pr["corr"] for pr in pairs]
    sizes = [pr["size"] for pr in pairs]
    models, masks, stats = gcr.find_batch(_abi.GCR_HOMOGRAPHY_AFFINE, corr, sizes, p, seeds=seeds, sample_tape=tape)
    for i, pr in enumerate(pairs):
        rc_o, H_o, m_o, st_o = oracle.find(_abi.GCR_HOMOGRAPHY_AFFINE, pr["corr"], oracle.make_size(*pr["size"]), p,
                                           seed=seeds[i], sample_tape=None if tape is None else tape[i])
        assert stats["status"][i] == rc_o, (i, stats["status"][i], rc_o)
        assert np.array_equal(masks[i], m_o), f"pair {i}: mask differs at {np.nonzero(masks[i] != m_o)[0][:10]}"
        if rc_o == 0:
            assert rel_model_err(models[i], H_o) < MODEL_TOL
        for f in ("iteration_number", "graph_cut_number", "models_scored", "inlier_number"):
            assert stats[f][i] == getattr(st_o, f), (i, f, stats[f][i], getattr(st_o, f))
    return models, masks, stats


@pytest.mark.parametrize("sampler,use_sprt", [(0, 0), (1, 0), (0, 1)])
def test_affine_homography_batch(oracle, gcr, sampler, use_sprt):
    pairs = [S.homography_affine_pair(40 + i, n=n, inlier_ratio=r)
             for i, (n, r) in enumerate([(600, 0.5), (1500, 0.3), (3000, 0.4), (40, 0.8)])]
    compare(oracle, gcr, pairs, ac_params(sampler=sampler, use_sprt=use_sprt, max_iterations=2000),
            seeds=[3, 4, 5, 6])


def test_affine_homography_tape_of_inlier_samples(oracle, gcr):
    """A tape of all-inlier minimal samples drives device and oracle through
    the same minimal models, local optimisations and final fit."""
    pairs, tapes = [], []
    for i in range(3):
        pr = S.homography_affine_pair(70 + i, n=1200, inlier_ratio=0.35)
        inl = np.nonzero(pr["inlier_gt"])[0]
        rng = np.random.Generator(np.random.PCG64(i))
        tapes.append(np.stack([rng.choice(inl, 2, replace=False) for _ in range(300)]).astype(np.int32))
        pairs.append(pr)
    compare(oracle, gcr, pairs, ac_params(max_iterations=300, min_iterations=300), seeds=[1, 2, 3],
            tape=np.stack(tapes))


def test_affine_homography_python_entry(oracle, gcr):
    """findHomography(..., solver=2) runs the affine kind with the reference
    binding's shapes and returns (model or None, mask) like the oracle."""
    pr = S.homography_affine_pair(90, n=800, inlier_ratio=0.5)
    h, w = pr["size"][:2]
    H, mask = gcr.findHomography(pr["corr"], h, w, h, w, threshold=3.0, sampler=0, use_sprt=False,
                                 max_iters=1000, solver=2, seed=9)
    p = ac_params(max_iterations=1000, use_sprt=0, seed=9)
    rc_o, H_o, m_o, _ = oracle.find(_abi.GCR_HOMOGRAPHY_AFFINE, pr["corr"], oracle.make_size(*pr["size"]), p,
                                    seed=9)
    assert np.array_equal(mask, m_o)
    assert (H is None) == (rc_o != 0 or m_o.sum() == 0)
    if H is not None:
        assert rel_model_err(H, H_o) < MODEL_TOL
