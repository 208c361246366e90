"""CPU tests of the oracle (the checker): known answers, golden vectors and
self-consistency. The reference ships no golden vectors for its H/F/E path;
the pins here are the published Philox known-answer vectors, the reference's
MAGSAC++ weight table (tests/golden/magsac_gamma_subset.json, made by
tests/golden/make_magsac_gamma.py) and exact synthetic data."""
import itertools
import json
import os

import numpy as np
import pytest

from pygcransac import _abi, synthetic as S

HERE = os.path.dirname(os.path.abspath(__file__))


def h_params(**kw):
    p = _abi.Params(threshold=3.0, confidence=0.99, spatial_coherence_weight=0.975, neighborhood_size=4,
                    max_iterations=10000, min_iterations=50, sampler=0, neighborhood=0, lo_number=50, seed=0)
    for k, v in kw.items():
        setattr(p, k, v)
    return p


def test_philox_known_answers(oracle):
    # Philox4x32-10 known-answer vectors published with Random123 (kat_vectors)
    assert oracle.philox([0, 0, 0, 0], [0, 0]) == [0x6627e8d5, 0xe169c58d, 0xbc57ac4c, 0x9b00dbd8]
    f = 0xffffffff
    assert oracle.philox([f, f, f, f], [f, f]) == [0x408f276d, 0x41c83b0e, 0xa20bc7c6, 0x6d5451fd]
    assert oracle.philox([0x243f6a88, 0x85a308d3, 0x13198a2e, 0x03707344], [0xa4093822, 0x299f31d0]) == \
        [0xd16cfe09, 0x94fdcceb, 0x5001e420, 0x24126ea1]
    # the stream layout: draw d of call c of stream s is word d&3 of counter {d>>2, c_lo, c_hi, s}
    assert [oracle.draw_u32(0, 0, 0, d) for d in range(4)] == oracle.philox([0, 0, 0, 0], [0, 0])
    assert oracle.draw_u32((7 << 32) | 5, 3, (2 << 32) | 9, 6) == oracle.philox([1, 9, 2, 3], [5, 7])[2]


def test_magsac_table_matches_reference(oracle):
    g = json.load(open(os.path.join(HERE, "golden", "magsac_gamma_subset.json")))
    for k, v in g["entries"].items():
        i = int(k)
        if i > 36000:  # the lookup clamps at 36000 (scoring_function.h:330)
            continue
        assert abs(oracle.magsac_gamma(i) - v) <= 1e-12 * max(1.0, abs(v)), i


def test_homography_exact_recovery(oracle):
    pr = S.homography_pair(3, n=400, inlier_ratio=0.5, sigma=0.0)
    rc, Hm, mask, st = oracle.find(0, pr["corr"], oracle.make_size(*pr["size"]), h_params(threshold=1.0))
    assert rc == 0
    Hn = Hm / Hm[2, 2]
    assert np.abs(Hn - pr["H_gt"]).max() / np.abs(pr["H_gt"]).max() < 1e-9
    assert mask[pr["inlier_gt"]].all()


def test_homography_cfg_pair(oracle):
    pr = S.homography_pair(0)
    rc, Hm, mask, st = oracle.find(0, pr["corr"], oracle.make_size(*pr["size"]), h_params())
    assert rc == 0
    assert (mask & pr["inlier_gt"]).sum() >= 790
    assert S.homography_error(Hm, pr["H_gt"]) < 1.0
    assert st.local_optimization_number >= 2 and st.graph_cut_number >= 1


def test_oracle_deterministic(oracle):
    pr = S.homography_pair(7, n=600)
    a = oracle.find(0, pr["corr"], oracle.make_size(*pr["size"]), h_params(seed=5))
    b = oracle.find(0, pr["corr"], oracle.make_size(*pr["size"]), h_params(seed=5))
    assert np.array_equal(a[1], b[1]) and np.array_equal(a[2], b[2])
    assert a[3].iteration_number == b[3].iteration_number


def test_too_few_points(oracle):
    pr = S.homography_pair(1, n=50)
    rc, *_ = oracle.find(0, pr["corr"][:3], oracle.make_size(*pr["size"]), h_params())
    assert rc == _abi.GCR_TOO_FEW_POINTS


def test_no_model_on_pure_outliers(oracle):
    rng = np.random.default_rng(0)
    corr = np.c_[rng.uniform(0, 640, (30, 1)), rng.uniform(0, 480, (30, 1)), rng.uniform(0, 640, (30, 1)),
                 rng.uniform(0, 480, (30, 1))]
    rc, Hm, mask, st = oracle.find(0, corr, oracle.make_size(480, 640, 480, 640), h_params(threshold=0.01))
    assert rc == _abi.GCR_NO_MODEL and mask.sum() == 0


def _energy(labels, d, r2le, lam, cells):
    """Energy of a labelling (label 1 = SINK = inlier) as built by GCRANSAC::labeling."""
    e = 0.0
    for i, L in enumerate(labels):
        if r2le[i]:
            e += 0.0 if L else (1 - lam) * (1 - d[i])
        else:
            e += (1 - lam) * d[i] if L else 0.0
    for cell in cells:
        for a, b in itertools.combinations(cell, 2):
            la, lb = labels[a], labels[b]
            if la == 0 and lb == 0:
                e += lam * 0.5 * (d[a] + d[b])
            elif la != lb:
                e += lam
    return e


@pytest.mark.parametrize("seed", range(6))
def test_labeling_is_minimal_sink_min_cut(oracle, seed):
    """The oracle's labelling is the minimiser of the graph-cut energy with the
    smallest SINK set (the BK convention that free nodes are SOURCE), checked by
    enumeration on a small problem."""
    rng = np.random.default_rng(seed)
    n = 11
    H = np.eye(3)
    x1 = rng.uniform(400, 600, (n, 2))
    x2 = x1 + rng.normal(0, 2.5, (n, 2))
    corr = np.c_[x1, x2]
    # one grid cell holds every point, so the graph is a single clique
    p = h_params(threshold=2.0, spatial_coherence_weight=0.6 + 0.05 * seed, neighborhood_size=1)
    lab = oracle.labeling(0, corr, oracle.make_size(1000, 1000, 1000, 1000), p, H.reshape(9))
    r2 = np.sum((x2 - x1) ** 2, axis=1)
    sq = 2.0 ** 2 * 9 / 4
    d = np.clip(r2 / sq, 0, 1)
    cells = [list(range(n))]
    lam = p.spatial_coherence_weight
    best = None
    minimisers = []
    for bits in range(1 << n):
        L = [(bits >> i) & 1 for i in range(n)]
        e = _energy(L, d, r2 <= sq, lam, cells)
        if best is None or e < best - 1e-12:
            best, minimisers = e, [L]
        elif abs(e - best) <= 1e-12:
            minimisers.append(L)
    inter = np.all(np.array(minimisers), axis=0)
    assert np.array_equal(lab, inter.astype(bool))


def test_radius_graph_is_the_exact_ball(oracle):
    """The oracle's radius neighbourhood (the FlannNeighborhoodGraph restated
    with an exact search) against a NumPy ball search with the same operation
    order: same neighbour counts, symmetric, no self-loops."""
    from pygcransac import synthetic as S
    pr = S.two_view_pair(77, n=400, inlier_ratio=0.5)
    c = pr["corr"]
    d = c[None, :, :] - c[:, None, :]
    d2 = ((d[..., 0] * d[..., 0] + d[..., 1] * d[..., 1]) + d[..., 2] * d[..., 2]) + d[..., 3] * d[..., 3]
    ref = (d2 <= 20.0 * 20.0) & ~np.eye(len(c), dtype=bool)
    assert np.array_equal(ref, ref.T) and ref.sum() > 0
    np.testing.assert_array_equal(oracle.radius_counts(c, 20.0), ref.sum(1))


@pytest.mark.parametrize("sampler", [3, 4])
def test_oracle_run_with_probabilities(oracle, sampler):
    """GCRANSAC::run alone with the importance (3) or AR (4) sampler on the
    probabilities it is given (a noiseless inlier indicator scaled to maximum
    1): the homography is recovered; without probabilities the run reports
    GCR_UNSUPPORTED (the sampler cannot be built) instead of running."""
    pr = S.homography_pair(11, n=1500)
    ph = np.where(pr["inlier_gt"], 0.9, 0.1)
    ph = ph / ph.max()
    p = _abi.Params(threshold=3.0, confidence=0.99, spatial_coherence_weight=0.975, neighborhood_size=4,
                    max_iterations=2000, min_iterations=50, sampler=sampler, lo_number=50, seed=3,
                    sampler_variance=0.1)
    cells = [160.0, 120.0, 160.0, 120.0]
    size = oracle.make_size(480, 640, 480, 640)
    rc, M, mask, st = oracle.run(_abi.GCR_HOMOGRAPHY, pr["corr"], pr["corr"], cells, 4, size, p, seed=3,
                                 probabilities=ph)
    assert rc == 0 and mask.sum() >= 0.9 * pr["inlier_gt"].sum()
    assert S.homography_error(M / M[2, 2], pr["H_gt"]) < 1.0
    rc2, _, _, _ = oracle.run(_abi.GCR_HOMOGRAPHY, pr["corr"], pr["corr"], cells, 4, size, p, seed=3)
    assert rc2 == _abi.GCR_UNSUPPORTED


def test_oracle_sample_tape_replays_its_own_draws(oracle):
    """The oracle's main sampler replaced by a tape of its own draws runs the
    same search (every count and the mask); a tape of other draws changes the
    run; a tape that ends early or holds -1 rows fails those calls."""
    from pygcransac import synthetic as S
    pr = S.homography_pair(3, n=600)
    sz = oracle.make_size(*pr["size"])
    p = _abi.Params(threshold=3.0, confidence=0.99, spatial_coherence_weight=0.975, neighborhood_size=4,
                    max_iterations=10000, min_iterations=50, sampler=0, neighborhood=0, lo_number=50, seed=0)
    rc, H, mask, st = oracle.find(0, pr["corr"], sz, p, seed=11)
    own, ok = oracle.sample_sequence(0, pr["corr"], 4, 11, 5000, sz)
    assert ok.all()
    rc2, H2, mask2, st2 = oracle.find(0, pr["corr"], sz, p, seed=11, sample_tape=own)
    assert rc == rc2 == 0 and np.array_equal(mask, mask2) and np.array_equal(H, H2)
    assert (st.iteration_number, st.graph_cut_number, st.models_scored) == \
        (st2.iteration_number, st2.graph_cut_number, st2.models_scored)
    other, _ = oracle.sample_sequence(0, pr["corr"], 4, 99, 5000, sz)
    _, _, _, st3 = oracle.find(0, pr["corr"], sz, p, seed=11, sample_tape=other)
    assert (st3.iteration_number, st3.models_scored) != (st.iteration_number, st.models_scored)
    # no usable call at all: 100 failed calls per iteration until the budget ends
    dead = np.full((300, 4), -1, np.int32)
    p.max_iterations = 200
    rc4, _, mask4, st4 = oracle.find(0, pr["corr"], sz, p, seed=11, sample_tape=dead)
    assert rc4 == _abi.GCR_NO_MODEL and not mask4.any() and st4.iteration_number >= 200


def test_contracted_build_moves_only_rounding_ties(oracle):
    """The FMA-contracted oracle build agrees with the plain build on ordinary
    pairs and differs on a pair whose local optimisation ends on a score tie
    at the last bits (a ragged 3489-point homography pair under P-NAPSAC):
    the plain build runs one more graph cut than the contracted one."""
    p = _abi.Params(threshold=3.0, confidence=0.99, spatial_coherence_weight=0.975, neighborhood_size=8,
                    max_iterations=2000, min_iterations=50, sampler=2, neighborhood=0, lo_number=20)
    res = {}
    for seed, n, s in ((528, 3489, 45), (11, 1200, 4)):
        pr = S.homography_pair(seed, n=n, inlier_ratio=0.4)
        for c in (False, True):
            if c:
                with oracle.contracted():
                    res[(seed, c)] = oracle.find(0, pr["corr"], oracle.make_size(*pr["size"]), p, seed=s)
            else:
                res[(seed, c)] = oracle.find(0, pr["corr"], oracle.make_size(*pr["size"]), p, seed=s)
    a, b = res[(11, False)], res[(11, True)]
    assert a[0] == b[0] == 0 and np.array_equal(a[2], b[2]) and a[3].graph_cut_number == b[3].graph_cut_number
    a, b = res[(528, False)], res[(528, True)]
    assert a[0] == b[0] == 0
    assert (a[3].graph_cut_number, b[3].graph_cut_number) == (5, 4)
    assert a[3].iteration_number == b[3].iteration_number
