"""Sample-tape replay: recorded minimal samples replace the main sampler's
draws (gcr_context_set_sample_tape / gcr_set_sample_tape, the `sample_tape`
keyword of the Python entries), the hook through which a run replays the
sample indices of another implementation.

* A tape of other draws (the oracle's sampler under another seed) drives the
  device and the oracle to the same run: exact masks, statuses, iteration and
  graph-cut counts, models within 1e-6 relative Frobenius error.
* A tape of the sampler's own draws reproduces the run without a tape bit for
  bit, so the replay follows the sampler's call numbering exactly.
* Calls past the end of the tape and rows marked -1 are unsuccessful calls on
  both sides.
"""
import ctypes

import numpy as np
import pytest

from pygcransac import _abi, synthetic as S

pytestmark = pytest.mark.gpu

MODEL_TOL = 1e-6
M = {_abi.GCR_HOMOGRAPHY: 4, _abi.GCR_FUNDAMENTAL: 7, _abi.GCR_ESSENTIAL: 5}


def rel_err(a, b):
    a = a / np.linalg.norm(a)
    b = b / np.linalg.norm(b)
    return min(np.linalg.norm(a - b), np.linalg.norm(a + b))


def case(kind, seed):
    if kind == _abi.GCR_HOMOGRAPHY:
        pr = S.homography_pair(seed, n=1200, inlier_ratio=0.35)
        p = _abi.Params(threshold=3.0, confidence=0.99, spatial_coherence_weight=0.975, neighborhood_size=4,
                        max_iterations=3000, min_iterations=50, sampler=0, neighborhood=0, lo_number=50, seed=0)
        return pr, p, None
    pr = S.two_view_pair(seed, n=1000, inlier_ratio=0.45)
    if kind == _abi.GCR_FUNDAMENTAL:
        p = _abi.Params(threshold=0.75, confidence=0.99, spatial_coherence_weight=0.975, neighborhood_size=8,
                        max_iterations=3000, min_iterations=50, sampler=0, neighborhood=0, lo_number=50, seed=0)
        return pr, p, None
    p = _abi.Params(threshold=0.75, confidence=0.99, spatial_coherence_weight=0.1, neighborhood_size=8,
                    max_iterations=3000, min_iterations=50, sampler=0, neighborhood=0, lo_number=20, seed=0)
    return pr, p, pr["K"]


def tape_of(oracle, pr, m, seed, calls):
    t, ok = oracle.sample_sequence(0, pr["corr"], m, seed, calls, oracle.make_size(*pr["size"]))
    t = t.astype(np.int32)
    t[~ok] = -1
    return t


@pytest.mark.parametrize("kind", [_abi.GCR_HOMOGRAPHY, _abi.GCR_FUNDAMENTAL, _abi.GCR_ESSENTIAL])
def test_tape_drives_device_like_oracle(oracle, gcr, kind):
    pr, p, K = case(kind, 300 + kind)
    m = M[kind]
    tape = tape_of(oracle, pr, m, seed=777, calls=3500)
    kw = {} if K is None else dict(K1=K, K2=K)
    rc, M_o, mask_o, st_o = oracle.find(kind, pr["corr"], oracle.make_size(*pr["size"]), p, seed=5, sample_tape=tape,
                                        **kw)
    Kb = None if K is None else np.concatenate([K.ravel(), K.ravel()])[None]
    models, masks, stats = gcr.find_batch(kind, [pr["corr"]], [pr["size"]], p, seeds=[5], K=Kb,
                                          sample_tape=tape[None])
    assert stats["status"][0] == rc == 0
    assert np.array_equal(masks[0], mask_o)
    assert stats["iteration_number"][0] == st_o.iteration_number
    assert stats["graph_cut_number"][0] == st_o.graph_cut_number
    assert rel_err(models[0], M_o) < MODEL_TOL
    # without the tape the run differs (the tape is what drove it)
    _, _, stats_free = gcr.find_batch(kind, [pr["corr"]], [pr["size"]], p, seeds=[5], K=Kb)
    assert stats_free["iteration_number"][0] != stats["iteration_number"][0] or \
        stats_free["models_scored"][0] != stats["models_scored"][0]


@pytest.mark.parametrize("kind", [_abi.GCR_HOMOGRAPHY, _abi.GCR_FUNDAMENTAL])
def test_tape_of_own_draws_equals_drawing(oracle, gcr, kind):
    pr, p, _ = case(kind, 320 + kind)
    tape = tape_of(oracle, pr, M[kind], seed=9, calls=3500)
    a = gcr.find_batch(kind, [pr["corr"]], [pr["size"]], p, seeds=[9])
    b = gcr.find_batch(kind, [pr["corr"]], [pr["size"]], p, seeds=[9], sample_tape=tape[None])
    assert np.array_equal(a[0], b[0]) and np.array_equal(a[1][0], b[1][0]) and np.array_equal(a[2], b[2])
    # the single-pair Python entry takes the same tape
    if kind == _abi.GCR_HOMOGRAPHY:
        H, mask = gcr.findHomography(pr["corr"], *pr["size"], None, threshold=3.0, use_sprt=False, sampler=0,
                                     use_space_partitioning=False, max_iters=3000, seed=9, sample_tape=tape)
        assert np.array_equal(mask, a[1][0])


def test_short_and_marked_tapes_fail_calls_like_oracle(oracle, gcr):
    kind = _abi.GCR_HOMOGRAPHY
    pr, p, _ = case(kind, 340)
    tape = tape_of(oracle, pr, 4, seed=21, calls=400)
    tape[::3] = -1  # every third call failed when recorded
    rc, M_o, mask_o, st_o = oracle.find(kind, pr["corr"], oracle.make_size(*pr["size"]), p, seed=2, sample_tape=tape)
    models, masks, stats = gcr.find_batch(kind, [pr["corr"]], [pr["size"]], p, seeds=[2], sample_tape=tape[None])
    assert stats["status"][0] == rc
    assert np.array_equal(masks[0], mask_o)
    assert stats["iteration_number"][0] == st_o.iteration_number


def test_device_batch_tape_per_pair(oracle):
    torch = pytest.importorskip("torch")
    lib = _abi.load()
    kind = _abi.GCR_HOMOGRAPHY
    pairs, tapes = [], []
    for i in range(3):
        pr, p, _ = case(kind, 360 + i)
        pairs.append(pr)
        tapes.append(tape_of(oracle, pr, 4, seed=50 + i, calls=3200))
    tape = np.ascontiguousarray(np.stack(tapes))
    corr = np.ascontiguousarray(np.concatenate([q["corr"] for q in pairs]))
    off = np.zeros(4, np.int64)
    off[1:] = np.cumsum([len(q["corr"]) for q in pairs])
    sz = np.zeros(3, _abi.SIZE_DTYPE)
    for i, q in enumerate(pairs):
        sz[i] = q["size"]
    seeds = np.array([4, 5, 6], np.uint64)
    d_corr = torch.from_numpy(corr).cuda()
    d_tape = torch.from_numpy(tape).cuda()
    pm = torch.zeros(27, dtype=torch.float64, device="cuda")
    pk = torch.zeros(len(corr), dtype=torch.uint8, device="cuda")
    ps = torch.zeros(3 * _abi.STATS_DTYPE.itemsize, dtype=torch.uint8, device="cuda")
    ptr = lambda t: ctypes.c_void_p(t.data_ptr())  # noqa: E731
    ctx = ctypes.c_void_p()
    assert lib.gcr_context_create(ctypes.byref(ctx)) == 0
    try:
        assert lib.gcr_context_set_sample_tape(ctx, ptr(d_tape), -1) == _abi.GCR_INVALID_ARG
        assert lib.gcr_context_set_sample_tape(ctx, ptr(d_tape), tape.shape[1]) == 0
        rc = lib.gcr_batch_run_device(ctx, kind, 3, ptr(d_corr), _abi.ptr(off), None, _abi.ptr(sz), ctypes.byref(p),
                                      _abi.ptr(seeds), ptr(pm), ptr(pk), ptr(ps), None)
        assert rc == 0, _abi.last_error()
        torch.cuda.synchronize()
    finally:
        lib.gcr_context_destroy(ctx)
    stats = np.frombuffer(ps.cpu().numpy().tobytes(), _abi.STATS_DTYPE)
    masks = pk.cpu().numpy().astype(bool)
    m_o, k_o, st_o, _ = oracle.find_batch(kind, corr, off, sz, p, seeds=seeds, sample_tape=tape)
    assert np.array_equal(stats["status"], st_o["status"])
    assert np.array_equal(stats["iteration_number"], st_o["iteration_number"])
    assert np.array_equal(masks, k_o)
