"""Drop-in ``pygcransac`` entry points backed by the GB300 engine (libgcr.so).

Function names, argument names, defaults and return conventions follow the
reference binding (src/pygcransac/src/bindings.cpp:1003-1022, 1091-1112,
1158-1178): each call returns ``(model 3x3 float64 or None, mask bool[N])`` and
raises ``ValueError`` for a bad shape or too few correspondences. Added keyword
arguments: ``seed`` (the sampler streams are seeded and replayable) and, in
``find_batch``, many image pairs in one device launch.

There is no CPU fallback: a missing libgcr.so raises ImportError on first use,
and options the device engine does not provide raise NotImplementedError.
"""
import numpy as np

from . import _abi

__all__ = ["findHomography", "findFundamentalMatrix", "findEssentialMatrix", "findPlanarEssentialMatrix", "find_batch",
           "default_params",
           "GCRError"]


class GCRError(RuntimeError):
    def __init__(self, status, msg):
        super().__init__(f"{_abi.STATUS_NAMES.get(status, status)}: {msg}")
        self.status = status


def default_params(kind):
    """gcr_params filled with the reference binding's defaults for `kind`."""
    import ctypes
    p = _abi.Params()
    _abi.load().gcr_default_params(kind, ctypes.byref(p))
    return p


def _params(kind, threshold, conf, spatial_coherence_weight, max_iters, min_iters, use_sprt, sampler,
            neighborhood, neighborhood_size, lo_number, use_space_partitioning=False, seed=0, scoring=0,
            min_inlier_ratio_for_sprt=0.00001, sampler_variance=0.1):
    p = _abi.Params()
    p.threshold = float(threshold)
    p.confidence = float(conf)
    p.spatial_coherence_weight = float(spatial_coherence_weight)
    p.neighborhood_size = float(neighborhood_size)
    p.max_iterations = int(max_iters)
    p.min_iterations = int(min_iters)
    p.sampler = int(sampler)
    p.neighborhood = int(neighborhood)
    p.lo_number = int(lo_number)
    p.scoring = int(scoring)
    p.use_sprt = int(bool(use_sprt))
    p.use_space_partitioning = int(bool(use_space_partitioning))
    p.seed = int(seed)
    p.min_inlier_ratio_for_sprt = float(min_inlier_ratio_for_sprt)
    p.sampler_variance = float(sampler_variance)
    return p


def _check_corr(correspondences, m, what, cols=4):
    c = np.ascontiguousarray(correspondences, dtype=np.float64)
    if c.ndim != 2 or c.shape[1] != cols:
        if cols == 8:
            raise ValueError(f"SIFT or affine correspondences should be an array with dims [n,8], n>={m}")
        raise ValueError(f"correspondences should be an array with dims [n,4], n>={m}")
    if c.shape[0] < m:
        raise ValueError(f"correspondences should be an array with dims [n,d], n>={m}")
    return c


def _raise_for(rc, where):
    if rc in (_abi.GCR_OK, _abi.GCR_NO_MODEL):
        return
    msg = _abi.last_error()
    if rc == _abi.GCR_UNSUPPORTED:
        raise NotImplementedError(f"{where}: {msg}")
    if rc in (_abi.GCR_INVALID_ARG, _abi.GCR_TOO_FEW_POINTS):
        raise ValueError(f"{where}: {msg}")
    raise GCRError(rc, f"{where}: {msg}")


def _probabilities(probabilities, n, sampler):
    """The weights of the importance and AR samplers (3, 4), else None (the
    other samplers ignore them, as in the reference)."""
    if int(sampler) not in (_abi.GCR_SAMPLER_IMPORTANCE, _abi.GCR_SAMPLER_AR):
        return None
    if probabilities is None:
        raise ValueError("samplers 3 and 4 need per-correspondence probabilities")
    p = np.ascontiguousarray(probabilities, dtype=np.float64).reshape(-1)
    if p.shape[0] != n:
        raise ValueError(f"probabilities has {p.shape[0]} entries for {n} correspondences")
    if not np.all(np.isfinite(p)) or np.any(p < 0) or not p.sum() > 0:
        raise ValueError("probabilities must be finite, non-negative and not all zero")
    return p


class _SampleTape:
    """Sets the host sample tape of this thread's entry calls inside the block
    (gcr_set_sample_tape): `tape` [calls, m] for one pair or [P, calls, m]
    for a batch, int point indices, -1 for a failed call; None leaves the
    sampler alone."""

    def __init__(self, tape, m, pairs=None):
        self.tape = None
        if tape is not None:
            t = np.ascontiguousarray(tape, np.int32)
            want = 2 if pairs is None else 3
            if t.ndim != want or t.shape[-1] != m or (pairs is not None and t.shape[0] != pairs):
                raise ValueError(f"sample_tape must have shape {'[calls, m]' if pairs is None else '[P, calls, m]'}"
                                 f" with m = {m}")
            self.tape = t

    def __enter__(self):
        if self.tape is not None:
            _raise_for(_abi.load().gcr_set_sample_tape(_abi.ptr(self.tape), int(self.tape.shape[-2])), "sample_tape")
        return self

    def __exit__(self, *exc):
        if self.tape is not None:
            _abi.load().gcr_set_sample_tape(None, 0)
        return False


_SAMPLE_SIZE = {_abi.GCR_HOMOGRAPHY: 4, _abi.GCR_FUNDAMENTAL: 7, _abi.GCR_ESSENTIAL: 5,
                _abi.GCR_HOMOGRAPHY_AFFINE: 2, _abi.GCR_FUNDAMENTAL_AFFINE: 3, _abi.GCR_FUNDAMENTAL_SIFT: 4,
                _abi.GCR_HOMOGRAPHY_SIFT: 2, _abi.GCR_ESSENTIAL_PLANAR: 2}
_ENTRY_NAME = {_abi.GCR_HOMOGRAPHY: "findHomography", _abi.GCR_FUNDAMENTAL: "findFundamentalMatrix",
               _abi.GCR_ESSENTIAL: "findEssentialMatrix", _abi.GCR_HOMOGRAPHY_AFFINE: "findHomography",
               _abi.GCR_FUNDAMENTAL_AFFINE: "findFundamentalMatrix", _abi.GCR_FUNDAMENTAL_SIFT: "findFundamentalMatrix",
               _abi.GCR_HOMOGRAPHY_SIFT: "findHomography", _abi.GCR_ESSENTIAL_PLANAR: "findPlanarEssentialMatrix"}
# entry points of the kinds with rows of 8 (same signature as gcr_find_homography)
_ROWS8_ENTRY = {_abi.GCR_HOMOGRAPHY_AFFINE: "gcr_find_homography_affine",
                _abi.GCR_HOMOGRAPHY_SIFT: "gcr_find_homography_sift",
                _abi.GCR_FUNDAMENTAL_AFFINE: "gcr_find_fundamental_affine",
                _abi.GCR_FUNDAMENTAL_SIFT: "gcr_find_fundamental_sift"}


def _run_one(kind, corr, size, params, K1=None, K2=None, return_stats=False, probabilities=None, sample_tape=None):
    with _SampleTape(sample_tape, _SAMPLE_SIZE[kind]):
        return _run_one_(kind, corr, size, params, K1, K2, return_stats, probabilities)


def _run_one_(kind, corr, size, params, K1=None, K2=None, return_stats=False, probabilities=None):
    import ctypes
    lib = _abi.load()
    n = corr.shape[0]
    prob = _probabilities(probabilities, n, params.sampler)
    model = np.zeros(9)
    mask = np.zeros(n, np.uint8)
    st = _abi.Stats()
    sz = _abi.ImageSize(*[int(v) for v in size])
    if kind == _abi.GCR_HOMOGRAPHY:
        rc = lib.gcr_find_homography(_abi.ptr(corr), n, ctypes.byref(sz), _abi.ptr(prob), ctypes.byref(params),
                                     _abi.ptr(model), _abi.ptr(mask), ctypes.byref(st))
    elif kind in _ROWS8_ENTRY:
        rc = getattr(lib, _ROWS8_ENTRY[kind])(_abi.ptr(corr), n, ctypes.byref(sz), _abi.ptr(prob),
                                              ctypes.byref(params), _abi.ptr(model), _abi.ptr(mask), ctypes.byref(st))
    elif kind == _abi.GCR_FUNDAMENTAL:
        rc = lib.gcr_find_fundamental(_abi.ptr(corr), n, ctypes.byref(sz), _abi.ptr(prob), ctypes.byref(params),
                                      _abi.ptr(model), _abi.ptr(mask), ctypes.byref(st))
    else:
        K1 = np.ascontiguousarray(K1, np.float64).reshape(9)
        K2 = np.ascontiguousarray(K2, np.float64).reshape(9)
        entry = lib.gcr_find_essential_planar if kind == _abi.GCR_ESSENTIAL_PLANAR else lib.gcr_find_essential
        rc = entry(_abi.ptr(corr), n, _abi.ptr(K1), _abi.ptr(K2), ctypes.byref(sz), _abi.ptr(prob),
                   ctypes.byref(params), _abi.ptr(model), _abi.ptr(mask), ctypes.byref(st))
    _raise_for(rc, _ENTRY_NAME[kind])
    maskb = mask.astype(bool)
    out = (None if rc == _abi.GCR_NO_MODEL or maskb.sum() == 0 else model.reshape(3, 3), maskb)
    return out + (st,) if return_stats else out


def findHomography(correspondences, h1, w1, h2, w2, probabilities=None, threshold=1.0, conf=0.99,
                   spatial_coherence_weight=0.975, max_iters=10000, min_iters=50, use_sprt=True,
                   min_inlier_ratio_for_sprt=0.00001, sampler=1, neighborhood=0, neighborhood_size=4.0,
                   use_space_partitioning=True, lo_number=50, sampler_variance=0.1, solver=0, seed=0,
                   return_stats=False, sample_tape=None):
    """Robust homography by Graph-Cut RANSAC (reference: bindings.cpp:859-983).
    solver 0: point correspondences [n, 4]; solver 1: SIFT correspondences
    [n, 8] (x1, y1, x2, y2, q1, q2, o1, o2: scales and orientations), two per
    minimal sample (findHomographySIFT_, gcransac_python.cpp:4813-5069);
    solver 2: affine correspondences [n, 8] (x1, y1, x2, y2, a11, a12, a21,
    a22), two per minimal sample (findHomographyAC_, :4553-4811); both
    drivers take samplers 0, 1, 3, 4 and no space partitioning.
    `sample_tape` [calls, m] replays recorded minimal samples in place of the
    main sampler's draws (gcr_set_sample_tape)."""
    if solver in (1, 2):
        kind = _abi.GCR_HOMOGRAPHY_SIFT if solver == 1 else _abi.GCR_HOMOGRAPHY_AFFINE
        c = _check_corr(correspondences, 4, "homography", cols=8)
        p = _params(kind, threshold, conf, spatial_coherence_weight, max_iters, min_iters,
                    use_sprt, sampler, neighborhood, neighborhood_size, lo_number, False, seed,
                    min_inlier_ratio_for_sprt=min_inlier_ratio_for_sprt, sampler_variance=sampler_variance)
        return _run_one(kind, c, (h1, w1, h2, w2), p, return_stats=return_stats,
                        probabilities=probabilities, sample_tape=sample_tape)
    if solver != 0:
        raise NotImplementedError(f"solver {solver} is not provided (0 points, 1 SIFT, 2 affine)")
    c = _check_corr(correspondences, 4, "homography")
    p = _params(_abi.GCR_HOMOGRAPHY, threshold, conf, spatial_coherence_weight, max_iters, min_iters, use_sprt,
                sampler, neighborhood, neighborhood_size, lo_number, use_space_partitioning, seed,
                min_inlier_ratio_for_sprt=min_inlier_ratio_for_sprt, sampler_variance=sampler_variance)
    return _run_one(_abi.GCR_HOMOGRAPHY, c, (h1, w1, h2, w2), p, return_stats=return_stats,
                    probabilities=probabilities, sample_tape=sample_tape)


def findFundamentalMatrix(correspondences, h1, w1, h2, w2, probabilities=None, threshold=1.0, conf=0.99,
                          spatial_coherence_weight=0.0, max_iters=10000, min_iters=50, use_sprt=True,
                          min_inlier_ratio_for_sprt=0.00001, sampler=1, neighborhood=1, neighborhood_size=20.0,
                          lo_number=50, sampler_variance=0.1, solver=0, seed=0, return_stats=False,
                          sample_tape=None):
    """Robust fundamental matrix by Graph-Cut RANSAC (reference: bindings.cpp:279-401).
    solver 0: point correspondences [n, 4]; solver 1: SIFT correspondences
    [n, 8] (x1, y1, x2, y2, q1, q2, o1, o2: scales and orientations), four per
    minimal sample (findFundamentalMatrixSIFT_, gcransac_python.cpp:2222-2518);
    solver 2: affine correspondences [n, 8] (x1, y1, x2, y2, a11, a12, a21,
    a22), three per minimal sample (findFundamentalMatrixAC_, :1924-2221);
    both take samplers 0, 1, 3, 4. `sample_tape` [calls, m] replays recorded
    minimal samples."""
    if solver in (1, 2):
        kind = _abi.GCR_FUNDAMENTAL_SIFT if solver == 1 else _abi.GCR_FUNDAMENTAL_AFFINE
        c = _check_corr(correspondences, 7, "fundamental", cols=8)
        p = _params(kind, threshold, conf, spatial_coherence_weight, max_iters, min_iters,
                    use_sprt, sampler, neighborhood, neighborhood_size, lo_number, False, seed,
                    min_inlier_ratio_for_sprt=min_inlier_ratio_for_sprt, sampler_variance=sampler_variance)
        return _run_one(kind, c, (h1, w1, h2, w2), p, return_stats=return_stats,
                        probabilities=probabilities, sample_tape=sample_tape)
    if solver != 0:
        raise NotImplementedError(f"solver {solver} is not provided (0 points, 1 SIFT, 2 affine)")
    c = _check_corr(correspondences, 7, "fundamental")
    p = _params(_abi.GCR_FUNDAMENTAL, threshold, conf, spatial_coherence_weight, max_iters, min_iters, use_sprt,
                sampler, neighborhood, neighborhood_size, lo_number, False, seed,
                min_inlier_ratio_for_sprt=min_inlier_ratio_for_sprt, sampler_variance=sampler_variance)
    return _run_one(_abi.GCR_FUNDAMENTAL, c, (h1, w1, h2, w2), p, return_stats=return_stats,
                    probabilities=probabilities, sample_tape=sample_tape)


def findEssentialMatrix(correspondences, K1, K2, h1, w1, h2, w2, probabilities=None, threshold=1.0, conf=0.99,
                        spatial_coherence_weight=0.1, max_iters=10000, min_iters=50, use_sprt=True,
                        min_inlier_ratio_for_sprt=0.01, sampler=1, neighborhood=1, neighborhood_size=20.0,
                        lo_number=50, sampler_variance=0.1, solver=0, seed=0, return_stats=False,
                        sample_tape=None):
    """Robust essential matrix by Graph-Cut RANSAC (reference: bindings.cpp:710-857).
    `sample_tape` [calls, 5] replays recorded minimal samples."""
    if solver != 0:
        raise NotImplementedError("only point correspondences (solver=0) are provided")
    c = _check_corr(correspondences, 5, "essential")
    p = _params(_abi.GCR_ESSENTIAL, threshold, conf, spatial_coherence_weight, max_iters, min_iters, use_sprt,
                sampler, neighborhood, neighborhood_size, lo_number, False, seed,
                min_inlier_ratio_for_sprt=min_inlier_ratio_for_sprt, sampler_variance=sampler_variance)
    return _run_one(_abi.GCR_ESSENTIAL, c, (h1, w1, h2, w2), p, K1=K1, K2=K2, return_stats=return_stats,
                    probabilities=probabilities, sample_tape=sample_tape)


def findPlanarEssentialMatrix(correspondences, K1, K2, h1, w1, h2, w2, probabilities=None, threshold=1.0, conf=0.99,
                              spatial_coherence_weight=0.975, max_iters=10000, min_iters=50, use_sprt=True,
                              min_inlier_ratio_for_sprt=0.00001, sampler=1, neighborhood=1, lo_number=50,
                              neighborhood_size=20.0, seed=0, return_stats=False, sample_tape=None):
    """Essential matrix of a planar camera motion (rotation about the
    camera's y axis, translation in its x-z plane) by Graph-Cut RANSAC
    (reference: bindings.cpp:610-707, 1114-1133; findPlanarEssentialMatrix_,
    gcransac_python.cpp:3531-3870): rows [n, 4] of pixels, n >= 3, two per
    minimal sample; MSAC; the AR sampler's variance is 0.1. `sample_tape`
    [calls, 2] replays recorded minimal samples."""
    c = _check_corr(correspondences, 3, "planar essential")
    p = _params(_abi.GCR_ESSENTIAL_PLANAR, threshold, conf, spatial_coherence_weight, max_iters, min_iters, use_sprt,
                sampler, neighborhood, neighborhood_size, lo_number, False, seed,
                min_inlier_ratio_for_sprt=min_inlier_ratio_for_sprt, sampler_variance=0.1)
    return _run_one(_abi.GCR_ESSENTIAL_PLANAR, c, (h1, w1, h2, w2), p, K1=K1, K2=K2, return_stats=return_stats,
                    probabilities=probabilities, sample_tape=sample_tape)


def find_batch(kind, correspondences, sizes, params, seeds=None, K=None, sample_tape=None):
    """Many pairs of one model kind in one device launch (host buffers).

    correspondences: list of [n_i, 4] arrays (rows of 8 for GCR_HOMOGRAPHY_AFFINE) or (concatenated
    [sum n_i, 4 or 8], offsets [P+1]).
    sizes: [P, 4] (h1, w1, h2, w2); params: an _abi.Params; K: [P, 18] for essential matrices.
    sample_tape: [P, calls, m] recorded minimal samples replacing the main sampler's draws.
    Returns (models [P, 3, 3], masks list of bool arrays, stats structured array).
    """
    P = len(correspondences[1]) - 1 if isinstance(correspondences, tuple) else len(correspondences)
    with _SampleTape(sample_tape, _SAMPLE_SIZE[kind], pairs=P):
        return _find_batch(kind, correspondences, sizes, params, seeds, K)


def _find_batch(kind, correspondences, sizes, params, seeds=None, K=None):
    lib = _abi.load()
    if isinstance(correspondences, tuple):
        corr, offsets = correspondences
        corr = np.ascontiguousarray(corr, np.float64)
        offsets = np.ascontiguousarray(offsets, np.int64)
    else:
        lens = [len(c) for c in correspondences]
        offsets = np.zeros(len(lens) + 1, np.int64)
        offsets[1:] = np.cumsum(lens)
        corr = np.ascontiguousarray(np.concatenate(correspondences, 0), np.float64)
    P = len(offsets) - 1
    sz = np.zeros(P, _abi.SIZE_DTYPE)
    s = np.asarray(sizes)
    sz["h1"], sz["w1"], sz["h2"], sz["w2"] = s[:, 0], s[:, 1], s[:, 2], s[:, 3]
    models = np.zeros((P, 9))
    masks = np.zeros(int(offsets[-1]), np.uint8)
    stats = np.zeros(P, _abi.STATS_DTYPE)
    seeds_a = None if seeds is None else np.ascontiguousarray(seeds, np.uint64)
    K_a = None if K is None else np.ascontiguousarray(K, np.float64)
    import ctypes
    rc = lib.gcr_find_batch(kind, P, _abi.ptr(corr), _abi.ptr(offsets), _abi.ptr(K_a), _abi.ptr(sz),
                            ctypes.byref(params), _abi.ptr(seeds_a), _abi.ptr(models), _abi.ptr(masks),
                            _abi.ptr(stats))
    _raise_for(rc, "find_batch")
    mb = masks.astype(bool)
    return models.reshape(P, 3, 3), [mb[offsets[i]:offsets[i + 1]] for i in range(P)], stats
