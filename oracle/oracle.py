"""Python handle on the oracle (test infrastructure only).

The oracle is a CPU FP64 restatement of the reference's Graph-Cut RANSAC path;
tests, smoke() and the CPU-baseline leg of bench.py use it as the checker.
Parity anchors: the reference ships no golden vectors for this path (its
tests assert inlier-count floors on SIFT matches that need OpenCV), so the
oracle is pinned by known-answer tests on exact synthetic data, by the MAGSAC++
gamma table read from the reference as text, and by self-consistency checks.
"""
import ctypes
import os
import subprocess
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "_build", "liboracle.so")
# the same sources with multiply-adds contracted into FMAs (the rounding of
# the reference built by gcc for aarch64); see `contracted`
LIB_CONTRACT = os.path.join(HERE, "_build", "liboracle_contract.so")
sys.path.insert(0, os.path.join(os.path.dirname(HERE), "graph-cut-ransac_gb300"))
from pygcransac import _abi  # noqa: E402  (POD types shared with the engine)

_libs = {}
_contract = False


class contracted:
    """Inside the block every oracle call runs the FMA-contracted build. A
    pair whose result differs between the two builds sits on a rounding-level
    tie (two scores equal to the last bits, a residual at the threshold): its
    outcome is not fixed by the algorithm at FP64 precision."""

    def __enter__(self):
        global _contract
        self._prev, _contract = _contract, True
        return self

    def __exit__(self, *exc):
        global _contract
        _contract = self._prev
        return False


def build():
    subprocess.check_call(["sh", os.path.join(HERE, "build.sh")])


def load(contract=None):
    contract = _contract if contract is None else bool(contract)
    if contract not in _libs:
        path = LIB_CONTRACT if contract else LIB
        if not os.path.exists(path):
            build()
        lib = ctypes.CDLL(path)
        P = ctypes.c_void_p
        lib.oracle_find.restype = ctypes.c_int
        lib.oracle_find.argtypes = [ctypes.c_int, P, ctypes.c_int64, P, P, P, P, ctypes.c_uint64, P, P, P]
        lib.oracle_find_batch.restype = ctypes.c_double
        lib.oracle_find_batch.argtypes = [ctypes.c_int, ctypes.c_int64, P, P, P, P, P, P, P, P, P, ctypes.c_int]
        lib.oracle_find_prob.restype = ctypes.c_int
        lib.oracle_find_prob.argtypes = [ctypes.c_int, P, ctypes.c_int64, P, P, P, P, P, ctypes.c_uint64, P, P, P]
        lib.oracle_radius_counts.restype = None
        lib.oracle_radius_counts.argtypes = [P, ctypes.c_int64, ctypes.c_double, P]
        lib.oracle_run.restype = ctypes.c_int
        lib.oracle_run.argtypes = [ctypes.c_int, P, P, ctypes.c_int64, P, ctypes.c_int32, P, P, ctypes.c_uint64, P,
                                   P, P]
        lib.oracle_run_prob.restype = ctypes.c_int
        lib.oracle_run_prob.argtypes = [ctypes.c_int, P, P, ctypes.c_int64, P, ctypes.c_int32, P, P, P,
                                        ctypes.c_uint64, P, P, P]
        lib.oracle_magsac_gamma.restype = ctypes.c_double
        lib.oracle_magsac_gamma.argtypes = [ctypes.c_int]
        lib.oracle_labeling.restype = ctypes.c_int
        lib.oracle_labeling.argtypes = [ctypes.c_int, P, ctypes.c_int64, P, P, P, P]
        lib.oracle_msac_score.restype = ctypes.c_double
        lib.oracle_msac_score.argtypes = [ctypes.c_int, P, ctypes.c_int64, P, ctypes.c_double, P]
        lib.oracle_minimal.restype = ctypes.c_int
        lib.oracle_minimal.argtypes = [ctypes.c_int, P, ctypes.c_int64, P, P]
        lib.oracle_nonminimal_essential.restype = ctypes.c_int
        lib.oracle_nonminimal_essential.argtypes = [P, ctypes.c_int64, P, ctypes.c_int64, P, P]
        lib.oracle_sturm10.restype = ctypes.c_int
        lib.oracle_sturm10.argtypes = [P, P]
        lib.oracle_sample_sequence.restype = ctypes.c_int
        lib.oracle_sample_sequence.argtypes = [ctypes.c_int, ctypes.c_int64, ctypes.c_int, ctypes.c_uint64,
                                               ctypes.c_int64, P, P, P, P]
        lib.oracle_philox.restype = None
        lib.oracle_philox.argtypes = [P, P, P]
        lib.oracle_set_sample_tape.restype = None
        lib.oracle_set_sample_tape.argtypes = [P, ctypes.c_int64]
        lib.oracle_draw_u32.restype = ctypes.c_uint32
        lib.oracle_draw_u32.argtypes = [ctypes.c_uint64, ctypes.c_uint32, ctypes.c_uint64, ctypes.c_uint32]
        _libs[contract] = lib
    return _libs[contract]


def _p(a):
    return None if a is None else a.ctypes.data_as(ctypes.c_void_p)  # keeps the array alive


def make_size(h1, w1, h2, w2):
    return _abi.ImageSize(int(h1), int(w1), int(h2), int(w2))


class _Tape:
    """The main sampler reads `tape` ([calls, m] or [pairs, calls, m] point
    indices, -1 for a failed call) for the calls inside the block; None
    leaves the sampler alone."""

    def __init__(self, tape):
        self.tape = None if tape is None else np.ascontiguousarray(tape, np.int32)

    def __enter__(self):
        if self.tape is not None:
            load().oracle_set_sample_tape(_p(self.tape), int(self.tape.shape[-2]))
        return self

    def __exit__(self, *exc):
        if self.tape is not None:
            load().oracle_set_sample_tape(None, 0)
        return False


def find(kind, corr, size, params, seed=None, K1=None, K2=None, probabilities=None, sample_tape=None):
    """Runs the oracle on one pair. Returns (status, model 3x3, mask bool[N], stats).
    `probabilities` feed the importance sampler (sampler 3); `sample_tape`
    [calls, m] replaces the main sampler's draws."""
    with _Tape(sample_tape):
        return _find(kind, corr, size, params, seed, K1, K2, probabilities)


def _find(kind, corr, size, params, seed=None, K1=None, K2=None, probabilities=None):
    lib = load()
    corr = np.ascontiguousarray(corr, dtype=np.float64)
    n = corr.shape[0]
    model = np.zeros(9)
    mask = np.zeros(n, np.uint8)
    st = _abi.Stats()
    K1 = None if K1 is None else np.ascontiguousarray(K1, np.float64)
    K2 = None if K2 is None else np.ascontiguousarray(K2, np.float64)
    seed = params.seed if seed is None else seed
    if probabilities is not None:
        pr = np.ascontiguousarray(probabilities, np.float64)
        rc = lib.oracle_find_prob(kind, _p(corr), n, _p(K1), _p(K2), _p(pr), ctypes.byref(size),
                                  ctypes.byref(params), seed, _p(model), _p(mask), ctypes.byref(st))
    else:
        rc = lib.oracle_find(kind, _p(corr), n, _p(K1), _p(K2), ctypes.byref(size), ctypes.byref(params),
                             seed, _p(model), _p(mask), ctypes.byref(st))
    return rc, model.reshape(3, 3), mask.astype(bool), st


def radius_counts(corr, radius):
    """Neighbour count of every point in the radius graph."""
    lib = load()
    corr = np.ascontiguousarray(corr, np.float64)
    out = np.zeros(len(corr), np.int64)
    lib.oracle_radius_counts(_p(corr), len(corr), float(radius), _p(out))
    return out


def run(kind, points, pixels, cell_sizes, divisions, size, params, seed=0, probabilities=None, sample_tape=None):
    """GCRANSAC::run alone (oracle_run): (status, model [3, 3], mask, stats).
    `probabilities` feed the importance and AR samplers (samplers 3 and 4);
    `sample_tape` [calls, m] replaces the main sampler's draws."""
    with _Tape(sample_tape):
        return _run(kind, points, pixels, cell_sizes, divisions, size, params, seed, probabilities)


def _run(kind, points, pixels, cell_sizes, divisions, size, params, seed=0, probabilities=None):
    lib = load()
    points = np.ascontiguousarray(points, np.float64)
    pixels = None if pixels is None else np.ascontiguousarray(pixels, np.float64)
    cs = np.ascontiguousarray(cell_sizes, np.float64)
    n = len(points)
    model = np.zeros(9)
    mask = np.zeros(n, np.uint8)
    st = _abi.Stats()
    if probabilities is not None:
        pr = np.ascontiguousarray(probabilities, np.float64)
        rc = lib.oracle_run_prob(kind, _p(points), _p(pixels), n, _p(cs), int(divisions), ctypes.byref(size),
                                 _p(pr), ctypes.byref(params), int(seed), _p(model), _p(mask), ctypes.byref(st))
    else:
        rc = lib.oracle_run(kind, _p(points), _p(pixels), n, _p(cs), int(divisions), ctypes.byref(size),
                            ctypes.byref(params), int(seed), _p(model), _p(mask), ctypes.byref(st))
    return rc, model.reshape(3, 3), mask.astype(bool), st


def find_batch(kind, corr, offsets, sizes, params, seeds=None, K=None, threads=1, sample_tape=None):
    """Pair-parallel oracle batch. Returns (models [P,9], masks, stats, wall seconds).
    `sample_tape` [P, calls, m] replaces the main sampler's draws of each pair."""
    with _Tape(sample_tape):
        return _find_batch(kind, corr, offsets, sizes, params, seeds, K, threads)


def _find_batch(kind, corr, offsets, sizes, params, seeds=None, K=None, threads=1):
    lib = load()
    corr = np.ascontiguousarray(corr, np.float64)
    offsets = np.ascontiguousarray(offsets, np.int64)
    P = len(offsets) - 1
    models = np.zeros((P, 9))
    masks = np.zeros(int(offsets[-1]), np.uint8)
    stats = np.zeros(P, _abi.STATS_DTYPE)
    s = np.asarray(sizes)
    if s.dtype != _abi.SIZE_DTYPE:
        # rows (h1, w1, h2, w2): fill the struct fields (a plain cast would
        # broadcast each value into every field)
        s = s.reshape(P, 4)
        sizes = np.zeros(P, _abi.SIZE_DTYPE)
        sizes["h1"], sizes["w1"], sizes["h2"], sizes["w2"] = s[:, 0], s[:, 1], s[:, 2], s[:, 3]
    else:
        sizes = np.ascontiguousarray(s)
    seeds = None if seeds is None else np.ascontiguousarray(seeds, np.uint64)
    K = None if K is None else np.ascontiguousarray(K, np.float64)
    t = lib.oracle_find_batch(kind, P, _p(corr), _p(offsets), _p(K), _p(sizes), ctypes.byref(params),
                              _p(seeds), _p(models), _p(masks), _p(stats), threads)
    return models, masks.astype(bool), stats, t


def magsac_gamma(i):
    return load().oracle_magsac_gamma(i)


def labeling(kind, corr, size, params, model):
    lib = load()
    corr = np.ascontiguousarray(corr, np.float64)
    model = np.ascontiguousarray(model, np.float64).reshape(9)
    out = np.zeros(corr.shape[0], np.uint8)
    lib.oracle_labeling(kind, _p(corr), corr.shape[0], ctypes.byref(size), ctypes.byref(params), _p(model),
                        _p(out))
    return out.astype(bool)


def msac_score(kind, corr, model, threshold):
    lib = load()
    corr = np.ascontiguousarray(corr, np.float64)
    model = np.ascontiguousarray(model, np.float64).reshape(9)
    cnt = np.zeros(1, np.int64)
    v = lib.oracle_msac_score(kind, _p(corr), corr.shape[0], _p(model), threshold, _p(cnt))
    return v, int(cnt[0])


def minimal(kind, corr, sample):
    lib = load()
    corr = np.ascontiguousarray(corr, np.float64)
    sample = np.ascontiguousarray(sample, np.int64)
    out = np.zeros((10, 9))
    k = lib.oracle_minimal(kind, _p(corr), corr.shape[0], _p(sample), _p(out))
    return k, out[:max(k, 0)].reshape(-1, 3, 3)


def sample_sequence(sampler, corr, m, seed, calls, size):
    lib = load()
    corr = np.ascontiguousarray(corr, np.float64)
    out = np.zeros((calls, m), np.int64)
    ok = np.zeros(calls, np.uint8)
    lib.oracle_sample_sequence(sampler, corr.shape[0], m, seed, calls, _p(corr), ctypes.byref(size), _p(out),
                               _p(ok))
    return out, ok.astype(bool)


def philox(ctr, key):
    c = np.ascontiguousarray(ctr, np.uint32)
    k = np.ascontiguousarray(key, np.uint32)
    out = np.zeros(4, np.uint32)
    load().oracle_philox(_p(c), _p(k), _p(out))
    return [int(v) for v in out]


def draw_u32(seed, stream, call, draw):
    return load().oracle_draw_u32(seed, stream, call, draw)


def nonminimal_essential(corr, sample, weights=None):
    """Stewenius fit of normalised correspondences; returns a list of 3x3 models."""
    lib = load()
    corr = np.ascontiguousarray(corr, dtype=np.float64)
    s = np.ascontiguousarray(sample, dtype=np.int64)
    w = None if weights is None else np.ascontiguousarray(weights, np.float64)
    out = np.zeros(90)
    k = lib.oracle_nonminimal_essential(_p(corr), corr.shape[0], _p(s), len(s), _p(w), _p(out))
    return [out[9 * i:9 * i + 9].reshape(3, 3) for i in range(k)]


def sturm10(coeffs):
    """Real roots of sum coeffs[i] x^i (degree 10) by Sturm bracketing."""
    lib = load()
    c = np.ascontiguousarray(coeffs, dtype=np.float64)
    r = np.zeros(10)
    k = lib.oracle_sturm10(_p(c), _p(r))
    return np.sort(r[:k])
