"""CPU checks of the C-ABI boundary: libgcr.so loads, exports every function
that include/gcr.h declares, and the ctypes mirror matches the C layout."""
import ctypes
import os
import re
import subprocess
import tempfile

import numpy as np
import pytest

from pygcransac import _abi

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "gcr.h")


def declared_functions():
    text = open(HEADER).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(gcr_[a-z_0-9]+)\s*\(", text)))


def test_library_exports_header_symbols():
    lib = _abi.load()
    names = declared_functions()
    assert "gcr_find_homography" in names and "gcr_batch_run_device" in names
    for n in names:
        assert hasattr(lib, n), n
    assert set(names) <= set(_abi.exported_symbols())


def test_struct_layout_matches_header():
    src = r'''
#include <stdio.h>
#include <stddef.h>
#include "gcr.h"
int main(void) {
  printf("%zu %zu %zu %zu %zu %zu %zu %zu %zu\n", sizeof(gcr_params), sizeof(gcr_stats), sizeof(gcr_image_size),
         offsetof(gcr_params, seed), offsetof(gcr_params, sampler), offsetof(gcr_stats, status),
         offsetof(gcr_params, use_space_partitioning), sizeof(gcr_tuning), offsetof(gcr_tuning, order));
  return 0;
}
'''
    with tempfile.TemporaryDirectory() as d:
        c = os.path.join(d, "t.c")
        exe = os.path.join(d, "t")
        open(c, "w").write(src)
        subprocess.check_call(["gcc", "-std=c99", "-I", os.path.join(ROOT, "include"), c, "-o", exe])
        out = [int(v) for v in subprocess.check_output([exe]).split()]
    P, S, Z = _abi.Params, _abi.Stats, _abi.ImageSize
    import ctypes
    T = _abi.Tuning
    assert out == [ctypes.sizeof(P), ctypes.sizeof(S), ctypes.sizeof(Z), P.seed.offset, P.sampler.offset,
                   S.status.offset, P.use_space_partitioning.offset, ctypes.sizeof(T), T.order.offset]


def test_python_argument_checks(gcr):
    with pytest.raises(ValueError):
        gcr.findHomography(np.zeros((10, 3)), 480, 640, 480, 640)
    with pytest.raises(ValueError):
        gcr.findHomography(np.zeros((3, 4)), 480, 640, 480, 640)
    with pytest.raises(ValueError):
        gcr.findFundamentalMatrix(np.zeros((6, 4)), 480, 640, 480, 640)
    with pytest.raises(ValueError):
        gcr.findEssentialMatrix(np.zeros((4, 4)), np.eye(3), np.eye(3), 480, 640, 480, 640)
    # the importance sampler needs one finite, non-negative weight per correspondence
    c = np.random.default_rng(0).uniform(0, 480, (50, 4))
    for bad in (None, np.ones(49), -np.ones(50), np.zeros(50), np.full(50, np.nan)):
        with pytest.raises(ValueError):
            gcr.findHomography(c, 480, 640, 480, 640, bad, sampler=3)


def test_default_params_follow_reference(gcr):
    p = gcr.default_params(_abi.GCR_HOMOGRAPHY)
    assert (p.threshold, p.confidence, p.spatial_coherence_weight, p.max_iterations, p.min_iterations) == \
        (1.0, 0.99, 0.975, 10000, 50)
    assert (p.sampler, p.neighborhood, p.neighborhood_size, p.lo_number) == (1, 0, 4.0, 50)
    f = gcr.default_params(_abi.GCR_FUNDAMENTAL)
    assert (f.spatial_coherence_weight, f.neighborhood, f.neighborhood_size) == (0.0, 1, 20.0)
    e = gcr.default_params(_abi.GCR_ESSENTIAL)
    assert (e.spatial_coherence_weight, e.neighborhood) == (0.1, 1)


def test_ptr_keeps_a_temporary_array_alive():
    """_abi.ptr(f(x)) passed straight into a call: the pointer object holds
    the array, so its memory is not freed before the call reads it."""
    import gc
    import weakref

    class Arr(np.ndarray):
        pass

    a = np.arange(16, dtype=np.float64).view(Arr)
    ref = weakref.ref(a)
    p = _abi.ptr(a)
    del a
    gc.collect()
    assert ref() is not None
    assert ctypes.cast(p, ctypes.POINTER(ctypes.c_double))[5] == 5.0
    del p
    gc.collect()
    assert ref() is None


def test_run_entries_check_probabilities_before_device_work():
    """gcr_run rejects the samplers that read probabilities, and
    gcr_run_with_probabilities rejects a missing, negative or non-finite
    probability: both return GCR_INVALID_ARG before any device call."""
    lib = _abi.load()
    n = 40
    pts = np.random.default_rng(1).uniform(0, 480, (n, 4))
    cells = np.array([160.0, 120.0, 160.0, 120.0])
    size = _abi.ImageSize(h1=480, w1=640, h2=480, w2=640)
    model = np.zeros(9)
    mask = np.zeros(n, np.uint8)
    st = _abi.Stats()
    for sampler in (_abi.GCR_SAMPLER_IMPORTANCE, _abi.GCR_SAMPLER_AR):
        p = _abi.Params(threshold=3.0, confidence=0.99, spatial_coherence_weight=0.975, neighborhood_size=4,
                        max_iterations=100, min_iterations=50, sampler=sampler, lo_number=50, sampler_variance=0.1)
        rc = lib.gcr_run(_abi.GCR_HOMOGRAPHY, _abi.ptr(pts), None, n, _abi.ptr(cells), 4, ctypes.byref(size),
                         ctypes.byref(p), _abi.ptr(model), _abi.ptr(mask), ctypes.byref(st))
        assert rc == _abi.GCR_INVALID_ARG and "gcr_run_with_probabilities" in _abi.last_error()
        for bad in (None, np.r_[np.ones(n - 1), -1.0], np.r_[np.ones(n - 1), np.inf], np.r_[np.ones(n - 1), np.nan]):
            rc = lib.gcr_run_with_probabilities(_abi.GCR_HOMOGRAPHY, _abi.ptr(pts), None, n, _abi.ptr(cells), 4,
                                                ctypes.byref(size), _abi.ptr(bad), ctypes.byref(p), _abi.ptr(model),
                                                _abi.ptr(mask), ctypes.byref(st))
            assert rc == _abi.GCR_INVALID_ARG, bad


def test_noalloc_entry_checks_arguments_before_device_work():
    """The allocation-free entry point applies the shared argument checks (a
    neighbourhood other than 0 or 1 is unsupported, a grid size that is not a
    number or above 1024 divisions is refused) and its own limits (samplers
    0-2, MSAC, the grid with a spatial term) before any device call; the
    dummy device pointers are never dereferenced."""
    lib = _abi.load()
    size = _abi.ImageSize(h1=480, w1=640, h2=480, w2=640)
    dummy = ctypes.c_void_p(16)

    def call(**kw):
        base = dict(threshold=3.0, confidence=0.99, spatial_coherence_weight=0.975, neighborhood_size=4,
                    max_iterations=100, min_iterations=50, sampler=0, neighborhood=0, lo_number=50)
        base.update(kw)
        p = _abi.Params(**base)
        return lib.gcr_find_homography_device_noalloc(dummy, 1000, ctypes.byref(size), ctypes.byref(p), 0, dummy,
                                                      dummy, dummy, None)

    assert call(spatial_coherence_weight=0.0, neighborhood=7) == _abi.GCR_UNSUPPORTED
    assert call(neighborhood=7) == _abi.GCR_UNSUPPORTED
    assert call(neighborhood_size=float("nan")) == _abi.GCR_INVALID_ARG
    assert call(neighborhood_size=0.5) == _abi.GCR_INVALID_ARG
    assert call(neighborhood_size=1e12) == _abi.GCR_UNSUPPORTED
    assert call(spatial_coherence_weight=0.0, neighborhood=1, neighborhood_size=float("inf")) == _abi.GCR_INVALID_ARG
    assert call(spatial_coherence_weight=0.5, neighborhood=1, neighborhood_size=20) == _abi.GCR_UNSUPPORTED
    assert call(sampler=3) == _abi.GCR_UNSUPPORTED
    assert call(scoring=_abi.GCR_SCORING_MAGSAC) == _abi.GCR_UNSUPPORTED
    assert call(threshold=-1.0) == _abi.GCR_INVALID_ARG


def test_batch_entry_refuses_grid_sizes_beyond_the_cell_key():
    """The batch entry refuses a grid of more than 1024 divisions per axis
    (cell keys hold 10 bits per axis) before any device work."""
    lib = _abi.load()
    n = 40
    pts = np.random.default_rng(2).uniform(0, 480, (n, 4))
    offsets = np.array([0, n], np.int64)
    sz = np.zeros(1, _abi.SIZE_DTYPE)
    sz[0] = (480, 640, 480, 640)
    p = _abi.Params(threshold=3.0, confidence=0.99, spatial_coherence_weight=0.975, neighborhood_size=5000,
                    max_iterations=100, min_iterations=50, sampler=0, neighborhood=0, lo_number=50)
    models = np.zeros(9)
    masks = np.zeros(n, np.uint8)
    stats = np.zeros(1, _abi.STATS_DTYPE)
    rc = lib.gcr_find_batch(_abi.GCR_HOMOGRAPHY, 1, _abi.ptr(pts), _abi.ptr(offsets), None, _abi.ptr(sz),
                            ctypes.byref(p), None, _abi.ptr(models), _abi.ptr(masks), _abi.ptr(stats))
    assert rc == _abi.GCR_UNSUPPORTED and "1024" in _abi.last_error()
