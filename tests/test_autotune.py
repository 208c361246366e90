"""CPU tests of the launch-shape autotuner's cache and selection logic
(pygcransac.autotune): the JSON cache is keyed by GPU name, model kind and
size bucket; the table handed to gcr_context_set_tuning selects, per batch,
the entry of its kind with the smallest bucket covering its largest pair (the
rule gcr_batch_prepare applies); the library refuses malformed tables."""
import ctypes

import pytest

from pygcransac import _abi, autotune as A


def test_cache_round_trip_keyed_by_gpu(tmp_path):
    path = str(tmp_path / "t.json")
    cache = {}
    A.record(cache, "GPU-A", _abi.GCR_FUNDAMENTAL, 4000, (64, 2, 1), {(64, 2, 1): 1.5, (256, 2, 0): 2.0})
    A.record(cache, "GPU-A", _abi.GCR_FUNDAMENTAL, 30000, (256, 1, 1))
    A.record(cache, "GPU-A", _abi.GCR_HOMOGRAPHY, 2000, (128, 2, 0))
    A.record(cache, "GPU-B", _abi.GCR_FUNDAMENTAL, 4000, (256, 2, 0))
    A.save_cache(cache, path)
    back = A.load_cache(path)
    assert back["GPU-A"]["1"]["4096"]["batch_calls"] == 64
    assert back["GPU-A"]["1"]["4096"]["ms"]["64/2/1"] == 1.5
    assert back["GPU-A"]["1"]["65536"]["ctas_per_sm"] == 1
    rows_a = A.table(back, "GPU-A")
    rows_b = A.table(back, "GPU-B")
    assert len(rows_a) == 3 and len(rows_b) == 1
    assert A.table(back, "GPU-C") == []


def test_selection_rule():
    cache = {}
    A.record(cache, "g", _abi.GCR_FUNDAMENTAL, 1000, (64, 2, 0))
    A.record(cache, "g", _abi.GCR_FUNDAMENTAL, 4000, (128, 2, 1))
    A.record(cache, "g", _abi.GCR_FUNDAMENTAL, 40000, (256, 1, 1))
    A.record(cache, "g", _abi.GCR_ESSENTIAL, 8000, (256, 2, 1))
    rows = A.table(cache, "g")
    pick = lambda kind, n: A.select(rows, kind, n)  # noqa: E731
    assert pick(_abi.GCR_FUNDAMENTAL, 900).batch_calls == 64
    assert pick(_abi.GCR_FUNDAMENTAL, 1024).batch_calls == 64
    assert pick(_abi.GCR_FUNDAMENTAL, 1025).batch_calls == 128
    assert pick(_abi.GCR_FUNDAMENTAL, 20000).ctas_per_sm == 1
    assert pick(_abi.GCR_ESSENTIAL, 8000).order == 1
    assert pick(_abi.GCR_HOMOGRAPHY, 100) is None
    assert pick(_abi.GCR_FUNDAMENTAL, 1 << 24) is None
    assert A.bucket_of(4096) == 4096 and A.bucket_of(4097) == 16384
    with pytest.raises(ValueError):
        A.bucket_of(1 << 25)


def test_candidates_cover_each_knob():
    assert {c[0] for c in A.CANDIDATES} == {64, 128, 256}
    assert {c[1] for c in A.CANDIDATES} == {1, 2}
    assert {c[2] for c in A.CANDIDATES} == {0, 1}


def test_library_refuses_bad_tables():
    lib = _abi.load()
    assert lib.gcr_context_set_tuning(None, None, 0) == _abi.GCR_INVALID_ARG
    t = _abi.Tuning()
    assert lib.gcr_context_last_tuning(None, ctypes.byref(t)) == _abi.GCR_INVALID_ARG
    assert ctypes.sizeof(_abi.Tuning) == 24


def test_staged_search_plan():
    s1 = A.stage_one()
    assert len(s1) == 4 and all(b == max(A.BATCH_CALLS) for b, _, _ in s1)
    assert {(c, o) for _, c, o in s1} == {(c, o) for c in A.CTAS_PER_SM for o in A.ORDERS}
    timings = {(256, 1, 0): 9.0, (256, 1, 1): 7.0, (256, 2, 0): 8.0, (256, 2, 1): 7.5}
    s2 = A.stage_two(timings)
    assert s2 == ((64, 1, 1), (128, 1, 1))
    assert set(s1) | set(s2) <= set(A.CANDIDATES)
