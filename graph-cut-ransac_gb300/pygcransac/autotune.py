"""Launch-shape autotuner of the pair engine.

The engine's persistent launch has three shape knobs that change its speed but
never its results (include/gcr.h, gcr_tuning):

* ``batch_calls``: sampler calls (hypotheses) each CTA draws, solves and
  scores together (the hypotheses per CTA of one batch), 64 / 128 / 256.
  Calls are counter-based and replayed in call order, so a smaller batch only
  wastes fewer hypotheses drawn past a run's termination point (the learned
  form stops after 50 iterations) at the price of fewer hypotheses in flight.
* ``ctas_per_sm``: resident engine CTAs per SM (1 or 2): two share the SM's
  FP64 pipe and hide each other's barrier waits; one runs each pair faster.
* ``order``: pairs in the caller's order, or largest first, so that a CTA
  does not take a large pair last and finish long after the others.

``tune`` times every candidate shape on a calibration batch (the same pairs
and parameters each time, results checked identical), ``record`` stores the
fastest per model kind and size bucket in a JSON cache keyed by GPU name, and
``apply`` installs the cached table on a context, where gcr_batch_prepare
picks the entry for the batch's kind and largest pair.
"""
import ctypes
import itertools
import json
import os

import numpy as np

from . import _abi

BATCH_CALLS = (64, 128, 256)
CTAS_PER_SM = (1, 2)
ORDERS = (0, 1)
CANDIDATES = tuple(itertools.product(BATCH_CALLS, CTAS_PER_SM, ORDERS))
# size buckets (largest pair of a batch, correspondences)
BUCKETS = (1024, 4096, 16384, 65536, (1 << 24) - 1)


def cache_path():
    """The tuning cache: $GCR_TUNING_CACHE, else _build/tuning.json next to the library."""
    return os.environ.get("GCR_TUNING_CACHE") or os.path.join(os.path.dirname(_abi.LIB_PATH), "tuning.json")


def bucket_of(max_n):
    for b in BUCKETS:
        if max_n <= b:
            return b
    raise ValueError(f"{max_n} correspondences exceed the engine's limit")


def load_cache(path=None):
    path = path or cache_path()
    if not os.path.exists(path):
        return {}
    with open(path) as f:
        return json.load(f)


def save_cache(cache, path=None):
    path = path or cache_path()
    os.makedirs(os.path.dirname(os.path.abspath(path)), exist_ok=True)
    tmp = path + ".tmp"
    with open(tmp, "w") as f:
        json.dump(cache, f, indent=1, sort_keys=True)
    os.replace(tmp, path)


def record(cache, gpu, kind, max_n, shape, timings=None):
    """Stores the shape (batch_calls, ctas_per_sm, order) of `kind` for the
    size bucket of `max_n` under the GPU name."""
    b = bucket_of(max_n)
    entry = {"batch_calls": int(shape[0]), "ctas_per_sm": int(shape[1]), "order": int(shape[2])}
    if timings is not None:
        entry["ms"] = {f"{c[0]}/{c[1]}/{c[2]}": float(t) for c, t in timings.items()}
    cache.setdefault(gpu, {}).setdefault(str(int(kind)), {})[str(b)] = entry
    return cache


def table(cache, gpu):
    """The gcr_tuning entries of one GPU, ready for gcr_context_set_tuning."""
    rows = []
    for kind, buckets in sorted(cache.get(gpu, {}).items()):
        for b, e in sorted(buckets.items(), key=lambda kv: int(kv[0])):
            rows.append(_abi.Tuning(kind=int(kind), max_n=int(b), batch_calls=e["batch_calls"],
                                    ctas_per_sm=e["ctas_per_sm"], order=e["order"], reserved=0))
    return rows


def select(rows, kind, max_n):
    """The entry gcr_batch_prepare uses for a batch (same rule as the
    library): kind matches, smallest max_n at or above the batch's largest
    pair; None when no entry covers it."""
    best = None
    for r in rows:
        if r.kind == kind and r.max_n >= max_n and (best is None or r.max_n < best.max_n):
            best = r
    return best


def set_table(ctx, rows):
    arr = (_abi.Tuning * max(1, len(rows)))(*rows)
    rc = _abi.load().gcr_context_set_tuning(ctx, arr if rows else None, len(rows))
    if rc != _abi.GCR_OK:
        raise RuntimeError(f"gcr_context_set_tuning: {_abi.last_error()}")


def apply(ctx, gpu=None, path=None):
    """Installs the cached table of this GPU on `ctx`; returns its entries."""
    gpu = gpu or gpu_name()
    rows = table(load_cache(path), gpu)
    set_table(ctx, rows)
    return rows


def last_tuning(ctx):
    t = _abi.Tuning()
    rc = _abi.load().gcr_context_last_tuning(ctx, ctypes.byref(t))
    if rc != _abi.GCR_OK:
        raise RuntimeError(_abi.last_error())
    return {"batch_calls": t.batch_calls, "ctas_per_sm": t.ctas_per_sm, "order": t.order, "max_n": t.max_n}


def gpu_name():
    import torch
    return torch.cuda.get_device_name()


def stage_one():
    """First stage of the staged search: every (CTAs per SM, order) at the
    largest batch."""
    return tuple((max(BATCH_CALLS), c, o) for c in CTAS_PER_SM for o in ORDERS)


def stage_two(timings):
    """Second stage: the other batch sizes at the fastest (CTAs per SM, order)
    of the first stage (`timings`: {shape: ms})."""
    _, c, o = min(timings, key=timings.get)
    return tuple((b, c, o) for b in BATCH_CALLS if (b, c, o) not in timings)


def tune(kind, d_corr, offsets, sizes, params, seeds=None, K=None, candidates=CANDIDATES, repeats=2,
         lo_precision=None, staged=False):
    """Times each candidate shape on the device-resident calibration batch
    (d_corr a torch CUDA tensor of [total, 4] doubles; offsets, sizes, seeds,
    K host arrays as for gcr_batch_run_device; lo_precision, when given, is
    set on the calibration context). With `staged` the search times
    stage_one() and then stage_two() of its timings (6 shapes instead of 12):
    the order and CTAs per SM set how the pairs spread over the SMs, the batch
    size mostly how many hypotheses are drawn past termination, so the two
    are searched one after the other. Returns (fastest shape, {shape: best
    milliseconds}). Raises if two shapes disagree on any result."""
    import torch
    lib = _abi.load()
    offsets = np.ascontiguousarray(offsets, np.int64)
    P = len(offsets) - 1
    total = int(offsets[-1])
    sz = np.zeros(P, _abi.SIZE_DTYPE)
    s = np.asarray(sizes)
    sz["h1"], sz["w1"], sz["h2"], sz["w2"] = s[:, 0], s[:, 1], s[:, 2], s[:, 3]
    seeds_a = None if seeds is None else np.ascontiguousarray(seeds, np.uint64)
    K_a = None if K is None else np.ascontiguousarray(K, np.float64)
    max_n = int(np.diff(offsets).max())
    pm = torch.zeros(P * 9, dtype=torch.float64, device="cuda")
    pk = torch.zeros(total, dtype=torch.uint8, device="cuda")
    ps = torch.zeros(P * _abi.STATS_DTYPE.itemsize, dtype=torch.uint8, device="cuda")
    vp = lambda t: ctypes.c_void_p(t.data_ptr())  # noqa: E731
    stream = torch.cuda.current_stream()
    ctx = ctypes.c_void_p()
    assert lib.gcr_context_create(ctypes.byref(ctx)) == _abi.GCR_OK, _abi.last_error()
    timings, ref = {}, None

    def stages():
        if not staged:
            yield from candidates
            return
        yield from stage_one()
        yield from stage_two(timings)

    try:
        if lo_precision is not None and lib.gcr_context_set_lo_precision(ctx, int(lo_precision)) != _abi.GCR_OK:
            raise RuntimeError(f"gcr_context_set_lo_precision: {_abi.last_error()}")
        for shape in stages():
            set_table(ctx, [_abi.Tuning(kind=int(kind), max_n=max_n, batch_calls=shape[0], ctas_per_sm=shape[1],
                                        order=shape[2], reserved=0)])
            best = float("inf")
            for _ in range(repeats):
                e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                e0.record(stream)
                rc = lib.gcr_batch_run_device(ctx, int(kind), P, vp(d_corr), _abi.ptr(offsets), _abi.ptr(K_a),
                                              _abi.ptr(sz), ctypes.byref(params), _abi.ptr(seeds_a), vp(pm), vp(pk),
                                              vp(ps), ctypes.c_void_p(stream.cuda_stream))
                if rc != _abi.GCR_OK:
                    raise RuntimeError(f"gcr_batch_run_device: {_abi.last_error()}")
                e1.record(stream)
                e1.synchronize()
                best = min(best, e0.elapsed_time(e1))
            timings[tuple(shape)] = best
            out = (pk.clone(), ps.clone(), pm.clone())
            if ref is None:
                ref = out
            elif not (torch.equal(out[0], ref[0]) and torch.equal(out[1], ref[1]) and torch.equal(out[2], ref[2])):
                raise RuntimeError(f"launch shape {shape} changed a result")
    finally:
        lib.gcr_context_destroy(ctx)
    fastest = min(timings, key=timings.get)
    return fastest, timings
