#!/usr/bin/env python
"""Throughput benchmark of the GB300 Graph-Cut RANSAC engine.

Default workload (`learned`): 1216 hard fundamental-matrix pairs per step
(4000 correspondences, 5-10 % inliers). `value` is the pairs/s of the
learned-proposal batched form: each step replays two CUDA graphs, the proposal
(neighbour features, MLP, per-pair ordering: three kernels) and the engine
(one persistent PROSAC launch with a 50-iteration budget, plus the mask
mapping); the plain form (uniform sampler, the reference's 10000-iteration
budget, one persistent launch) is timed on the same pairs and reported under
`plain`, with both median model errors. `equal_error` sweeps the plain form's
iteration budget on a subset of the same pairs and compares the two forms at
equal median model error.

The default run also measures the other workloads with a few steps each and
reports them under `workloads`: `homography` (2000 correspondences),
`fundamental` (5000, P-NAPSAC), `essential` (batched, 200-8000, MAGSAC++) and
`serving` (4096 pairs split across H / F / E, 2000-40000 correspondences,
learned and plain forms on three streams, per-pair latency percentiles). Each
carries its own `value`, `e2e`, `cpu_baseline` and median model error.
`--workload X` makes X the headline instead.

Correspondences are resident in HBM for `value` (CUDA events on the launching
stream, L2 flushed between steps by a 256 MiB write); `e2e` is the same metric
through the public API with host buffers, host<->device copies included.
`--impl reference` times the CPU restatement of the reference's path (the
oracle, plain method) on all host cores instead.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gcr|reference]
                  [--workload learned|serving|homography|fundamental|essential] [--pairs P]
                  [--no-side] [--side-steps S] [--no-sweep]
"""
import argparse
import ctypes
import json
import os
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(ROOT, "graph-cut-ransac_gb300"))

from pygcransac import _abi, autotune, synthetic as S  # noqa: E402

METRIC = "image pairs/sec at equal model error; learned vs plain GC-RANSAC on 1 GB300"

# Algorithmic FP32 work of one residual evaluation (one model x one correspondence):
# H transfer error 21 FLOP, Sampson distance 35 FLOP.
FLOP_PER_RESIDUAL = {"homography": 21, "fundamental": 35, "essential": 35, "learned": 35, "fundamental_affine": 35,
                     "fundamental_sift": 35, "homography_sift": 21, "essential_planar": 35}

WORKLOADS = {
    # 2000 correspondences in 640x480, 40 % inliers (sigma 1 px), threshold 3 px,
    # confidence 0.99, uniform sampler, 4^4 grid, lambda 0.975, 50 LO trials
    "homography": dict(kind=_abi.GCR_HOMOGRAPHY, n=2000, ratio=0.4, threshold=3.0, sampler=0, grid=4,
                       lam=0.975, pairs=1216),
    # 5000 correspondences of a two-view scene (depth 2-10 m, f = 800 px,
    # rotation up to 30 deg, unit baseline), 25 % inliers (sigma 0.5 px),
    # threshold 0.75 px, P-NAPSAC sampler, 8^4 grid, lambda 0.975, 7-point
    # solver + graph-cut LO, DEGENSAC on
    "fundamental": dict(kind=_abi.GCR_FUNDAMENTAL, n=5000, ratio=0.25, threshold=0.75, sampler=2, grid=8,
                        lam=0.975, pairs=608),
    # SIFT correspondences of the same homography scenes (feature scales and
    # orientations consistent with the homography's Jacobian, 0.01 rad / 1 %
    # noise): the two-SIFT solver, otherwise as the homography workload
    # without space partitioning
    "homography_sift": dict(kind=_abi.GCR_HOMOGRAPHY_SIFT, n=2000, ratio=0.4, threshold=3.0, sampler=0, grid=4,
                            lam=0.975, pairs=1216),
    # affine correspondences of the same scene (each inlier on a local plane,
    # its 2x2 affine map the Jacobian of the plane's homography + 0.01 noise):
    # 5000 per pair, 25 % inliers, threshold 0.75 px, uniform sampler (the
    # affine driver offers no P-NAPSAC), 8^4 grid, lambda 0.975, the
    # three-affine solver + graph-cut LO, no DEGENSAC
    "fundamental_affine": dict(kind=_abi.GCR_FUNDAMENTAL_AFFINE, n=5000, ratio=0.25, threshold=0.75, sampler=0,
                               grid=8, lam=0.975, pairs=608),
    # SIFT correspondences of the same scene (feature scales and orientations
    # consistent with the local affine maps, 0.01 rad / 1 % noise): the
    # four-SIFT solver, otherwise as the affine workload
    "fundamental_sift": dict(kind=_abi.GCR_FUNDAMENTAL_SIFT, n=5000, ratio=0.25, threshold=0.75, sampler=0,
                             grid=8, lam=0.975, pairs=608),
    # calibrated pairs (f = 800 px, scene as above) with log-uniform 200-8000
    # correspondences and inlier ratio uniform in 10-70 % (sigma 0.5 px),
    # threshold 0.75 px (divided by the focal length), uniform sampler, 8^4
    # grid, lambda 0.1, 5-point solver + graph-cut LO, MAGSAC++ scoring
    "essential": dict(kind=_abi.GCR_ESSENTIAL, n=(200, 8000), ratio=(0.1, 0.7), threshold=0.75, sampler=0, grid=8,
                      lam=0.1, pairs=1024, scoring=_abi.GCR_SCORING_MAGSAC),
    # planar camera motion (rotation about the camera's y axis up to 30 deg,
    # unit translation in its x-z plane; scene, f and noise as above): 1024
    # pairs x 2000 correspondences, 30 % inliers, threshold 0.75 px, uniform
    # sampler, 8^4 grid, lambda 0.975, the two-point planar solver with the
    # bundle-adjustment non-minimal fits, MSAC, SPRT off
    "essential_planar": dict(kind=_abi.GCR_ESSENTIAL_PLANAR, n=2000, ratio=0.3, threshold=0.75, sampler=0, grid=8,
                             lam=0.975, pairs=1024),
    # hard fundamental-matrix pairs: 4000 correspondences of the two-view scene
    # above at 5-10 % inliers. Plain form: uniform sampler with the reference's
    # 10000-iteration budget; learned form: the network's order drives PROSAC
    # with a 50-iteration budget. Same threshold, grid, lambda and LO.
    "learned": dict(kind=_abi.GCR_FUNDAMENTAL, n=4000, ratio=(0.05, 0.10), threshold=0.75, sampler=0, grid=8,
                    lam=0.975, pairs=1216, learned_iters=50),
    # mixed serving batch: pairs split evenly across H / F / E (pair i has kind
    # i mod 3), correspondences log-uniform over 2k-40k, inliers uniform over
    # 5-60 %, 16^4 grid, the learned proposal for every kind; MSAC; plain
    # form: uniform sampler, 10000 iterations; learned form: PROSAC on the
    # learned order, 50 iterations
    "serving": dict(kind=None, n=(2000, 40000), ratio=(0.05, 0.60), threshold=None, sampler=0, grid=16,
                    lam=None, pairs=4096, learned_iters=50),
}

SERVING_KINDS = [  # (generator, kind, threshold, lambda)
    ("homography", _abi.GCR_HOMOGRAPHY, 3.0, 0.975),
    ("fundamental", _abi.GCR_FUNDAMENTAL, 0.75, 0.975),
    ("essential", _abi.GCR_ESSENTIAL, 0.75, 0.1),
]

# launch shapes the serving mix's autotuning tries (a subset, to keep the
# calibration of six batches short)
SERVING_CANDIDATES = ((256, 2, 0), (256, 2, 1), (256, 1, 1), (64, 2, 1))

# plain-form iteration budgets of the equal-error comparison
SWEEP_BUDGETS = (10000, 30000, 100000, 300000, 1000000)

CHECKPOINT = os.path.join(ROOT, "graph-cut-ransac_gb300", "pygcransac", "weights", "proposal_fundamental.gcrl")


def _gen_pair(job):
    """One synthetic pair (runs in a spawn pool)."""
    workload, seed, n, ratio = job
    if workload == "homography":
        pr = S.homography_pair(seed, n=n, inlier_ratio=ratio)
        return pr["corr"], pr["size"], pr["H_gt"]
    if workload == "fundamental_affine":
        pr = S.two_view_affine_pair(seed, n=n, inlier_ratio=ratio)
        return pr["corr"], pr["size"], pr
    if workload == "fundamental_sift":
        pr = S.two_view_sift_pair(seed, n=n, inlier_ratio=ratio)
        return pr["corr"], pr["size"], pr
    if workload == "homography_sift":
        pr = S.homography_sift_pair(seed, n=n, inlier_ratio=ratio)
        return pr["corr"], pr["size"], pr["H_gt"]
    if workload == "essential_planar":
        pr = S.two_view_pair(seed, n=n, inlier_ratio=ratio, planar_motion=True)
        return pr["corr"], pr["size"], pr
    pr = S.two_view_pair(seed, n=n, inlier_ratio=ratio)
    return pr["corr"], pr["size"], pr


def _draw_sizes(w, pairs, seed0):
    if isinstance(w["n"], tuple) or isinstance(w["ratio"], tuple):
        rng = np.random.Generator(np.random.PCG64(seed0 + 7919))
        ns = (np.exp(rng.uniform(np.log(w["n"][0]), np.log(w["n"][1]), pairs)).astype(int)
              if isinstance(w["n"], tuple) else np.full(pairs, w["n"]))
        ratios = rng.uniform(w["ratio"][0], w["ratio"][1], pairs)
    else:
        ns = np.full(pairs, w["n"])
        ratios = np.full(pairs, w["ratio"])
    return ns, ratios


def _generate(jobs):
    if len(jobs) >= 256:
        import multiprocessing as mp
        with mp.get_context("spawn").Pool(max(1, min(16, os.cpu_count() or 1))) as pool:
            return pool.map(_gen_pair, jobs, chunksize=16)
    return [_gen_pair(j) for j in jobs]


def build_pairs(workload, pairs, seed0):
    """Returns (corr, offsets, sizes, ground truths, K [P, 18] or None)."""
    w = WORKLOADS[workload]
    ns, ratios = _draw_sizes(w, pairs, seed0)
    out = _generate([(workload, seed0 + i, int(ns[i]), float(ratios[i])) for i in range(pairs)])
    corr = [c for c, _, _ in out]
    sizes = [z for _, z, _ in out]
    gts = [g for _, _, g in out]
    Ks = ([np.concatenate([g["K"].ravel(), g["K"].ravel()]) for g in gts]
          if workload in ("essential", "essential_planar") else [])
    offsets = np.zeros(pairs + 1, np.int64)
    offsets[1:] = np.cumsum([len(c) for c in corr])
    K = np.ascontiguousarray(np.array(Ks), np.float64) if Ks else None
    return np.ascontiguousarray(np.concatenate(corr), np.float64), offsets, np.array(sizes), gts, K


def build_serving_groups(pairs, seed0):
    """The serving mix, grouped by kind: a list of dicts (name, kind,
    threshold, lam, ids, corr, offsets, sizes, K, gts); pair i has kind i mod 3."""
    w = WORKLOADS["serving"]
    ns, ratios = _draw_sizes(w, pairs, seed0)
    out = _generate([(SERVING_KINDS[i % 3][0], seed0 + i, int(ns[i]), float(ratios[i])) for i in range(pairs)])
    groups = []
    for k, (name, kind, thr, lam) in enumerate(SERVING_KINDS):
        ids = np.arange(k, pairs, 3)
        c = [out[i][0] for i in ids]
        off = np.zeros(len(ids) + 1, np.int64)
        off[1:] = np.cumsum([len(x) for x in c])
        gts = [out[i][2] for i in ids]
        K = None
        if kind == _abi.GCR_ESSENTIAL:
            K = np.ascontiguousarray([np.concatenate([g["K"].ravel(), g["K"].ravel()]) for g in gts])
        groups.append(dict(name=name, kind=kind, threshold=thr, lam=lam, ids=ids,
                           corr=np.ascontiguousarray(np.concatenate(c), np.float64), offsets=off,
                           sizes=np.array([out[i][1] for i in ids]), K=K, gts=gts))
    return groups


def params_for(workload, seed=0):
    w = WORKLOADS[workload]
    return _abi.Params(threshold=w["threshold"], confidence=0.99, spatial_coherence_weight=w["lam"],
                       neighborhood_size=w["grid"], max_iterations=10000, min_iterations=50,
                       sampler=w["sampler"], neighborhood=0, lo_number=50, seed=seed,
                       scoring=w.get("scoring", _abi.GCR_SCORING_MSAC))


def serving_params(g, iters, grid=16):
    return _abi.Params(threshold=g["threshold"], confidence=0.99, spatial_coherence_weight=g["lam"],
                       neighborhood_size=grid, max_iterations=iters, min_iterations=min(50, iters), sampler=0,
                       neighborhood=0, lo_number=50, seed=0, scoring=_abi.GCR_SCORING_MSAC)


def size_array(sizes):
    z = np.zeros(len(sizes), _abi.SIZE_DTYPE)
    z["h1"], z["w1"], z["h2"], z["w2"] = sizes[:, 0], sizes[:, 1], sizes[:, 2], sizes[:, 3]
    return z


def model_errors(workload, models, gts, limit=64):
    """Median-ready model errors against ground truth on the first `limit` pairs
    (H: RMS transfer px; F: mean Sampson px of clean correspondences)."""
    if workload in ("homography", "homography_sift"):
        return [S.homography_error(m / m[2, 2] if abs(m[2, 2]) > 1e-12 else m, g) for m, g in zip(models, gts)]
    if workload in ("fundamental", "fundamental_affine", "fundamental_sift"):
        return [S.fundamental_error(m, g, n=200) for m, g in list(zip(models, gts))[:limit]]
    if workload == "learned":
        return [S.fundamental_error(m, g, n=100) for m, g in zip(models, gts)]
    if workload in ("essential", "essential_planar"):
        return [S.essential_error(m, g) for m, g in zip(models, gts)]
    return []


def serving_errors(name, models, gts):
    if name == "homography":
        return [S.homography_error(m / m[2, 2] if abs(m[2, 2]) > 1e-12 else m, g["H_gt"] if isinstance(g, dict)
                                   else g) for m, g in zip(models, gts)]
    if name == "fundamental":
        return [S.fundamental_error(m, g, n=100) for m, g in zip(models, gts)]
    return [S.essential_error(m, g) for m, g in zip(models, gts)]


def equal_error(e_plain, e_learned):
    """The plain form's median error is no worse than the learned form's, within
    5 % relative or 0.05 absolute (px or deg)."""
    return e_plain <= e_learned * 1.05 or e_plain <= e_learned + 0.05


class ClockSampler:
    """nvidia-smi clock/throttle sampling during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.proc = None
        self.path = None

    def start(self):
        try:
            fd, self.path = tempfile.mkstemp(suffix=".csv")
            os.close(fd)
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except (OSError, FileNotFoundError):
            self.proc = None

    def stop(self):
        if self.proc is None:
            return None
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        rows = []
        for line in open(self.path):
            parts = [p.strip() for p in line.split(",")]
            if len(parts) >= 9:
                rows.append(parts)
        os.unlink(self.path)
        if not rows:
            return None
        sm = [float(r[1]) for r in rows if r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in rows if r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[k] for r in rows for k in range(4) if r[5 + k].strip() == "Active"})
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(rows)}


def fp32_peak_tflops(torch):
    """Measured FP32 CUDA-core peak: cuBLAS SGEMM 8192^3 with TF32 disabled."""
    torch.backends.cuda.matmul.allow_tf32 = False
    a = torch.randn(8192, 8192, device="cuda")
    b = torch.randn(8192, 8192, device="cuda")
    for _ in range(2):
        a @ b
    torch.cuda.synchronize()
    best = 0.0
    for _ in range(5):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        a @ b
        e1.record()
        e1.synchronize()
        best = max(best, 2 * 8192 ** 3 / (e0.elapsed_time(e1) * 1e-3) / 1e12)
    del a, b
    return best


def replica_shard(workload, pairs, rank):
    """The batch and sampler seeds of one replica: every rank runs its own
    independent pairs (weak scaling, no collective on the data path)."""
    corr, offsets, sizes, gts, K = build_pairs(workload, pairs, 1000003 * rank)
    seeds = np.arange(pairs, dtype=np.uint64) + np.uint64(pairs * rank)
    return corr, offsets, sizes, gts, K, seeds


def aggregate_rate(units_per_rank, seconds, world, dist=None, device="cpu"):
    """Whole-job rate over replicas: units of all ranks divided by the slowest
    rank's time (max over ranks)."""
    t = seconds
    if dist is not None:
        import torch
        tt = torch.tensor([seconds], device=device, dtype=torch.float64)
        dist.all_reduce(tt, op=dist.ReduceOp.MAX)
        t = float(tt.item())
    return units_per_rank * world / t, t


def fp64_peak_tflops(torch):
    """Measured FP64 peak: cuBLAS DGEMM 4096^3."""
    a = torch.randn(4096, 4096, device="cuda", dtype=torch.float64)
    b = torch.randn(4096, 4096, device="cuda", dtype=torch.float64)
    a @ b
    torch.cuda.synchronize()
    best = 0.0
    for _ in range(3):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        a @ b
        e1.record()
        e1.synchronize()
        best = max(best, 2 * 4096 ** 3 / (e0.elapsed_time(e1) * 1e-3) / 1e12)
    del a, b
    return best


def cpu_baseline(workload, corr, offsets, sizes, p, K=None, target_s=10.0, max_pairs=1 << 30):
    """The oracle (CPU restatement of the reference path) on all host cores,
    on a bounded sample of the same workload. Returns (pairs/s, cores, sample)."""
    return cpu_baseline_kind(WORKLOADS[workload]["kind"], corr, offsets, sizes, p, K, target_s, max_pairs)


def cpu_baseline_kind(kind, corr, offsets, sizes, p, K=None, target_s=10.0, max_pairs=1 << 30, stride=1):
    """`stride` > 1 samples every stride-th pair of the batch (a stratified
    sample when the batch is in random size order)."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle
    threads = os.cpu_count() or 1
    P = len(offsets) - 1
    pool = np.arange(0, P, max(1, stride))

    def run(k):
        # k pairs, cycling over the sampled pairs when k exceeds them
        idx = pool[np.arange(k) % len(pool)]
        lens = np.diff(offsets)[idx]
        off = np.zeros(k + 1, np.int64)
        off[1:] = np.cumsum(lens)
        c = np.concatenate([corr[offsets[i]:offsets[i + 1]] for i in idx])
        _, _, _, t = oracle.find_batch(kind, c, off, size_array(sizes[idx]), p, seeds=idx.astype(np.uint64),
                                       K=None if K is None else np.ascontiguousarray(K[idx]), threads=threads)
        return k, t

    k, t = run(max(2 * threads, 8))
    rate = k / max(t, 1e-9)
    k2 = int(min(max_pairs, max(k, rate * target_s)))
    if k2 > k:
        k, t = run(k2)
    what = "pairs cycling over the step's batch" if stride <= 1 else f"pairs cycling over every {stride}th pair"
    return k / t, threads, f"{k} {what} ({t:.1f} s)"


def timed_steps(torch, fns, steps, flush, stream):
    """Runs `steps` steps; a step calls every function of `fns` in order with a
    CUDA event after each. Returns the total milliseconds of each part."""
    parts = [0.0] * len(fns)
    for _ in range(steps):
        flush.fill_(1)
        ev = [torch.cuda.Event(enable_timing=True) for _ in range(len(fns) + 1)]
        ev[0].record(stream)
        for k, fn in enumerate(fns):
            fn()
            ev[k + 1].record(stream)
        ev[-1].synchronize()
        for k in range(len(fns)):
            parts[k] += ev[k].elapsed_time(ev[k + 1])
    return parts


def vp(t):
    return ctypes.c_void_p(t.data_ptr())


def tune_shape(torch, args, kind, d_corr, offsets, sizes, params, seeds, K=None, candidates=None, lo_precision=None):
    """Autotunes the engine's launch shape on the first pairs of the batch
    (results are identical for every shape) and records it in the tuning
    cache. Returns the gcr_tuning table for the whole batch and a summary."""
    P = len(offsets) - 1
    # the calibration batch is the step's own batch unless limited: the best
    # shape depends on how many waves of pairs the CTAs run
    n = P if args.tune_pairs <= 0 else min(P, args.tune_pairs)
    max_n = int(np.diff(offsets).max())
    if args.no_tune:
        return [], {"shape": "defaults (256 calls per batch, CTAs per SM as the occupancy allows, caller's order)"}
    best, timings = autotune.tune(kind, d_corr, offsets[:n + 1], sizes[:n], params, seeds[:n],
                                  None if K is None else K[:n], candidates=candidates or autotune.CANDIDATES,
                                  repeats=1, lo_precision=lo_precision, staged=candidates is None)
    gpu = autotune.gpu_name()
    try:
        autotune.save_cache(autotune.record(autotune.load_cache(), gpu, kind, max_n, best, timings))
    except OSError:
        pass
    row = _abi.Tuning(kind=int(kind), max_n=max_n, batch_calls=best[0], ctas_per_sm=best[1], order=best[2],
                      reserved=0)
    summary = {"batch_calls": best[0], "ctas_per_sm": best[1], "order": ["caller", "largest first"][best[2]],
               "calibration_pairs": n, "candidates": len(timings),
               "search": "staged (CTAs per SM x order at 256 calls, then calls per batch)" if candidates is None
               else "given candidates",
               "calibration_ms": {f"{c[0]}/{c[1]}/{c[2]}": round(t, 3) for c, t in sorted(timings.items())}}
    return [row], summary


def plain_budget_sweep(torch, lib, d_corr, offsets, sizes, gts, seeds, P, budgets, flush, learned_eval):
    """The plain form (uniform sampler) on the first P pairs at each iteration
    budget: pairs/s of one launch and the median model error; the learned form
    on the same pairs through `learned_eval(P) -> (pairs/s, median error)`."""
    off = np.ascontiguousarray(offsets[:P + 1])
    total = int(off[-1])
    ctx = ctypes.c_void_p()
    assert lib.gcr_context_create(ctypes.byref(ctx)) == 0, _abi.last_error()
    pm = torch.zeros(P * 9, dtype=torch.float64, device="cuda")
    pk = torch.zeros(total, dtype=torch.uint8, device="cuda")
    ps = torch.zeros(P * _abi.STATS_DTYPE.itemsize, dtype=torch.uint8, device="cuda")
    sz = size_array(sizes[:P])
    stream = torch.cuda.current_stream()
    rows = []
    for it in budgets:
        p = params_for("learned")
        p.max_iterations = int(it)
        flush.fill_(1)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        rc = lib.gcr_batch_run_device(ctx, _abi.GCR_FUNDAMENTAL, P, vp(d_corr), _abi.ptr(off), None, _abi.ptr(sz),
                                      ctypes.byref(p), _abi.ptr(seeds[:P]), vp(pm), vp(pk), vp(ps),
                                      ctypes.c_void_p(stream.cuda_stream))
        assert rc == 0, _abi.last_error()
        e1.record(stream)
        e1.synchronize()
        ms = e0.elapsed_time(e1)
        st = np.frombuffer(ps.cpu().numpy().tobytes(), _abi.STATS_DTYPE)
        err = model_errors("learned", pm.cpu().numpy().reshape(P, 3, 3), gts[:P])
        rows.append({"max_iterations": int(it), "pairs_per_s": P / ms * 1e3, "median_model_error": float(np.median(err)),
                     "iterations_mean": float(st["iteration_number"].mean())})
    lib.gcr_context_destroy(ctx)
    v_l, e_l = learned_eval(P)
    reached = [r for r in rows if equal_error(r["median_model_error"], e_l)]
    out = {"pairs": P, "plain": rows, "learned": {"pairs_per_s": v_l, "median_model_error": e_l},
           "criterion": "plain median error <= learned median error x 1.05 or + 0.05 px"}
    if reached:
        r = reached[0]
        out["plain_budget_at_equal_error"] = r["max_iterations"]
        out["learned_over_plain_at_equal_error"] = v_l / r["pairs_per_s"]
    else:
        r = rows[-1]
        out["plain_budget_at_equal_error"] = None
        out["learned_over_plain_lower_bound"] = v_l / r["pairs_per_s"]
        out["note"] = (f"plain did not reach equal error at <= {r['max_iterations']} iterations "
                       f"(median {r['median_model_error']:.3g} px vs learned {e_l:.3g} px); the ratio to the "
                       f"largest budget measured is a lower bound of the ratio at equal error")
    return out


def run_learned(args, P, w, cfg, world, rank, local_rank, dist, torch):
    """The learned-proposal batched form against the plain form on the same
    pairs: each step replays CUDA graphs of (features + MLP + per-pair order)
    and (PROSAC engine launch + mask mapping); the plain form replays its
    engine launch with the uniform sampler and the reference budget."""
    from pygcransac.learned import LearnedBatch, LearnedProposal
    lib = _abi.load()
    corr, offsets, sizes, gts, K, seeds = replica_shard(args.workload, P, rank)
    kind = w["kind"]
    if os.path.exists(CHECKPOINT):
        net = LearnedProposal.load(CHECKPOINT)
        cfg["network"] = (f"checkpoint trained on {net.info.get('labelled_pairs')} pairs at "
                          f"{net.info.get('inlier_ratio')} inlier ratio, labels = {net.info.get('labels')}")
    else:
        from pygcransac.train_proposal import train
        net, _ = train(pairs=2048, out=None, log=lambda m: None)
        cfg["network"] = "no checkpoint: trained before timing on 2048 pairs labelled by the plain method"
    cfg["learned_iterations"] = w["learned_iters"]
    stream = torch.cuda.current_stream()
    flush = torch.empty(256 << 20, dtype=torch.uint8, device="cuda")
    d_corr = torch.from_numpy(corr).cuda()
    total = int(offsets[-1])

    # plain form
    ctx_p = ctypes.c_void_p()
    assert lib.gcr_context_create(ctypes.byref(ctx_p)) == 0, _abi.last_error()
    p_plain = params_for(args.workload)
    rows, cfg["tuning_plain"] = tune_shape(torch, args, kind, d_corr, offsets, sizes, p_plain, seeds)
    autotune.set_table(ctx_p, rows)
    pm = torch.zeros(P * 9, dtype=torch.float64, device="cuda")
    pk = torch.zeros(total, dtype=torch.uint8, device="cuda")
    ps = torch.zeros(P * _abi.STATS_DTYPE.itemsize, dtype=torch.uint8, device="cuda")
    sz = size_array(sizes)
    rc = lib.gcr_batch_prepare(ctx_p, kind, P, vp(d_corr), _abi.ptr(offsets), None, _abi.ptr(sz),
                               ctypes.byref(p_plain), _abi.ptr(seeds), vp(pm), vp(pk), vp(ps))
    assert rc == 0, _abi.last_error()
    cap = torch.cuda.Stream()
    g_plain = torch.cuda.CUDAGraph()
    with torch.cuda.stream(cap):
        with torch.cuda.graph(g_plain, stream=cap):
            assert lib.gcr_batch_launch(ctx_p, ctypes.c_void_p(cap.cuda_stream)) == 0, _abi.last_error()

    # learned form: propose (3 kernels) and engine + mask mapping, two graphs
    p_l = params_for(args.workload)
    p_l.max_iterations = w["learned_iters"]
    p_l.min_iterations = min(50, w["learned_iters"])
    p_l.lo_number = args.learned_lo
    cfg["learned_lo_number"] = args.learned_lo
    lo_prec = _abi.GCR_LO_FP32 if args.learned_lo_precision == "fp32" else _abi.GCR_LO_FP64
    cfg["learned_lo_precision"] = (
        "fp32 per-correspondence terms in every fundamental-matrix fit after the minimal solver "
        "(LO trials, IRLS, final refit, epilogue), fp64 reductions and solves" if lo_prec == _abi.GCR_LO_FP32
        else "fp64")
    b = LearnedBatch(net, kind, d_corr, offsets, sizes, p_l, seeds, lo_precision=lo_prec)
    # the learned engine's shape, tuned on the ordered correspondences
    assert lib.gcr_learned_propose(vp(d_corr), vp(b.d_off), vp(b.d_sz), P, b.max_n, total, vp(net.bf16),
                                   vp(b.d_feat), vp(b.d_logits), vp(b.d_sorted), vp(b.d_perm), None) == 0
    torch.cuda.synchronize()
    p_tune = _abi.Params(**{f: getattr(p_l, f) for f, _ in p_l._fields_})
    p_tune.sampler = 1
    rows, cfg["tuning"] = tune_shape(torch, args, kind, b.d_sorted, offsets, sizes, p_tune, seeds,
                                     lo_precision=lo_prec)
    autotune.set_table(b.ctx, rows)
    b.prepare()
    g_prop, g_eng = torch.cuda.CUDAGraph(), torch.cuda.CUDAGraph()
    sp = ctypes.c_void_p(cap.cuda_stream)
    with torch.cuda.stream(cap):
        with torch.cuda.graph(g_prop, stream=cap):
            assert lib.gcr_learned_propose(vp(d_corr), vp(b.d_off), vp(b.d_sz), P, b.max_n, total, vp(net.bf16),
                                           vp(b.d_feat), vp(b.d_logits), vp(b.d_sorted), vp(b.d_perm), sp) == 0
        with torch.cuda.graph(g_eng, stream=cap):
            assert lib.gcr_batch_launch(b.ctx, sp) == 0, _abi.last_error()
            engine_launches = int(lib.gcr_last_launch_count())
            assert lib.gcr_learned_unpermute_mask(vp(b.d_sorted_masks), vp(b.d_perm), vp(b.d_off), vp(b.d_por),
                                                  total, vp(b.d_masks), sp) == 0
    launches_per_step = 3 + engine_launches + 1

    for _ in range(args.warmup):
        g_plain.replay()
        g_prop.replay()
        g_eng.replay()
    torch.cuda.synchronize()
    plain_ms = sum(timed_steps(torch, [g_plain.replay], args.steps, flush, stream))
    clocks = ClockSampler(local_rank)
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    clocks.start()
    prop_ms, eng_ms = timed_steps(torch, [g_prop.replay, g_eng.replay], args.steps, flush, stream)
    torch.cuda.synchronize()
    clk = clocks.stop()
    total_ms = prop_ms + eng_ms
    value, _ = aggregate_rate(P * args.steps, total_ms / 1e3, world, dist, "cuda")
    plain_value, _ = aggregate_rate(P * args.steps, plain_ms / 1e3, world, dist, "cuda")

    models, _, stats = b.results()
    err_l = model_errors(args.workload, models, gts)
    lo_compare = None
    if not args.no_lo_compare:
        # the same ordered pairs through the engine in the other LO precision:
        # engine time and median model error of each
        other = _abi.GCR_LO_FP64 if lo_prec == _abi.GCR_LO_FP32 else _abi.GCR_LO_FP32
        bo = LearnedBatch(net, kind, d_corr, offsets, sizes, p_l, seeds, lo_precision=other)
        autotune.set_table(bo.ctx, rows)
        bo.prepare()
        assert lib.gcr_learned_propose(vp(d_corr), vp(bo.d_off), vp(bo.d_sz), P, bo.max_n, total, vp(net.bf16),
                                       vp(bo.d_feat), vp(bo.d_logits), vp(bo.d_sorted), vp(bo.d_perm), None) == 0
        g_other = torch.cuda.CUDAGraph()
        with torch.cuda.stream(cap):
            with torch.cuda.graph(g_other, stream=cap):
                assert lib.gcr_batch_launch(bo.ctx, sp) == 0, _abi.last_error()
                assert lib.gcr_learned_unpermute_mask(vp(bo.d_sorted_masks), vp(bo.d_perm), vp(bo.d_off),
                                                      vp(bo.d_por), total, vp(bo.d_masks), sp) == 0
        for _ in range(args.warmup):
            g_other.replay()
        torch.cuda.synchronize()
        other_ms = sum(timed_steps(torch, [g_other.replay], args.steps, flush, stream))
        mo, _, so = bo.results()
        eo = model_errors(args.workload, mo, gts)
        bo.close()
        name = {_abi.GCR_LO_FP32: "fp32", _abi.GCR_LO_FP64: "fp64"}
        lo_compare = {
            name[lo_prec]: {"engine_ms_per_step": eng_ms / args.steps, "median_model_error": float(np.median(err_l)),
                            "status_ok_fraction": float(np.mean(stats["status"] == 0))},
            name[other]: {"engine_ms_per_step": other_ms / args.steps, "median_model_error": float(np.median(eo)),
                          "status_ok_fraction": float(np.mean(so["status"] == 0))},
        }
        f64, f32 = lo_compare["fp64"], lo_compare["fp32"]
        lo_compare["fp64_over_fp32_engine_time"] = f64["engine_ms_per_step"] / f32["engine_ms_per_step"]
        lo_compare["equal_error"] = equal_error(f32["median_model_error"], f64["median_model_error"])
    plain_models = pm.cpu().numpy().reshape(P, 3, 3)
    plain_stats = np.frombuffer(ps.cpu().numpy().tobytes(), _abi.STATS_DTYPE)
    err_p = model_errors(args.workload, plain_models, gts)

    # end to end through the LearnedBatch API: pinned host correspondences in,
    # models, masks and statistics out, every step
    h_corr = torch.from_numpy(corr).pin_memory()
    h_models = torch.empty(P * 9, dtype=torch.float64).pin_memory()
    h_masks = torch.empty(total, dtype=torch.uint8).pin_memory()
    h_stats = torch.empty(P * _abi.STATS_DTYPE.itemsize, dtype=torch.uint8).pin_memory()

    def e2e_step():
        d_corr.copy_(h_corr, non_blocking=True)
        b.launch()
        h_models.copy_(b.d_models, non_blocking=True)
        h_masks.copy_(b.d_masks, non_blocking=True)
        h_stats.copy_(b.d_stats, non_blocking=True)
        torch.cuda.synchronize()

    e2e_step()
    e2e_t = 0.0
    for _ in range(args.steps):
        flush.fill_(1)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        e2e_step()
        e2e_t += time.perf_counter() - t0
    e2e_value, _ = aggregate_rate(P * args.steps, e2e_t, world, dist, "cuda")

    # equal model error: plain budgets against the learned form on one wave of pairs
    sweep = None
    if not args.no_sweep:
        def learned_eval(n):
            bl = LearnedBatch(net, kind, d_corr, offsets[:n + 1], sizes[:n], p_l, seeds[:n], lo_precision=lo_prec)
            autotune.set_table(bl.ctx, rows)
            bl.prepare()
            bl.launch()
            torch.cuda.synchronize()
            flush.fill_(1)
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            bl.launch()
            e1.record(stream)
            e1.synchronize()
            ml, _, _ = bl.results()
            bl.close()
            return n / e0.elapsed_time(e1) * 1e3, float(np.median(model_errors(args.workload, ml, gts[:n])))
        sweep = plain_budget_sweep(torch, lib, d_corr, offsets, sizes, gts, seeds, min(P, args.sweep_pairs),
                                   args.sweep_budgets, flush, learned_eval)
    if rank != 0:
        b.close()
        lib.gcr_context_destroy(ctx_p)
        return None
    n_per = np.diff(offsets)
    peak = fp32_peak_tflops(torch)
    eng_s = eng_ms / args.steps / 1e3
    flops = float(np.sum(stats["models_scored"] * n_per)) * FLOP_PER_RESIDUAL[args.workload]
    mlp_flops = 2.0 * total * (32 * 128 + 2 * 128 * 128 + 128)
    achieved = flops / eng_s / 1e12
    traffic = fp64_work = traffic_note = None
    tp = os.path.join(ROOT, "profiles", "traffic_learned.json")
    if os.path.exists(tp):
        t = json.load(open(tp))
        traffic = t["bytes_per_pair"] * P
        fp64_work = t["fp64_flop_per_pair"] * P
        traffic_note = f"ncu capture of a {t.get('pairs', 152)}-pair launch, scaled to {P} pairs by the pair count"
    peak64 = fp64_peak_tflops(torch)
    line = {
        "metric": METRIC, "value": value, "unit": "pairs/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": total_ms / args.steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": ("fp32 scoring / fp32 per-point LO terms, fp64 solves / bf16 weights, fp32 accumulation (MLP)"
                  if lo_prec == _abi.GCR_LO_FP32 else
                  "fp32 scoring / fp64 solvers / bf16 weights, fp32 accumulation (MLP)"),
        "data": "synthetic", "config": cfg,
        "median_model_error": float(np.median(err_l)),
        "status_ok_fraction": float(np.mean(stats["status"] == 0)),
        "plain": {"value": plain_value, "unit": "pairs/s", "ms_per_step": plain_ms / args.steps,
                  "median_model_error": float(np.median(err_p)),
                  "iterations_mean": float(np.mean(plain_stats["iteration_number"]))},
        "learned_over_plain": value / plain_value,
        "equal_error": sweep,
        "error_unit": "px, mean Sampson distance of 100 noise-free ground-truth correspondences per pair",
        "proposal_ms_per_step": prop_ms / args.steps, "engine_ms_per_step": eng_ms / args.steps,
        "lo_precision": lo_compare,
        "roofline": {"bound": "fp32", "achieved": achieved, "peak": peak, "unit": "TFLOP/s",
                     "frac": achieved / peak if peak else None, "traffic": traffic, "traffic_source": traffic_note,
                     "peak_source": "cuBLAS SGEMM 8192^3, TF32 off, measured in this run",
                     "kernel": "pair engine (PROSAC, learned order)",
                     "work": f"{FLOP_PER_RESIDUAL[args.workload]} FLOP x models_scored x N per pair"},
        "roofline_fp64": None if fp64_work is None else {
            "bound": "fp64", "achieved": fp64_work / eng_s / 1e12, "peak": peak64, "unit": "TFLOP/s",
            "frac": fp64_work / eng_s / 1e12 / peak64, "peak_source": "cuBLAS DGEMM 4096^3, measured in this run",
            "work": "FP64 FLOP per pair executed by the engine kernel (ncu SASS counts, FMA = 2) x pairs"},
        "proposal_flops_per_step": mlp_flops,
        "e2e": {"value": e2e_value, "unit": "pairs/s", "h2d_bytes_per_step": int(corr.nbytes),
                "d2h_bytes_per_step": int(P * 9 * 8 + total + P * _abi.STATS_DTYPE.itemsize)},
        "gpu_launches": int(launches_per_step * args.steps),
        "clocks": clk,
    }
    if not args.no_cpu_baseline and world == 1:
        v, cores, sample = cpu_baseline(args.workload, corr, offsets, sizes, p_plain, None)
        line["cpu_baseline"] = {"value": v, "unit": "pairs/s", "cores": cores, "kind": "port",
                                "sample": sample + "; plain method (uniform sampler, 10000 iterations)"}
    b.close()
    lib.gcr_context_destroy(ctx_p)
    return line


def run_kind(args, workload, P, steps, warmup, world, rank, local_rank, dist, torch, clocks_on=True):
    """One persistent engine launch per step (single model kind), replayed from
    a CUDA graph; `e2e` through gcr_find_batch with pinned host buffers."""
    w = WORKLOADS[workload]
    lib = _abi.load()
    corr, offsets, sizes, gts, K, seeds = replica_shard(workload, P, rank)
    p = params_for(workload)
    kind = w["kind"]
    szs = size_array(sizes)
    d_corr = torch.from_numpy(corr).cuda()
    d_models = torch.zeros(P * 9, dtype=torch.float64, device="cuda")
    d_masks = torch.zeros(int(offsets[-1]), dtype=torch.uint8, device="cuda")
    d_stats = torch.zeros(P * _abi.STATS_DTYPE.itemsize, dtype=torch.uint8, device="cuda")
    flush = torch.empty(256 << 20, dtype=torch.uint8, device="cuda")
    ctx = ctypes.c_void_p()
    assert lib.gcr_context_create(ctypes.byref(ctx)) == 0, _abi.last_error()
    stream = torch.cuda.current_stream()
    rows, tuning = tune_shape(torch, args, kind, d_corr, offsets, sizes, p, seeds, K)
    autotune.set_table(ctx, rows)

    # one persistent launch per batch (plus the K^-1 normalisation for E),
    # prepared once and recorded into a CUDA graph; a step is one replay
    rc = lib.gcr_batch_prepare(ctx, kind, P, vp(d_corr), _abi.ptr(offsets), _abi.ptr(K), _abi.ptr(szs),
                               ctypes.byref(p), _abi.ptr(seeds), vp(d_models), vp(d_masks), vp(d_stats))
    assert rc == 0, _abi.last_error()
    graph = torch.cuda.CUDAGraph()
    cap = torch.cuda.Stream()
    with torch.cuda.stream(cap):
        with torch.cuda.graph(graph, stream=cap):
            rc = lib.gcr_batch_launch(ctx, ctypes.c_void_p(cap.cuda_stream))
    assert rc == 0, _abi.last_error()
    launches_per_step = int(lib.gcr_last_launch_count())

    for _ in range(warmup):
        graph.replay()
    torch.cuda.synchronize()
    clocks = ClockSampler(local_rank) if clocks_on else None
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    if clocks:
        clocks.start()
    total_ms = sum(timed_steps(torch, [graph.replay], steps, flush, stream))
    torch.cuda.synchronize()
    clk = clocks.stop() if clocks else None
    value, _ = aggregate_rate(P * steps, total_ms / 1e3, world, dist, "cuda")
    if dist:
        dist.barrier()

    stats = np.frombuffer(d_stats.cpu().numpy().tobytes(), _abi.STATS_DTYPE)
    models = d_models.cpu().numpy().reshape(P, 3, 3)
    n_per = np.diff(offsets)
    flops = float(np.sum(stats["models_scored"] * n_per)) * FLOP_PER_RESIDUAL[workload]
    errs = model_errors(workload, models, gts)

    # end to end through the host-buffer entry: pinned inputs, copies timed
    h_corr = torch.from_numpy(corr).pin_memory()
    h_models = torch.zeros(P * 9, dtype=torch.float64).pin_memory()
    h_masks = torch.zeros(int(offsets[-1]), dtype=torch.uint8).pin_memory()
    h_stats = torch.zeros(P * _abi.STATS_DTYPE.itemsize, dtype=torch.uint8).pin_memory()

    def e2e_step():
        rc = lib.gcr_find_batch(kind, P, vp(h_corr), _abi.ptr(offsets), _abi.ptr(K), _abi.ptr(szs),
                                ctypes.byref(p), _abi.ptr(seeds), vp(h_models), vp(h_masks), vp(h_stats))
        assert rc == 0, _abi.last_error()

    e2e_step()
    e2e_t = 0.0
    for _ in range(steps):
        flush.fill_(1)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        e2e_step()
        e2e_t += time.perf_counter() - t0
    e2e_value, e2e_t = aggregate_rate(P * steps, e2e_t, world, dist, "cuda")
    lib.gcr_context_destroy(ctx)
    if rank != 0:
        return None
    peak = fp32_peak_tflops(torch)
    achieved = flops / (total_ms / steps / 1e3) / 1e12
    traffic = fp64_work = traffic_note = None
    tp = os.path.join(ROOT, "profiles", f"traffic_{workload}.json")
    if os.path.exists(tp):
        t = json.load(open(tp))
        traffic = t["bytes_per_pair"] * P
        fp64_work = t["fp64_flop_per_pair"] * P
        traffic_note = f"ncu capture of a {t.get('pairs', 152)}-pair launch, scaled to {P} pairs by the pair count"
    peak64 = fp64_peak_tflops(torch)
    line = {
        "value": value, "unit": "pairs/s", "steps": steps, "warmup": warmup, "ms_per_step": total_ms / steps,
        "pairs_per_step": P, "config": {"tuning": tuning},
        "median_model_error": float(np.median(errs)) if errs else None,
        "status_ok_fraction": float(np.mean(stats["status"] == 0)),
        "roofline": {"bound": "fp32", "achieved": achieved, "peak": peak, "unit": "TFLOP/s",
                     "frac": achieved / peak if peak else None, "traffic": traffic, "traffic_source": traffic_note,
                     "peak_source": "cuBLAS SGEMM 8192^3, TF32 off, measured in this run",
                     "work": f"{FLOP_PER_RESIDUAL[workload]} FLOP x models_scored x N per pair"},
        # the FP64 pipe is the unit the kernel keeps busiest (solvers, LO fits):
        # executed FP64 FLOP per pair from the ncu capture in profiles/, over the
        # live DGEMM peak
        "roofline_fp64": None if fp64_work is None else {
            "bound": "fp64", "achieved": fp64_work / (total_ms / steps / 1e3) / 1e12, "peak": peak64,
            "unit": "TFLOP/s", "frac": fp64_work / (total_ms / steps / 1e3) / 1e12 / peak64,
            "peak_source": "cuBLAS DGEMM 4096^3, measured in this run",
            "work": "FP64 FLOP per pair executed by the kernel (ncu SASS counts, FMA = 2) x pairs"},
        "e2e": {"value": e2e_value, "unit": "pairs/s", "h2d_bytes_per_step": int(corr.nbytes),
                "d2h_bytes_per_step": int(P * 9 * 8 + offsets[-1] + P * _abi.STATS_DTYPE.itemsize)},
        "gpu_launches": int(launches_per_step * steps),
        "clocks": clk,
    }
    if not args.no_cpu_baseline and world == 1:
        v, cores, sample = cpu_baseline(workload, corr, offsets, sizes, p, K,
                                        target_s=10.0 if workload == args.workload else 6.0)
        line["cpu_baseline"] = {"value": v, "unit": "pairs/s", "cores": cores, "kind": "port", "sample": sample}
    return line


def run_serving(args, P, steps, warmup, world, rank, local_rank, dist, torch, clocks_on=True):
    """Mixed H / F / E batch: one engine launch per kind, the three kinds on
    their own streams. Learned form = proposal + PROSAC engine + mask mapping
    per kind (one CUDA graph each); plain form = uniform-sampler engine launch
    per kind (one CUDA graph each). Per-pair service times come from the
    engine's global-timer stamps.

    Every device buffer a captured graph reads or writes is owned by the
    kind's record below for the whole run: a graph keeps raw addresses, so a
    buffer released to the caching allocator (and returned to the driver by
    the empty_cache() that graph capture performs) would leave the replay
    writing into freed memory."""
    from pygcransac.learned import LearnedBatch, LearnedProposal
    lib = _abi.load()
    w = WORKLOADS["serving"]
    groups = build_serving_groups(P, 1000003 * rank)
    net = LearnedProposal.load(CHECKPOINT)
    cfg = dict(network="the fundamental-matrix checkpoint, applied to every kind",
               kinds={g["name"]: dict(pairs=int(len(g["ids"])), threshold=g["threshold"],
                                      spatial_coherence_weight=g["lam"]) for g in groups},
               learned_iterations=w["learned_iters"], correspondences="log-uniform 2000-40000",
               inlier_ratio="uniform 5-60 %", grid=w["grid"])
    flush = torch.empty(256 << 20, dtype=torch.uint8, device="cuda")
    main = torch.cuda.current_stream()
    streams = [torch.cuda.Stream() for _ in groups]
    recs = []
    for gi, g in enumerate(groups):
        n_pairs, total = len(g["ids"]), int(g["offsets"][-1])
        rec = dict(group=g, stream=streams[gi])
        rec["d_corr"] = torch.from_numpy(g["corr"]).cuda()
        rec["times_p"] = torch.zeros(2 * n_pairs, dtype=torch.int64, device="cuda")
        rec["times_l"] = torch.zeros(2 * n_pairs, dtype=torch.int64, device="cuda")
        rec["pm"] = torch.zeros(n_pairs * 9, dtype=torch.float64, device="cuda")
        rec["pk"] = torch.zeros(total, dtype=torch.uint8, device="cuda")
        rec["ps"] = torch.zeros(n_pairs * _abi.STATS_DTYPE.itemsize, dtype=torch.uint8, device="cuda")
        rec["seeds"] = np.arange(n_pairs, dtype=np.uint64) + np.uint64(gi * 1000003)
        ctx = ctypes.c_void_p()
        assert lib.gcr_context_create(ctypes.byref(ctx)) == 0
        rec["ctx"] = ctx
        assert lib.gcr_context_set_pair_times(ctx, vp(rec["times_p"])) == 0
        pp = serving_params(g, 10000, w["grid"])
        rows, cfg.setdefault("tuning_plain", {})[g["name"]] = tune_shape(
            torch, args, g["kind"], rec["d_corr"], g["offsets"], g["sizes"], pp, rec["seeds"], g["K"],
            candidates=SERVING_CANDIDATES)
        autotune.set_table(ctx, rows)
        rc = lib.gcr_batch_prepare(ctx, g["kind"], n_pairs, vp(rec["d_corr"]), _abi.ptr(g["offsets"]),
                                   _abi.ptr(g["K"]), _abi.ptr(size_array(g["sizes"])), ctypes.byref(pp),
                                   _abi.ptr(rec["seeds"]), vp(rec["pm"]), vp(rec["pk"]), vp(rec["ps"]))
        assert rc == 0, _abi.last_error()
        rec["g_plain"] = torch.cuda.CUDAGraph()
        with torch.cuda.stream(streams[gi]):
            with torch.cuda.graph(rec["g_plain"], stream=streams[gi]):
                assert lib.gcr_batch_launch(ctx, ctypes.c_void_p(streams[gi].cuda_stream)) == 0
        pl = serving_params(g, w["learned_iters"], w["grid"])
        b = LearnedBatch(net, g["kind"], rec["d_corr"], g["offsets"], g["sizes"], pl, rec["seeds"], g["K"])
        assert lib.gcr_context_set_pair_times(b.ctx, vp(rec["times_l"])) == 0
        assert lib.gcr_learned_propose(vp(rec["d_corr"]), vp(b.d_off), vp(b.d_sz), b.P, b.max_n, b.total,
                                       vp(net.bf16), vp(b.d_feat), vp(b.d_logits), vp(b.d_sorted), vp(b.d_perm),
                                       None) == 0
        torch.cuda.synchronize()
        pt = _abi.Params(**{f: getattr(pl, f) for f, _ in pl._fields_})
        pt.sampler = 1
        rows, cfg.setdefault("tuning", {})[g["name"]] = tune_shape(
            torch, args, g["kind"], b.d_sorted, g["offsets"], g["sizes"], pt, rec["seeds"], g["K"],
            candidates=SERVING_CANDIDATES)
        autotune.set_table(b.ctx, rows)
        b.prepare()
        rec["batch"] = b
        rec["g_learned"] = torch.cuda.CUDAGraph()
        with torch.cuda.stream(streams[gi]):
            with torch.cuda.graph(rec["g_learned"], stream=streams[gi]):
                rec["launches_learned"] = b.launch(streams[gi])
        recs.append(rec)

    def step(key):
        start = torch.cuda.Event(enable_timing=True)
        stop = torch.cuda.Event(enable_timing=True)
        flush.fill_(1)
        start.record(main)
        for r in recs:
            r["stream"].wait_event(start)
            with torch.cuda.stream(r["stream"]):
                r[key].replay()
        for r in recs:
            e = torch.cuda.Event()
            e.record(r["stream"])
            main.wait_event(e)
        stop.record(main)
        stop.synchronize()
        return start.elapsed_time(stop)

    def lat(key):
        t = np.concatenate([r[key].cpu().numpy().reshape(-1, 2) for r in recs]).astype(np.float64)
        service = (t[:, 1] - t[:, 0]) / 1e6
        done = (t[:, 1] - t[:, 0].min()) / 1e6
        return {"service_ms_p50": float(np.percentile(service, 50)), "service_ms_p99": float(np.percentile(service, 99)),
                "completion_ms_p50": float(np.percentile(done, 50)), "completion_ms_p99": float(np.percentile(done, 99))}

    for _ in range(warmup):
        step("g_plain")
        step("g_learned")
    plain_ms = sum(step("g_plain") for _ in range(steps))
    plain_lat = lat("times_p")
    clocks = ClockSampler(local_rank) if clocks_on else None
    torch.cuda.synchronize()
    if clocks:
        clocks.start()
    learned_ms = sum(step("g_learned") for _ in range(steps))
    clk = clocks.stop() if clocks else None
    learned_lat = lat("times_l")
    value, _ = aggregate_rate(P * steps, learned_ms / 1e3, world, dist, "cuda")
    plain_value, _ = aggregate_rate(P * steps, plain_ms / 1e3, world, dist, "cuda")
    errs_l, errs_p, ok_l, ok_p = {}, {}, [], []
    for r in recs:
        g = r["group"]
        ml, _, stl = r["batch"].results()
        mp = r["pm"].cpu().numpy().reshape(-1, 3, 3)
        stp = np.frombuffer(r["ps"].cpu().numpy().tobytes(), _abi.STATS_DTYPE)
        errs_l[g["name"]] = float(np.median(serving_errors(g["name"], ml, g["gts"])))
        errs_p[g["name"]] = float(np.median(serving_errors(g["name"], mp, g["gts"])))
        ok_l.append(stl["status"] == 0)
        ok_p.append(stp["status"] == 0)

    # end to end: pinned host correspondences in, models / masks / stats out
    for r in recs:
        b = r["batch"]
        r["h_corr"] = torch.from_numpy(r["group"]["corr"]).pin_memory()
        r["h_out"] = (torch.empty(b.P * 9, dtype=torch.float64).pin_memory(),
                      torch.empty(b.total, dtype=torch.uint8).pin_memory(),
                      torch.empty(b.P * _abi.STATS_DTYPE.itemsize, dtype=torch.uint8).pin_memory())

    def e2e_step():
        for r in recs:
            b, o = r["batch"], r["h_out"]
            with torch.cuda.stream(r["stream"]):
                r["d_corr"].copy_(r["h_corr"], non_blocking=True)
                b.launch(r["stream"])
                o[0].copy_(b.d_models, non_blocking=True)
                o[1].copy_(b.d_masks, non_blocking=True)
                o[2].copy_(b.d_stats, non_blocking=True)
        torch.cuda.synchronize()

    e2e_step()
    e2e_t = 0.0
    for _ in range(steps):
        flush.fill_(1)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        e2e_step()
        e2e_t += time.perf_counter() - t0
    e2e_value, _ = aggregate_rate(P * steps, e2e_t, world, dist, "cuda")
    line = None
    if rank == 0:
        line = {
            "value": value, "unit": "pairs/s", "steps": steps, "warmup": warmup, "ms_per_step": learned_ms / steps,
            "pairs_per_step": P, "config": cfg,
            "median_model_error": errs_l, "status_ok_fraction": float(np.mean(np.concatenate(ok_l))),
            "latency": learned_lat,
            "plain": {"value": plain_value, "unit": "pairs/s", "ms_per_step": plain_ms / steps,
                      "median_model_error": errs_p, "status_ok_fraction": float(np.mean(np.concatenate(ok_p))),
                      "latency": plain_lat},
            "learned_over_plain": value / plain_value,
            "error_unit": "H: RMS transfer px; F: mean Sampson px; E: max(rotation, translation) deg",
            "e2e": {"value": e2e_value, "unit": "pairs/s",
                    "h2d_bytes_per_step": int(sum(r["group"]["corr"].nbytes for r in recs)),
                    "d2h_bytes_per_step": int(sum(o.numel() * o.element_size() for r in recs for o in r["h_out"]))},
            "gpu_launches": int(sum(r["launches_learned"] for r in recs) * steps),
            "clocks": clk,
        }
        if not args.no_cpu_baseline and world == 1:
            # the oracle (plain method) per kind on a bounded sample of its pairs
            rates, samples, cores = [], [], 1
            for r in recs:
                g = r["group"]
                v, cores, sample = cpu_baseline_kind(g["kind"], g["corr"], g["offsets"], g["sizes"],
                                                     serving_params(g, 10000, w["grid"]), g["K"], target_s=6.0,
                                                     stride=7)
                rates.append(v)
                samples.append(f"{g['name']}: {sample}")
            line["cpu_baseline"] = {"value": 3.0 / sum(1.0 / v for v in rates), "unit": "pairs/s", "cores": cores,
                                    "kind": "port", "sample": "; ".join(samples) + "; combined as equal thirds"}
    for r in recs:
        lib.gcr_context_destroy(r["ctx"])
        r["batch"].close()
    return line


def describe(workload, P, world):
    w = WORKLOADS[workload]
    if workload == "essential":
        desc = (f"{workload}: {P} calibrated pairs/step x {w['n'][0]}-{w['n'][1]} (log-uniform) correspondences, "
                f"{int(w['ratio'][0]*100)}-{int(w['ratio'][1]*100)}% inliers, MAGSAC++")
    elif workload == "learned":
        desc = (f"learned: {P} fundamental-matrix pairs/step x {w['n']} correspondences, "
                f"{int(w['ratio'][0]*100)}-{int(w['ratio'][1]*100)}% inliers; learned order -> PROSAC "
                f"({w['learned_iters']} iterations) vs plain uniform sampler (10000 iterations)")
    elif workload == "serving":
        desc = (f"serving: {P} pairs/step split evenly across H / F / E, 2000-40000 (log-uniform) correspondences, "
                f"5-60% inliers; learned order -> PROSAC ({w['learned_iters']} iterations) vs plain uniform "
                f"sampler (10000 iterations), one launch per kind on three streams")
    else:
        desc = f"{workload}: {P} pairs/step x {w['n']} correspondences, {int(w['ratio']*100)}% inliers"
    cfg = {"workload": desc, "pairs_per_step": P, "correspondences": w["n"], "threshold": w["threshold"],
           "sampler": w["sampler"], "grid": w["grid"], "spatial_coherence_weight": w["lam"],
           "scoring": "MAGSAC++" if w.get("scoring") == _abi.GCR_SCORING_MAGSAC else "MSAC",
           "launch": "one persistent engine launch per step, replayed from a CUDA graph",
           "l2": "flushed between steps (256 MiB write)",
           "parallelism": f"replicas x{world}"}
    return cfg


def reference_arm(args, P, cfg):
    """The CPU restatement of the reference path (plain method) on all host
    cores, on bounded samples of the workload."""
    w = WORKLOADS[args.workload]
    vals = []
    if args.workload == "serving":
        groups = build_serving_groups(P, 0)
        for it in range(args.warmup + args.steps):
            rates, samples = [], []
            for g in groups:
                v, cores, sample = cpu_baseline_kind(g["kind"], g["corr"], g["offsets"], g["sizes"],
                                                     serving_params(g, 10000, w["grid"]), g["K"],
                                                     target_s=1.0 if it < args.warmup else 4.0, stride=7)
                rates.append(v)
                samples.append(f"{g['name']}: {sample}")
            if it >= args.warmup:
                vals.append(3.0 / sum(1.0 / r for r in rates))
        sample = "; ".join(samples) + "; combined as equal thirds"
    else:
        corr, offsets, sizes, gts, K = build_pairs(args.workload, P, 0)
        p = params_for(args.workload)
        for _ in range(args.warmup):
            cpu_baseline(args.workload, corr, offsets, sizes, p, K, target_s=1.0, max_pairs=64)
        for _ in range(args.steps):
            v, cores, sample = cpu_baseline(args.workload, corr, offsets, sizes, p, K, target_s=8.0)
            vals.append(v)
    v = float(np.median(vals))
    return {"metric": METRIC, "value": v, "unit": "pairs/s", "n_gpus": args.gpus, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": 1e3 * P / v, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic", "config": cfg, "impl": "reference",
            "cpu_baseline": {"value": v, "unit": "pairs/s", "cores": cores, "kind": "port", "sample": sample},
            "e2e": {"value": v, "unit": "pairs/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gcr", choices=["gcr", "reference"])
    ap.add_argument("--workload", default="learned", choices=sorted(WORKLOADS))
    ap.add_argument("--pairs", type=int, default=0)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--learned-lo", type=int, default=50,
                    help="LO trials of the learned form (the reference's default is 50)")
    ap.add_argument("--learned-lo-precision", default="fp32", choices=["fp32", "fp64"],
                    help="arithmetic of the learned form's fundamental-matrix fits after the minimal solver")
    ap.add_argument("--no-lo-compare", action="store_true",
                    help="skip the learned engine's run in the other LO precision")
    ap.add_argument("--no-side", action="store_true", help="skip the other workloads")
    ap.add_argument("--side-steps", type=int, default=3, help="timed steps of each other workload")
    ap.add_argument("--no-sweep", action="store_true", help="skip the plain-budget sweep of the learned workload")
    ap.add_argument("--sweep-pairs", type=int, default=304)
    ap.add_argument("--sweep-budgets", default=",".join(str(b) for b in SWEEP_BUDGETS))
    ap.add_argument("--no-tune", action="store_true", help="keep the default launch shape (no autotuning)")
    ap.add_argument("--tune-pairs", type=int, default=0,
                    help="calibration pairs of the autotuner (0: the whole batch of the step)")
    args = ap.parse_args()
    args.sweep_budgets = [int(float(x)) for x in args.sweep_budgets.split(",") if x]

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local_rank = int(os.environ.get("LOCAL_RANK", "0"))
    w = WORKLOADS[args.workload]
    P = args.pairs or w["pairs"]
    cfg = describe(args.workload, P, world)

    if args.impl == "reference":
        if rank == 0:
            print(json.dumps(reference_arm(args, P, cfg)))
        return

    import torch
    torch.cuda.set_device(local_rank)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=torch.device("cuda", local_rank))

    if args.workload == "learned":
        line = run_learned(args, P, w, cfg, world, rank, local_rank, dist, torch)
    elif args.workload == "serving":
        sub = run_serving(args, P, args.steps, args.warmup, world, rank, local_rank, dist, torch)
        line = None if sub is None else {"metric": METRIC, **sub}
    else:
        sub = run_kind(args, args.workload, P, args.steps, args.warmup, world, rank, local_rank, dist, torch)
        line = None if sub is None else {"metric": METRIC, **sub}
    if line is not None:
        line.update({"n_gpus": world, "steps": args.steps, "warmup": args.warmup, "higher_is_better": True,
                     "scaling": "weak", "vs_baseline": None, "data": "synthetic"})
        line.setdefault("dtype", "fp32 scoring / fp64 solvers" +
                        (" / bf16 weights, fp32 accumulation (MLP)" if args.workload == "serving" else ""))
        if args.workload != "learned":
            line["config"] = {**cfg, **line.get("config", {})}

    # the other workloads, a few steps each (same replicas and timing rules)
    if not args.no_side:
        side = {}
        for name in ("homography", "homography_sift", "fundamental", "fundamental_affine", "fundamental_sift",
                     "essential", "essential_planar", "serving"):
            if name == args.workload:
                continue
            sw = WORKLOADS[name]
            if name == "serving":
                sub = run_serving(args, sw["pairs"], args.side_steps, max(3, args.warmup), world, rank, local_rank,
                                  dist, torch, clocks_on=False)
            else:
                sub = run_kind(args, name, sw["pairs"], args.side_steps, max(3, args.warmup), world, rank, local_rank,
                               dist, torch, clocks_on=False)
            if sub is not None:
                sub["config"] = {**describe(name, sw["pairs"], world), **sub.get("config", {})}
                side[name] = sub
        if line is not None:
            line["workloads"] = side
    if line is not None:
        print(json.dumps(line))
    if dist:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
