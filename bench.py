#!/usr/bin/env python
"""Throughput benchmark of the GB300 Graph-Cut RANSAC engine.

Default workload (`learned`): 1216 hard fundamental-matrix pairs per step
(4000 correspondences, 5-10 % inliers). `value` is the pairs/s of the
learned-proposal batched form: each step replays two CUDA graphs, the proposal
(neighbour features, MLP, per-pair ordering: three kernels) and the engine
(one persistent PROSAC launch with a 50-iteration budget, plus the mask
mapping); the plain form (uniform sampler, the reference's 10000-iteration
budget, one persistent launch) is timed on the same pairs and reported under
`plain`, with both median model errors. The other workloads (`homography`,
`fundamental`, `essential`) time one persistent engine launch per step.
Correspondences are resident in HBM for `value` (CUDA events on the launching
stream, L2 flushed between steps by a 256 MiB write); `e2e` is the same metric
through the public API with host buffers, host<->device copies included.
`--impl reference` times the CPU restatement of the reference's path (the
oracle, plain method) on all host cores instead.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gcr|reference]
                  [--workload learned|homography|fundamental|essential] [--pairs P]
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

from pygcransac import _abi, synthetic as S  # noqa: E402

METRIC = "image pairs/sec at equal model error; learned vs plain GC-RANSAC on 1 GB300"

# Algorithmic FP32 work of one residual evaluation (one model x one correspondence):
# H transfer error 21 FLOP, Sampson distance 35 FLOP.
FLOP_PER_RESIDUAL = {"homography": 21, "fundamental": 35, "essential": 35, "learned": 35}

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
    # calibrated pairs (f = 800 px, scene as above) with log-uniform 200-8000
    # correspondences and inlier ratio uniform in 10-70 % (sigma 0.5 px),
    # threshold 0.75 px (divided by the focal length), uniform sampler, 8^4
    # grid, lambda 0.1, 5-point solver + graph-cut LO, MAGSAC++ scoring
    "essential": dict(kind=_abi.GCR_ESSENTIAL, n=(200, 8000), ratio=(0.1, 0.7), threshold=0.75, sampler=0, grid=8,
                      lam=0.1, pairs=1024, scoring=_abi.GCR_SCORING_MAGSAC),
    # hard fundamental-matrix pairs: 4000 correspondences of the two-view scene
    # above at 5-10 % inliers. Plain form: uniform sampler with the reference's
    # 10000-iteration budget; learned form: the network's order drives PROSAC
    # with a 50-iteration budget. Same threshold, grid, lambda and LO.
    "learned": dict(kind=_abi.GCR_FUNDAMENTAL, n=4000, ratio=(0.05, 0.10), threshold=0.75, sampler=0, grid=8,
                    lam=0.975, pairs=1216, learned_iters=50),
}

CHECKPOINT = os.path.join(ROOT, "graph-cut-ransac_gb300", "pygcransac", "weights", "proposal_fundamental.gcrl")


def _gen_pair(job):
    """One synthetic pair (runs in a spawn pool)."""
    workload, seed, n, ratio = job
    if workload == "homography":
        pr = S.homography_pair(seed, n=n, inlier_ratio=ratio)
        return pr["corr"], pr["size"], pr["H_gt"]
    pr = S.two_view_pair(seed, n=n, inlier_ratio=ratio)
    return pr["corr"], pr["size"], pr


def build_pairs(workload, pairs, seed0):
    """Returns (corr, offsets, sizes, ground truths, K [P, 18] or None)."""
    w = WORKLOADS[workload]
    if isinstance(w["n"], tuple) or isinstance(w["ratio"], tuple):
        rng = np.random.Generator(np.random.PCG64(seed0 + 7919))
        ns = (np.exp(rng.uniform(np.log(w["n"][0]), np.log(w["n"][1]), pairs)).astype(int)
              if isinstance(w["n"], tuple) else np.full(pairs, w["n"]))
        ratios = rng.uniform(w["ratio"][0], w["ratio"][1], pairs)
    else:
        ns = np.full(pairs, w["n"])
        ratios = np.full(pairs, w["ratio"])
    jobs = [(workload, seed0 + i, int(ns[i]), float(ratios[i])) for i in range(pairs)]
    if pairs >= 256:
        import multiprocessing as mp
        with mp.get_context("spawn").Pool(max(1, min(16, os.cpu_count() or 1))) as pool:
            out = pool.map(_gen_pair, jobs, chunksize=16)
    else:
        out = [_gen_pair(j) for j in jobs]
    corr = [c for c, _, _ in out]
    sizes = [z for _, z, _ in out]
    gts = [g for _, _, g in out]
    Ks = [np.concatenate([g["K"].ravel(), g["K"].ravel()]) for g in gts] if workload == "essential" else []
    offsets = np.zeros(pairs + 1, np.int64)
    offsets[1:] = np.cumsum([len(c) for c in corr])
    K = np.ascontiguousarray(np.array(Ks), np.float64) if Ks else None
    return np.ascontiguousarray(np.concatenate(corr), np.float64), offsets, np.array(sizes), gts, K


def params_for(workload, seed=0):
    w = WORKLOADS[workload]
    return _abi.Params(threshold=w["threshold"], confidence=0.99, spatial_coherence_weight=w["lam"],
                       neighborhood_size=w["grid"], max_iterations=10000, min_iterations=50,
                       sampler=w["sampler"], neighborhood=0, lo_number=50, seed=seed,
                       scoring=w.get("scoring", _abi.GCR_SCORING_MSAC))


def size_array(sizes):
    z = np.zeros(len(sizes), _abi.SIZE_DTYPE)
    z["h1"], z["w1"], z["h2"], z["w2"] = sizes[:, 0], sizes[:, 1], sizes[:, 2], sizes[:, 3]
    return z


def model_errors(workload, models, gts, limit=64):
    """Median-ready model errors against ground truth on the first `limit` pairs
    (H: RMS transfer px; F: mean Sampson px of clean correspondences)."""
    if workload == "homography":
        return [S.homography_error(m / m[2, 2] if abs(m[2, 2]) > 1e-12 else m, g) for m, g in zip(models, gts)]
    if workload == "fundamental":
        return [S.fundamental_error(m, g, n=200) for m, g in list(zip(models, gts))[:limit]]
    if workload == "learned":
        return [S.fundamental_error(m, g, n=100) for m, g in zip(models, gts)]
    if workload == "essential":
        return [S.essential_error(m, g) for m, g in zip(models, gts)]
    return []


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


def cpu_baseline_kind(kind, corr, offsets, sizes, p, K=None, target_s=10.0, max_pairs=1 << 30):
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle
    threads = os.cpu_count() or 1
    P = len(offsets) - 1

    def run(k):
        # k pairs, cycling over the step's batch when k exceeds it
        idx = np.arange(k) % P
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
    return k / t, threads, f"{k} pairs cycling over the step's batch ({t:.1f} s)"


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
    pm = torch.zeros(P * 9, dtype=torch.float64, device="cuda")
    pk = torch.zeros(total, dtype=torch.uint8, device="cuda")
    ps = torch.zeros(P * _abi.STATS_DTYPE.itemsize, dtype=torch.uint8, device="cuda")
    vp = lambda t: ctypes.c_void_p(t.data_ptr())  # noqa: E731
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
    b = LearnedBatch(net, kind, d_corr, offsets, sizes, p_l, seeds)
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
    plain_models = pm.cpu().numpy().reshape(P, 3, 3)
    plain_stats = np.frombuffer(ps.cpu().numpy().tobytes(), _abi.STATS_DTYPE)
    err_l = model_errors(args.workload, models, gts)
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
    if rank != 0:
        b.close()
        lib.gcr_context_destroy(ctx_p)
        if dist:
            dist.destroy_process_group()
        return
    n_per = np.diff(offsets)
    peak = fp32_peak_tflops(torch)
    eng_s = eng_ms / args.steps / 1e3
    flops = float(np.sum(stats["models_scored"] * n_per)) * FLOP_PER_RESIDUAL[args.workload]
    mlp_flops = 2.0 * total * (32 * 128 + 2 * 128 * 128 + 128)
    achieved = flops / eng_s / 1e12
    traffic = fp64_work = None
    tp = os.path.join(ROOT, "profiles", "traffic_learned.json")
    if os.path.exists(tp):
        t = json.load(open(tp))
        traffic = t["bytes_per_pair"] * P
        fp64_work = t["fp64_flop_per_pair"] * P
    peak64 = fp64_peak_tflops(torch)
    line = {
        "metric": METRIC, "value": value, "unit": "pairs/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": total_ms / args.steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "fp32 scoring / fp64 solvers / bf16 weights, fp32 accumulation (MLP)",
        "data": "synthetic", "config": cfg,
        "median_model_error": float(np.median(err_l)),
        "status_ok_fraction": float(np.mean(stats["status"] == 0)),
        "plain": {"value": plain_value, "unit": "pairs/s", "ms_per_step": plain_ms / args.steps,
                  "median_model_error": float(np.median(err_p)),
                  "iterations_mean": float(np.mean(plain_stats["iteration_number"]))},
        "learned_over_plain": value / plain_value,
        "error_unit": "px, mean Sampson distance of 100 noise-free ground-truth correspondences per pair",
        "proposal_ms_per_step": prop_ms / args.steps, "engine_ms_per_step": eng_ms / args.steps,
        "roofline": {"bound": "fp32", "achieved": achieved, "peak": peak, "unit": "TFLOP/s",
                     "frac": achieved / peak if peak else None, "traffic": traffic,
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
    print(json.dumps(line))
    b.close()
    lib.gcr_context_destroy(ctx_p)
    if dist:
        dist.destroy_process_group()


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
    args = ap.parse_args()

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local_rank = int(os.environ.get("LOCAL_RANK", "0"))
    w = WORKLOADS[args.workload]
    P = args.pairs or w["pairs"]
    if args.workload == "essential":
        desc = (f"{args.workload}: {P} calibrated pairs/step x {w['n'][0]}-{w['n'][1]} (log-uniform) correspondences, "
                f"{int(w['ratio'][0]*100)}-{int(w['ratio'][1]*100)}% inliers, MAGSAC++")
    elif args.workload == "learned":
        desc = (f"learned: {P} fundamental-matrix pairs/step x {w['n']} correspondences, "
                f"{int(w['ratio'][0]*100)}-{int(w['ratio'][1]*100)}% inliers; learned order -> PROSAC "
                f"({w['learned_iters']} iterations) vs plain uniform sampler (10000 iterations)")
    else:
        desc = f"{args.workload}: {P} pairs/step x {w['n']} correspondences, {int(w['ratio']*100)}% inliers"
    cfg = {"workload": desc,
           "pairs_per_step": P, "correspondences": w["n"], "threshold": w["threshold"], "sampler": w["sampler"],
           "grid": w["grid"], "spatial_coherence_weight": w["lam"],
           "scoring": "MAGSAC++" if w.get("scoring") == _abi.GCR_SCORING_MAGSAC else "MSAC",
           "launch": "one persistent engine launch per step, replayed from a CUDA graph",
           "l2": "flushed between steps (256 MiB write)",
           "parallelism": f"replicas x{world}"}

    if args.impl == "reference":
        if rank != 0:
            return
        corr, offsets, sizes, gts, K = build_pairs(args.workload, P, 0)
        p = params_for(args.workload)
        for _ in range(args.warmup):
            cpu_baseline(args.workload, corr, offsets, sizes, p, K, target_s=1.0, max_pairs=64)
        vals = []
        for _ in range(args.steps):
            v, cores, sample = cpu_baseline(args.workload, corr, offsets, sizes, p, K, target_s=8.0)
            vals.append(v)
        v = float(np.median(vals))
        print(json.dumps({"metric": METRIC, "value": v, "unit": "pairs/s", "n_gpus": args.gpus,
                          "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * P / v,
                          "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
                          "data": "synthetic", "config": cfg, "impl": "reference",
                          "cpu_baseline": {"value": v, "unit": "pairs/s", "cores": cores, "kind": "port",
                                           "sample": sample},
                          "e2e": {"value": v, "unit": "pairs/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}))
        return

    import torch
    torch.cuda.set_device(local_rank)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=torch.device("cuda", local_rank))

    if args.workload == "learned":
        return run_learned(args, P, w, cfg, world, rank, local_rank, dist, torch)

    lib = _abi.load()
    corr, offsets, sizes, gts, K, seeds = replica_shard(args.workload, P, rank)
    p = params_for(args.workload)
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

    # one persistent launch per batch (plus the K^-1 normalisation for E),
    # prepared once and recorded into a CUDA graph; a step is one replay
    rc = lib.gcr_batch_prepare(ctx, kind, P, ctypes.c_void_p(d_corr.data_ptr()), _abi.ptr(offsets), _abi.ptr(K),
                               _abi.ptr(szs), ctypes.byref(p), _abi.ptr(seeds), ctypes.c_void_p(d_models.data_ptr()),
                               ctypes.c_void_p(d_masks.data_ptr()), ctypes.c_void_p(d_stats.data_ptr()))
    assert rc == 0, _abi.last_error()
    graph = torch.cuda.CUDAGraph()
    cap = torch.cuda.Stream()
    with torch.cuda.stream(cap):
        with torch.cuda.graph(graph, stream=cap):
            rc = lib.gcr_batch_launch(ctx, ctypes.c_void_p(cap.cuda_stream))
    assert rc == 0, _abi.last_error()
    launches_per_step = int(lib.gcr_last_launch_count())

    def step():
        graph.replay()
        return launches_per_step

    for _ in range(args.warmup):
        step()
    torch.cuda.synchronize()
    clocks = ClockSampler(local_rank)
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    clocks.start()
    total_ms, launches = 0.0, 0
    for _ in range(args.steps):
        flush.fill_(1)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        launches += step()
        e1.record(stream)
        e1.synchronize()
        total_ms += e0.elapsed_time(e1)
    torch.cuda.synchronize()
    clk = clocks.stop()
    value, t_rank = aggregate_rate(P * args.steps, total_ms / 1e3, world, dist, "cuda")
    if dist:
        dist.barrier()

    stats = np.frombuffer(d_stats.cpu().numpy().tobytes(), _abi.STATS_DTYPE)
    models = d_models.cpu().numpy().reshape(P, 3, 3)
    n_per = np.diff(offsets)
    flops = float(np.sum(stats["models_scored"] * n_per)) * FLOP_PER_RESIDUAL[args.workload]
    errs = model_errors(args.workload, models, gts)

    # end to end through the host-buffer entry: pinned inputs, copies timed
    h_corr = torch.from_numpy(corr).pin_memory()
    h_models = torch.zeros(P * 9, dtype=torch.float64).pin_memory()
    h_masks = torch.zeros(int(offsets[-1]), dtype=torch.uint8).pin_memory()
    h_stats = torch.zeros(P * _abi.STATS_DTYPE.itemsize, dtype=torch.uint8).pin_memory()

    def e2e_step():
        rc = lib.gcr_find_batch(kind, P, ctypes.c_void_p(h_corr.data_ptr()), _abi.ptr(offsets), _abi.ptr(K),
                                _abi.ptr(szs), ctypes.byref(p), _abi.ptr(seeds),
                                ctypes.c_void_p(h_models.data_ptr()), ctypes.c_void_p(h_masks.data_ptr()),
                                ctypes.c_void_p(h_stats.data_ptr()))
        assert rc == 0, _abi.last_error()

    e2e_step()
    e2e_t = 0.0
    for _ in range(args.steps):
        flush.fill_(1)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        e2e_step()
        e2e_t += time.perf_counter() - t0
    e2e_value, e2e_t = aggregate_rate(P * args.steps, e2e_t, world, dist, "cuda")

    if rank != 0:
        if dist:
            dist.destroy_process_group()
        return
    peak = fp32_peak_tflops(torch)
    achieved = flops / (total_ms / args.steps / 1e3) / 1e12
    traffic = None
    fp64_work = None
    tp = os.path.join(ROOT, "profiles", f"traffic_{args.workload}.json")
    if os.path.exists(tp):
        t = json.load(open(tp))
        traffic = t["bytes_per_pair"] * P
        fp64_work = t["fp64_flop_per_pair"] * P
    peak64 = fp64_peak_tflops(torch)
    line = {
        "metric": METRIC, "value": value, "unit": "pairs/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": total_ms / args.steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "fp32 scoring / fp64 solvers", "data": "synthetic", "config": cfg,
        "median_model_error": float(np.median(errs)) if errs else None,
        "status_ok_fraction": float(np.mean(stats["status"] == 0)),
        "roofline": {"bound": "fp32", "achieved": achieved, "peak": peak, "unit": "TFLOP/s",
                     "frac": achieved / peak if peak else None, "traffic": traffic,
                     "peak_source": "cuBLAS SGEMM 8192^3, TF32 off, measured in this run",
                     "work": f"{FLOP_PER_RESIDUAL[args.workload]} FLOP x models_scored x N per pair"},
        # the FP64 pipe is the unit the kernel keeps busiest (solvers, LO fits):
        # executed FP64 FLOP per pair from the ncu capture in profiles/, over the
        # live DGEMM peak
        "roofline_fp64": None if fp64_work is None else {
            "bound": "fp64", "achieved": fp64_work / (total_ms / args.steps / 1e3) / 1e12, "peak": peak64,
            "unit": "TFLOP/s", "frac": fp64_work / (total_ms / args.steps / 1e3) / 1e12 / peak64,
            "peak_source": "cuBLAS DGEMM 4096^3, measured in this run",
            "work": "FP64 FLOP per pair executed by the kernel (ncu SASS counts, FMA = 2) x pairs"},
        "e2e": {"value": e2e_value, "unit": "pairs/s", "h2d_bytes_per_step": int(corr.nbytes),
                "d2h_bytes_per_step": int(P * 9 * 8 + offsets[-1] + P * _abi.STATS_DTYPE.itemsize)},
        "gpu_launches": int(launches),
        "clocks": clk,
    }
    if not args.no_cpu_baseline and world == 1:
        v, cores, sample = cpu_baseline(args.workload, corr, offsets, sizes, p, K)
        line["cpu_baseline"] = {"value": v, "unit": "pairs/s", "cores": cores, "kind": "port", "sample": sample}
    print(json.dumps(line))
    lib.gcr_context_destroy(ctx)
    if dist:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
