"""Train the learned inlier-probability proposal and write its checkpoint.

  python -m pygcransac.train_proposal [--pairs 200000] [--out PATH]
      (run from graph-cut-ransac_gb300/, or with it on sys.path)

Data: two-view scenes of the fundamental-matrix workload (4000
correspondences, depth 2-10 m, f = 800 px, rotation up to 30 deg, unit
baseline, sigma 0.5 px, uniform outliers) at inlier ratios where the plain
method converges (default 15-50 %). Labels: the inlier masks that the plain
method (this engine, uniform sampler, 7-point solver + graph-cut LO, threshold
0.75 px, 10000 iterations) returns for each pair; the ground truth is never
read. Pairs are generated, labelled and trained on in chunks (one pass over
every pair), so the device holds one chunk's features at a time.
"""
import argparse
import multiprocessing as mp
import os
import sys
import time

import numpy as np

from . import _abi, find_batch
from . import synthetic as S
from .learned import LearnedProposal

DEFAULT_OUT = os.path.join(os.path.dirname(os.path.abspath(__file__)), "weights", "proposal_fundamental.gcrl")
TRAIN_SEED0 = 50_000_000  # training scenes: seeds from here on (the benchmark and tests use smaller seeds)


def label_params(seed=0):
    return _abi.Params(threshold=0.75, confidence=0.99, spatial_coherence_weight=0.975, neighborhood_size=8,
                       max_iterations=10000, min_iterations=50, sampler=0, neighborhood=0, lo_number=50, seed=seed,
                       scoring=_abi.GCR_SCORING_MSAC)


def _gen(args):
    seed, n, lo, hi = args
    rng = np.random.Generator(np.random.PCG64(seed ^ 0x5EED))
    pr = S.two_view_pair(seed, n=n, inlier_ratio=float(rng.uniform(lo, hi)))
    return pr["corr"], pr["size"]


def generate(pool, seeds, n, ratio):
    jobs = [(int(s), n, ratio[0], ratio[1]) for s in seeds]
    out = pool.map(_gen, jobs, chunksize=16) if pool else list(map(_gen, jobs))
    return [c for c, _ in out], np.array([z for _, z in out])


def label(corr_list, sizes, seed):
    """Plain-method inlier masks (uniform sampler), one per pair."""
    _, masks, stats = find_batch(_abi.GCR_FUNDAMENTAL, corr_list, sizes, label_params(seed))
    ok = (stats["status"] == 0) & (stats["inlier_number"] >= 21)
    return masks, ok


def train(pairs=200000, chunk=2048, n=4000, ratio=(0.15, 0.5), lr=1e-3, lr_final=1e-4, batch_rows=65536,
          seed=0, out=DEFAULT_OUT, workers=None, log=print):
    import torch
    ctx = mp.get_context("spawn")
    pool = ctx.Pool(workers or max(1, min(16, os.cpu_count() or 1))) if pairs > 64 else None
    try:
        net = LearnedProposal(seed=seed)
        chunks = (pairs + chunk - 1) // chunk
        t0 = time.time()
        losses, kept = [], 0
        for c in range(chunks):
            seeds = TRAIN_SEED0 + np.arange(c * chunk, min(pairs, (c + 1) * chunk))
            corr_list, sizes = generate(pool, seeds, n, ratio)
            masks, ok = label(corr_list, sizes, seed + c)
            keep = np.flatnonzero(ok)
            kept += len(keep)
            if len(keep) == 0:
                continue
            feat, offsets = net.host_features([corr_list[i] for i in keep], sizes[keep])
            y = torch.from_numpy(np.concatenate([masks[i] for i in keep]).astype(np.float32)).to(net.device)
            # learning rate: linear decay from lr to lr_final over the chunks
            a = c / max(1, chunks - 1)
            hist = net.train_rows(feat, y, epochs=1, lr=lr + (lr_final - lr) * a, batch_rows=batch_rows,
                                  seed=seed * 1000003 + c)
            losses.append(float(np.mean(hist)))
            log(f"chunk {c + 1}/{chunks}: {len(keep)} labelled pairs, loss {losses[-1]:.4f}, "
                f"{time.time() - t0:.0f} s")
        info = dict(pairs=int(pairs), labelled_pairs=int(kept), correspondences=int(n),
                    inlier_ratio=[float(ratio[0]), float(ratio[1])], labels="plain method inlier masks",
                    train_seed0=TRAIN_SEED0, lr=[lr, lr_final], batch_rows=batch_rows,
                    final_loss=losses[-1] if losses else None)
        if out:
            os.makedirs(os.path.dirname(out), exist_ok=True)
            net.save(out, info)
        return net, losses
    finally:
        if pool:
            pool.close()
            pool.join()


def main(argv=None):
    ap = argparse.ArgumentParser(description=__doc__.split("\n")[0])
    ap.add_argument("--pairs", type=int, default=200000)
    ap.add_argument("--chunk", type=int, default=2048)
    ap.add_argument("--n", type=int, default=4000)
    ap.add_argument("--ratio", type=float, nargs=2, default=(0.15, 0.5))
    ap.add_argument("--lr", type=float, default=1e-3)
    ap.add_argument("--out", default=DEFAULT_OUT)
    ap.add_argument("--seed", type=int, default=0)
    a = ap.parse_args(argv)
    train(pairs=a.pairs, chunk=a.chunk, n=a.n, ratio=tuple(a.ratio), lr=a.lr, seed=a.seed, out=a.out,
          log=lambda s: print(s, file=sys.stderr, flush=True))


if __name__ == "__main__":
    main()
