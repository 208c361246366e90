"""The mixed serving batch's launch pattern at a size that fits the suite: one
context per model kind and form, buffers allocated through torch kind by kind,
every batch recorded into a CUDA graph on its own stream (graph capture
releases torch's cached blocks to the driver), the three kinds replayed
concurrently on three streams, twice.

The plain form must equal the oracle pair by pair (exact masks, statuses,
iteration and graph-cut counts, models within 1e-6 relative Frobenius error);
the learned form must equal the same pipeline run outside a graph on a fresh
context. Pair sizes are log-uniform over 2000-40000 correspondences with 5-60 %
inliers on a 16^4 grid, as in the serving mix.

Every buffer a captured graph writes stays referenced for the whole test: a
graph keeps raw device addresses, and a buffer dropped between capture and
replay is returned to the driver by the next capture's empty_cache()."""
import ctypes
import os

import numpy as np
import pytest

from pygcransac import _abi, synthetic as S

pytestmark = pytest.mark.gpu

MODEL_TOL = 1e-6
PAIRS_PER_KIND = 12
KINDS = [  # (generator, kind, threshold, lambda)
    ("homography", _abi.GCR_HOMOGRAPHY, 3.0, 0.975),
    ("fundamental", _abi.GCR_FUNDAMENTAL, 0.75, 0.975),
    ("essential", _abi.GCR_ESSENTIAL, 0.75, 0.1),
]


def params(thr, lam, iters):
    return _abi.Params(threshold=thr, confidence=0.99, spatial_coherence_weight=lam, neighborhood_size=16,
                       max_iterations=iters, min_iterations=min(50, iters), sampler=0, neighborhood=0, lo_number=50,
                       seed=0)


def rel_err(a, b):
    a = a / np.linalg.norm(a)
    b = b / np.linalg.norm(b)
    return min(np.linalg.norm(a - b), np.linalg.norm(a + b))


def make_groups():
    rng = np.random.default_rng(4096)
    groups = []
    for k, (name, kind, thr, lam) in enumerate(KINDS):
        ns = np.exp(rng.uniform(np.log(2000), np.log(40000), PAIRS_PER_KIND)).astype(int)
        ns[0] = 40000  # the largest pair of the mix
        ratios = rng.uniform(0.05, 0.6, PAIRS_PER_KIND)
        pairs = []
        for i in range(PAIRS_PER_KIND):
            seed = 7000 + 100 * k + i
            if name == "homography":
                pairs.append(S.homography_pair(seed, n=int(ns[i]), inlier_ratio=float(ratios[i])))
            else:
                pairs.append(S.two_view_pair(seed, n=int(ns[i]), inlier_ratio=float(ratios[i])))
        corr = np.ascontiguousarray(np.concatenate([q["corr"] for q in pairs]), np.float64)
        off = np.zeros(len(pairs) + 1, np.int64)
        off[1:] = np.cumsum([len(q["corr"]) for q in pairs])
        sz = np.zeros(len(pairs), _abi.SIZE_DTYPE)
        for i, q in enumerate(pairs):
            sz[i] = q["size"]
        K = None
        if kind == _abi.GCR_ESSENTIAL:
            K = np.ascontiguousarray([np.concatenate([q["K"].ravel(), q["K"].ravel()]) for q in pairs])
        groups.append(dict(name=name, kind=kind, thr=thr, lam=lam, pairs=pairs, corr=corr, off=off, sz=sz, K=K,
                           seeds=np.arange(len(pairs), dtype=np.uint64) + np.uint64(11 + 1000 * k)))
    return groups


def test_serving_pattern_three_streams_graphs(oracle, gcr):
    torch = pytest.importorskip("torch")
    from pygcransac.learned import LearnedBatch, LearnedProposal, find_batch_learned
    lib = _abi.load()
    net = LearnedProposal.load(os.path.join(os.path.dirname(gcr.__file__), "weights", "proposal_fundamental.gcrl"))
    groups = make_groups()
    streams = [torch.cuda.Stream() for _ in groups]
    ptr = lambda t: ctypes.c_void_p(t.data_ptr())  # noqa: E731
    recs = []
    for g, s in zip(groups, streams):
        P, total = len(g["pairs"]), int(g["off"][-1])
        r = dict(g=g, s=s)
        r["d_corr"] = torch.from_numpy(g["corr"]).cuda()
        r["pm"] = torch.zeros(P * 9, dtype=torch.float64, device="cuda")
        r["pk"] = torch.zeros(total, dtype=torch.uint8, device="cuda")
        r["ps"] = torch.zeros(P * _abi.STATS_DTYPE.itemsize, dtype=torch.uint8, device="cuda")
        r["times"] = torch.zeros(2 * P, dtype=torch.int64, device="cuda")
        ctx = ctypes.c_void_p()
        assert lib.gcr_context_create(ctypes.byref(ctx)) == 0
        r["ctx"] = ctx
        assert lib.gcr_context_set_pair_times(ctx, ptr(r["times"])) == 0
        p = params(g["thr"], g["lam"], 2000)
        rc = lib.gcr_batch_prepare(ctx, g["kind"], P, ptr(r["d_corr"]), _abi.ptr(g["off"]), _abi.ptr(g["K"]),
                                   _abi.ptr(g["sz"]), ctypes.byref(p), _abi.ptr(g["seeds"]), ptr(r["pm"]),
                                   ptr(r["pk"]), ptr(r["ps"]))
        assert rc == 0, _abi.last_error()
        r["g_plain"] = torch.cuda.CUDAGraph()
        with torch.cuda.stream(s):
            with torch.cuda.graph(r["g_plain"], stream=s):
                assert lib.gcr_batch_launch(ctx, ctypes.c_void_p(s.cuda_stream)) == 0, _abi.last_error()
        pl = params(g["thr"], g["lam"], 50)
        b = LearnedBatch(net, g["kind"], r["d_corr"], g["off"], [q["size"] for q in g["pairs"]], pl, g["seeds"], g["K"])
        b.prepare()
        r["batch"] = b
        r["g_learned"] = torch.cuda.CUDAGraph()
        with torch.cuda.stream(s):
            with torch.cuda.graph(r["g_learned"], stream=s):
                b.launch(s)
        recs.append(r)
        torch.cuda.empty_cache()

    main = torch.cuda.current_stream()

    def replay(key):
        start = torch.cuda.Event()
        start.record(main)
        for r in recs:
            r["s"].wait_event(start)
            with torch.cuda.stream(r["s"]):
                r[key].replay()
        torch.cuda.synchronize()

    results = []
    for rep in range(2):
        for r in recs:
            r["ps"].zero_()
            r["pk"].zero_()
            r["batch"].d_stats.zero_()
        replay("g_plain")
        replay("g_learned")
        results.append([(r["pm"].clone(), r["pk"].clone(), r["ps"].clone(), r["batch"].results()) for r in recs])
    # both replays agree bit for bit
    for a, b in zip(results[0], results[1]):
        assert torch.equal(a[0], b[0]) and torch.equal(a[1], b[1]) and torch.equal(a[2], b[2])
        assert np.array_equal(a[3][0], b[3][0])
        assert all(np.array_equal(x, y) for x, y in zip(a[3][1], b[3][1]))

    threads = os.cpu_count() or 1
    for r, (pm, pk, ps, (ml, kl, sl)) in zip(recs, results[0]):
        g = r["g"]
        P = len(g["pairs"])
        stats = np.frombuffer(ps.cpu().numpy().tobytes(), _abi.STATS_DTYPE)
        models = pm.cpu().numpy().reshape(P, 3, 3)
        masks = pk.cpu().numpy().astype(bool)
        t = r["times"].cpu().numpy().reshape(P, 2)
        assert np.all(t[:, 1] >= t[:, 0]) and np.all(t[:, 0] > 0), g["name"]
        p = params(g["thr"], g["lam"], 2000)
        m_o, k_o, st_o, _ = oracle.find_batch(g["kind"], g["corr"], g["off"], g["sz"], p, seeds=g["seeds"],
                                              K=g["K"], threads=threads)
        assert np.array_equal(stats["status"], st_o["status"]), g["name"]
        assert np.array_equal(stats["iteration_number"], st_o["iteration_number"]), g["name"]
        assert np.array_equal(stats["graph_cut_number"], st_o["graph_cut_number"]), g["name"]
        for i in range(P):
            sl_ = slice(g["off"][i], g["off"][i + 1])
            assert np.array_equal(masks[sl_], k_o[sl_]), (g["name"], i)
            if st_o["status"][i] == 0:
                assert rel_err(models[i], m_o[i].reshape(3, 3)) < MODEL_TOL, (g["name"], i)
        # the learned form outside a graph, on a fresh context
        pl = params(g["thr"], g["lam"], 50)
        ml2, kl2, sl2 = find_batch_learned(g["kind"], [q["corr"] for q in g["pairs"]], [q["size"] for q in g["pairs"]],
                                           pl, net, seeds=g["seeds"], K=g["K"])
        assert np.array_equal(sl["status"], sl2["status"]), g["name"]
        assert np.array_equal(sl["iteration_number"], sl2["iteration_number"]), g["name"]
        assert np.array_equal(ml, ml2), g["name"]
        assert all(np.array_equal(a, b) for a, b in zip(kl, kl2)), g["name"]
    for r in recs:
        lib.gcr_context_destroy(r["ctx"])
        r["batch"].close()
