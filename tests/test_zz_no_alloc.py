"""GPU test of gcr_find_homography_device_noalloc, the allocation-free
single-pair entry point, through the C-ABI: two calls in a row on one stream
must give the masks, statistics and (within 1e-6 relative Frobenius error)
the models of the allocating entry point gcr_find_batch on the same pairs,
for each sampler the entry point provides (uniform, PROSAC, P-NAPSAC) and with
SPRT and space partitioning, alone and together.
The file name sorts last so that the test also runs after every other test."""
import ctypes

import numpy as np
import pytest

from pygcransac import _abi, synthetic as S

pytestmark = pytest.mark.gpu

MODEL_TOL = 1e-6


def h_params(**kw):
    base = dict(threshold=3.0, confidence=0.99, spatial_coherence_weight=0.975, neighborhood_size=4,
                max_iterations=10000, min_iterations=50, sampler=0, neighborhood=0, lo_number=50, seed=0,
                min_inlier_ratio_for_sprt=1e-5)
    base.update(kw)
    return _abi.Params(**base)


CONFIGS = {
    "uniform": {},
    "prosac": dict(sampler=1),
    "pnapsac": dict(sampler=2),
    "sprt": dict(use_sprt=1),
    "space_partitioning": dict(use_space_partitioning=1),
    "sprt_and_space_partitioning": dict(sampler=1, use_sprt=1, use_space_partitioning=1),
}


def rel_model_err(a, b):
    a = a / np.linalg.norm(a)
    b = b / np.linalg.norm(b)
    return min(np.linalg.norm(a - b), np.linalg.norm(a + b))


@pytest.mark.parametrize("config", sorted(CONFIGS))
def test_noalloc_matches_allocating_entry(gcr, config):
    torch = pytest.importorskip("torch")
    lib = _abi.load()
    p = h_params(**CONFIGS[config])
    cases = [(S.homography_pair(5, n=2000), 7), (S.homography_pair(6, n=4096, inlier_ratio=0.3), 8)]
    stream = torch.cuda.current_stream()
    outs = []
    for pr, seed in cases:
        corr = torch.from_numpy(np.ascontiguousarray(pr["corr"])).cuda()
        n = corr.shape[0]
        model = torch.zeros(9, dtype=torch.float64, device="cuda")
        mask = torch.zeros(n, dtype=torch.uint8, device="cuda")
        stats = torch.zeros(_abi.STATS_DTYPE.itemsize, dtype=torch.uint8, device="cuda")
        h1, w1, h2, w2 = pr["size"]
        size = _abi.ImageSize(h1=h1, w1=w1, h2=h2, w2=w2)
        rc = lib.gcr_find_homography_device_noalloc(
            ctypes.c_void_p(corr.data_ptr()), n, ctypes.byref(size), ctypes.byref(p), seed,
            ctypes.c_void_p(model.data_ptr()), ctypes.c_void_p(mask.data_ptr()),
            ctypes.c_void_p(stats.data_ptr()), ctypes.c_void_p(stream.cuda_stream))
        assert rc == _abi.GCR_OK, _abi.last_error()
        outs.append((corr, model, mask, stats))
    torch.cuda.synchronize()
    for (pr, seed), (_, model, mask, stats) in zip(cases, outs):
        st = np.frombuffer(stats.cpu().numpy().tobytes(), dtype=_abi.STATS_DTYPE)[0]
        models, masks, ref = gcr.find_batch(_abi.GCR_HOMOGRAPHY, [pr["corr"]], [pr["size"]], p, seeds=[seed])
        assert st["status"] == ref["status"][0] == 0
        assert np.array_equal(mask.cpu().numpy(), masks[0])
        assert rel_model_err(model.cpu().numpy().reshape(3, 3), models[0]) < MODEL_TOL
        for k in ("iteration_number", "graph_cut_number", "local_optimization_number", "inlier_number",
                  "models_scored", "flags"):
            assert st[k] == ref[k][0], k


def test_noalloc_rejects_more_than_4096_points(gcr):
    lib = _abi.load()
    p = h_params()
    size = _abi.ImageSize(h1=480, w1=640, h2=480, w2=640)
    dummy = ctypes.c_void_p(16)  # never dereferenced: the size check fails first
    rc = lib.gcr_find_homography_device_noalloc(dummy, 4097, ctypes.byref(size), ctypes.byref(p), 0, dummy, dummy,
                                                dummy, None)
    assert rc == _abi.GCR_CAPACITY
    assert "4096" in _abi.last_error()
