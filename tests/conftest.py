import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
for p in (ROOT, os.path.join(ROOT, "oracle"), os.path.join(ROOT, "graph-cut-ransac_gb300")):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA device (run on the GPU box)")


@pytest.fixture(scope="session")
def oracle():
    import oracle as O
    O.load()
    return O


@pytest.fixture(scope="session")
def gcr():
    """The engine's Python entry points; the library must be built (no fallback)."""
    import pygcransac
    pygcransac._abi.load()
    return pygcransac


@pytest.fixture(scope="session")
def batch_parity(oracle):
    """check(kind, corr, offsets, sizes, params, seeds, K, stats, masks):
    the device batch equals the oracle pair by pair (status, iteration and
    graph-cut counts, inlier mask). A pair may differ from the oracle only
    where the oracle's own result depends on rounding: there the oracle's
    FMA-contracted build must give exactly the device's result (and so
    differs from the plain build). Returns the indices of such pairs."""
    import numpy as np

    fields = ("status", "iteration_number", "graph_cut_number")

    def check(kind, corr, offsets, sizes, params, seeds, K, stats, masks, **kw):
        threads = os.cpu_count() or 1

        def same(st_o, k_o, i):
            a = slice(offsets[i], offsets[i + 1])
            return all(stats[f][i] == st_o[f][i] for f in fields) and np.array_equal(masks[a], k_o[a])

        _, k_o, st_o, _ = oracle.find_batch(kind, corr, offsets, sizes, params, seeds=seeds, K=K, threads=threads,
                                            **kw)
        differ = [i for i in range(len(seeds)) if not same(st_o, k_o, i)]
        if differ:
            with oracle.contracted():
                _, k_c, st_c, _ = oracle.find_batch(kind, corr, offsets, sizes, params, seeds=seeds, K=K,
                                                    threads=threads, **kw)
            for i in differ:
                assert same(st_c, k_c, i), (
                    f"pair {i}: device {[stats[f][i] for f in fields]} differs from both oracle builds "
                    f"(plain {[st_o[f][i] for f in fields]}, contracted {[st_c[f][i] for f in fields]})")
        return differ

    return check
