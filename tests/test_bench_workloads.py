"""CPU checks of the bench's single-kind workloads: every workload builds its
synthetic pairs with the row width and intrinsics its model kind needs, and
its model-error measure gives (near) zero on the ground truth, so the
bench's error columns measure the engine and not the harness."""
import os
import sys

import numpy as np
import pytest

sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
import bench  # noqa: E402
from pygcransac import _abi  # noqa: E402

ROWS8 = {_abi.GCR_HOMOGRAPHY_AFFINE, _abi.GCR_HOMOGRAPHY_SIFT, _abi.GCR_FUNDAMENTAL_AFFINE, _abi.GCR_FUNDAMENTAL_SIFT}
ESSENTIAL = {_abi.GCR_ESSENTIAL, _abi.GCR_ESSENTIAL_PLANAR}


@pytest.mark.parametrize("workload", sorted(w for w in bench.WORKLOADS if w not in ("serving", "learned")))
def test_workload_pairs_and_errors(workload):
    w = bench.WORKLOADS[workload]
    corr, offsets, sizes, gts, K = bench.build_pairs(workload, 2, 1000)
    cols = 8 if w["kind"] in ROWS8 else 4
    assert corr.shape == (offsets[-1], cols)
    assert len(offsets) == 3 and np.all(np.diff(offsets) > 0)
    assert sizes.shape == (2, 4)
    if w["kind"] in ESSENTIAL:
        assert K is not None and K.shape == (2, 18)
    else:
        assert K is None
    assert workload in bench.FLOP_PER_RESIDUAL
    if w["kind"] in (_abi.GCR_HOMOGRAPHY, _abi.GCR_HOMOGRAPHY_SIFT):
        models = [g / g[2, 2] for g in gts]
    elif w["kind"] in ESSENTIAL:
        models = [g["E_gt"] for g in gts]
    else:
        models = [g["F_gt"] for g in gts]
    errs = bench.model_errors(workload, models, gts)
    assert len(errs) == 2 and max(errs) < 1e-4, errs  # px or degrees (arccos near 1 loses digits)
