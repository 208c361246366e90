"""The C++ plugin surface (include/gcransac/GCRANSAC.h): a program written
against gcransac::GCRANSAC<Estimator, GridNeighborhoodGraph<4>, Scoring,
Preemption, Selector>::run (tests/plugin/plugin_run.cpp) compiles against the
header and libgcr.so, and on the GPU its results equal the oracle's
GCRANSAC::run (oracle_run: no driver epilogue, caller-given grid and
coordinates): identical masks and iteration / graph-cut / LO counts, models
within 1e-6 relative Frobenius error."""
import os
import shutil
import struct
import subprocess

import numpy as np
import pytest

from pygcransac import _abi, synthetic as S

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
LIBDIR = os.path.join(ROOT, "graph-cut-ransac_gb300", "_build")
MODEL_TOL = 1e-6


def compile_driver(out_dir):
    exe = os.path.join(out_dir, "plugin_run")
    cxx = shutil.which("g++") or shutil.which("c++")
    if cxx is None:
        pytest.skip("no C++ compiler")
    subprocess.run([cxx, "-std=c++17", "-O1", "-Wall", "-Werror", "-I", os.path.join(ROOT, "include"),
                    os.path.join(ROOT, "tests", "plugin", "plugin_run.cpp"), "-L", LIBDIR, "-lgcr",
                    f"-Wl,-rpath,{LIBDIR}", "-o", exe], check=True, capture_output=True, text=True)
    return exe


def test_header_compiles_and_links(tmp_path):
    if not os.path.exists(os.path.join(LIBDIR, "libgcr.so")):
        pytest.skip("libgcr.so not built")
    assert os.path.exists(compile_driver(str(tmp_path)))


def write_input(path, kind, pts, pix, cfg, K=None):
    n = len(pts)
    with open(path, "wb") as f:
        f.write(struct.pack("<6i", kind, cfg["sampler"], cfg["scoring"], cfg["sprt"], cfg["sp"], cfg["div"]))
        f.write(struct.pack("<q3d2qiQd", n, cfg["thr"], 0.99, cfg["lam"], cfg["max_it"], cfg["min_it"], 50, cfg["seed"],
                            cfg.get("ratio", 0.01)))
        f.write(np.asarray(cfg["cell"], "<f8").tobytes())
        f.write(np.asarray(cfg["sizes"], "<f8").tobytes())
        f.write(np.ascontiguousarray(pts, "<f8").tobytes())
        f.write(np.ascontiguousarray(pix, "<f8").tobytes())
        Kf = np.eye(3) if K is None else K
        f.write(np.asarray(Kf, "<f8").tobytes() * 2)
        f.write(struct.pack("<d", cfg.get("variance", 0.1)))
        pr = cfg.get("probs")
        f.write(np.ascontiguousarray(np.ones(n) if pr is None else pr, "<f8").tobytes())


def read_output(path):
    b = open(path, "rb").read()
    has = struct.unpack_from("<i", b, 0)[0]
    model = np.frombuffer(b, "<f8", 9, 4).reshape(3, 3)
    it, gc, lo = struct.unpack_from("<3q", b, 76)
    score = struct.unpack_from("<d", b, 100)[0]
    ni = struct.unpack_from("<q", b, 108)[0]
    inl = np.frombuffer(b, "<i8", ni, 116)
    return has, model, (it, gc, lo), score, inl


def rel_err(a, b):
    a = a / np.linalg.norm(a)
    b = b / np.linalg.norm(b)
    return min(np.linalg.norm(a - b), np.linalg.norm(a + b))


def cases():
    K = S.intrinsics()
    Ki = np.linalg.inv(K)
    out = []
    pr = S.homography_pair(11, n=1500)
    base = dict(sampler=0, scoring=0, sprt=0, sp=0, div=4, thr=3.0, lam=0.975, max_it=2000, min_it=50, seed=3,
                cell=[160.0, 120.0, 160.0, 120.0], sizes=[640.0, 480.0, 640.0, 480.0])
    out.append(("H uniform MSAC", _abi.GCR_HOMOGRAPHY, pr["corr"], pr["corr"], base, None))
    out.append(("H SPRT + space partitioning", _abi.GCR_HOMOGRAPHY, pr["corr"], pr["corr"],
                dict(base, sprt=1, sp=1, ratio=0.01, seed=4), None))
    pf = S.two_view_pair(12, n=2000, inlier_ratio=0.35)
    fcfg = dict(base, div=8, thr=0.75, cell=[80.0, 60.0, 80.0, 60.0], max_it=3000)
    out.append(("F P-NAPSAC MSAC", _abi.GCR_FUNDAMENTAL, pf["corr"], pf["corr"], dict(fcfg, sampler=2, seed=5), None))
    order = np.argsort(~pf["inlier_gt"], kind="stable")  # a quality order for PROSAC
    out.append(("F PROSAC MAGSAC++", _abi.GCR_FUNDAMENTAL, pf["corr"][order], pf["corr"][order],
                dict(fcfg, sampler=1, scoring=1, seed=6), None))
    pe = S.two_view_pair(13, n=1200, inlier_ratio=0.4)
    c = pe["corr"]
    nrm = np.c_[(np.c_[c[:, :2], np.ones(len(c))] @ Ki.T)[:, :2], (np.c_[c[:, 2:], np.ones(len(c))] @ Ki.T)[:, :2]]
    out.append(("E normalised points, pixel grid, MAGSAC++", _abi.GCR_ESSENTIAL, nrm, c,
                dict(fcfg, scoring=1, lam=0.1, thr=0.75 / 800.0, seed=7), K))
    out.append(("E SPRT", _abi.GCR_ESSENTIAL, nrm, c, dict(fcfg, sprt=1, lam=0.1, thr=0.75 / 800.0, seed=8), K))
    # the radius graph (FlannNeighborhoodGraph): divisions 0, radius in cell[0]
    out.append(("F radius graph", _abi.GCR_FUNDAMENTAL, pf["corr"], pf["corr"],
                dict(fcfg, div=0, cell=[20.0, 1.0, 1.0, 1.0], seed=9), None))
    out.append(("E radius graph", _abi.GCR_ESSENTIAL, nrm, c,
                dict(fcfg, div=0, cell=[20.0, 1.0, 1.0, 1.0], lam=0.1, thr=0.75 / 800.0, seed=10), K))
    # samplers reading per-point probabilities (largest 1, as the AR sampler
    # wants them): a noisy inlier indicator
    rng = np.random.default_rng(14)
    ph = np.clip(np.where(pr["inlier_gt"], 0.8, 0.2) + rng.normal(0, 0.1, len(pr["corr"])), 0.01, 0.99)
    ph /= ph.max()
    out.append(("H importance sampler", _abi.GCR_HOMOGRAPHY, pr["corr"], pr["corr"],
                dict(base, sampler=3, probs=ph, seed=11), None))
    pq = np.clip(np.where(pf["inlier_gt"], 0.7, 0.3) + rng.normal(0, 0.1, len(pf["corr"])), 0.01, 0.99)
    pq /= pq.max()
    out.append(("F AR sampler", _abi.GCR_FUNDAMENTAL, pf["corr"], pf["corr"],
                dict(fcfg, sampler=4, probs=pq, variance=0.1, seed=12), None))
    return out


def test_ar_sampler_rejects_unscaled_probabilities(tmp_path):
    """The AR sampler class throws (driver exit code 3) for probabilities
    whose maximum is not 1; no device work is started."""
    if not os.path.exists(os.path.join(LIBDIR, "libgcr.so")):
        pytest.skip("libgcr.so not built")
    exe = compile_driver(str(tmp_path))
    pf = S.two_view_pair(15, n=300, inlier_ratio=0.5)
    cfg = dict(sampler=4, scoring=0, sprt=0, sp=0, div=8, thr=0.75, lam=0.975, max_it=100, min_it=50, seed=1,
               cell=[80.0, 60.0, 80.0, 60.0], sizes=[640.0, 480.0, 640.0, 480.0], probs=np.full(300, 0.5))
    fin, fout = str(tmp_path / "in.bin"), str(tmp_path / "out.bin")
    write_input(fin, _abi.GCR_FUNDAMENTAL, pf["corr"], pf["corr"], cfg)
    r = subprocess.run([exe, fin, fout], capture_output=True, text=True)
    assert r.returncode == 3 and "maximum is 1" in r.stderr


@pytest.mark.gpu
@pytest.mark.parametrize("idx", range(10))
def test_plugin_run_matches_oracle_run(tmp_path, oracle, idx):
    name, kind, pts, pix, cfg, K = cases()[idx]
    exe = compile_driver(str(tmp_path))
    fin, fout = str(tmp_path / "in.bin"), str(tmp_path / "out.bin")
    write_input(fin, kind, pts, pix, cfg, K)
    r = subprocess.run([exe, fin, fout], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    has, model, counts, score, inl = read_output(fout)
    radius = cfg["div"] == 0
    p = _abi.Params(threshold=cfg["thr"], confidence=0.99, spatial_coherence_weight=cfg["lam"],
                    neighborhood_size=cfg["cell"][0] if radius else cfg["div"], max_iterations=cfg["max_it"],
                    min_iterations=cfg["min_it"], sampler=cfg["sampler"], neighborhood=1 if radius else 0,
                    lo_number=50, seed=cfg["seed"], scoring=cfg["scoring"],
                    use_sprt=cfg["sprt"], use_space_partitioning=cfg["sp"],
                    min_inlier_ratio_for_sprt=cfg.get("ratio", 0.01), sampler_variance=cfg.get("variance", 0.1))
    z = cfg["sizes"]
    rc, M, mask, st = oracle.run(kind, pts, pix, cfg["cell"], max(cfg["div"], 1), oracle.make_size(int(z[1]), int(z[0]),
                                                                                            int(z[3]), int(z[2])),
                                 p, seed=cfg["seed"], probabilities=cfg.get("probs"))
    assert has == (rc == 0), name
    ref = np.flatnonzero(mask)
    assert np.array_equal(inl, ref), f"{name}: inliers differ ({len(inl)} vs {len(ref)})"
    assert counts == (st.iteration_number, st.graph_cut_number, st.local_optimization_number), name
    if rc == 0:
        assert rel_err(model, M) < MODEL_TOL, name
        assert abs(score - st.score) <= 1e-9 * max(1.0, abs(st.score)), name
