"""Builds libgcr.so (the CUDA engine and its C-ABI) in-tree for sm_103a.

Usage: python graph-cut-ransac_gb300/build.py [--jobs N]
Each translation unit is compiled by its own nvcc process in parallel, then
linked into graph-cut-ransac_gb300/_build/libgcr.so.
"""
import argparse
import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
OUT = os.path.join(HERE, "_build")
SOURCES = ["gcr_kind_f.cu", "gcr_kind_fa.cu", "gcr_kind_fs.cu", "gcr_kind_e.cu", "gcr_api.cu", "gcr_kind_h.cu", "gcr_kind_ha.cu",
           "gcr_kind_hs.cu", "gcr_kind_ep.cu", "gcr_noalloc.cu", "gcr_learned.cu"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler", "-ffp-contract=off",
         "--expt-relaxed-constexpr",
         "-Xptxas", "-warn-spills"]


def nvcc():
    cand = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(cand):
        raise RuntimeError("nvcc not found")
    return cand


def compile_one(src, extra, out=OUT):
    obj = os.path.join(out, os.path.splitext(src)[0] + ".o")
    cmd = [nvcc(), *ARCH, *FLAGS, *extra, "-c", os.path.join(CSRC, src), "-o", obj]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed for {src}:\n{r.stdout}\n{r.stderr}")
    return obj, r.stderr


def build(jobs=4, verbose=False, extra=(), out=OUT, sources=None):
    """Compiles every source (or `sources`) with `extra` nvcc flags into
    `out`/libgcr.so."""
    os.makedirs(out, exist_ok=True)
    srcs = [s for s in (sources or SOURCES) if os.path.exists(os.path.join(CSRC, s))]
    with cf.ThreadPoolExecutor(max_workers=jobs) as ex:
        results = list(ex.map(lambda s: compile_one(s, list(extra), out), srcs))
    objs = [o for o, _ in results]
    if verbose:
        for _, log in results:
            if log.strip():
                print(log, file=sys.stderr)
    lib = os.path.join(out, "libgcr.so")
    tmp = lib + ".tmp"
    cmd = [nvcc(), *ARCH, "-shared", "-o", tmp, *objs, "-lcudart"]
    subprocess.run(cmd, check=True)
    os.replace(tmp, lib)
    return lib


if __name__ == "__main__":
    ap = argparse.ArgumentParser()
    ap.add_argument("--jobs", type=int, default=4)
    ap.add_argument("-v", action="store_true")
    a = ap.parse_args()
    print(build(a.jobs, a.v))
