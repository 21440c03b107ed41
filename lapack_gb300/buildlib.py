"""Builds liblapack_gb300.so in-tree: every CUDA translation unit for
sm_103a (one -gencode), compiled in parallel, linked into one shared
library next to this file."""
import concurrent.futures as cf
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "liblapack_gb300.so")
NVCC = os.environ.get("NVCC", "nvcc")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
# host code is compiled without floating-point contraction (-ffp-contract=off):
# host-side arithmetic then rounds the same on x86-64 and on AArch64
COMMON = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "-Xcompiler", "-fvisibility=default",
          "-Xcompiler", "-ffp-contract=off", "--expt-relaxed-constexpr"]
SOURCES = ["getrf.cu", "trsm.cu", "panel_node.cu", "panel_node_f64.cu", "mixed.cu", "gemm_tc.cu", "capi.cu", "prof.cu", "noalloc.cu", "batched.cu", "adjoint.cu", "refine.cu", "chol.cu", "zlu.cu", "zlu_tiles.cu", "lapacke.cpp"]


def _sources():
    return [os.path.join(CSRC, s) for s in SOURCES] + \
        [os.path.join(CSRC, s) for s in sorted(os.listdir(CSRC)) if s.endswith((".cuh", ".h"))] + \
        [os.path.join(HERE, "..", "include", "lapack_gb300.h")]


def up_to_date():
    if not os.path.exists(LIB):
        return False
    t = os.path.getmtime(LIB)
    return all(os.path.getmtime(p) <= t for p in _sources() if os.path.exists(p))


def _compile(src, extra):
    obj = os.path.join(BUILD, os.path.basename(src) + ".o")
    if src.endswith(".cpp"):
        cmd = [NVCC, "-x", "c++"] + COMMON + ["-c", src, "-o", obj]
    else:
        cmd = [NVCC] + ARCH + COMMON + extra + ["-c", src, "-o", obj]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"compile failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    return obj, r.stderr


def build(verbose=False, force=False, ptxas_info=False):
    if not force and up_to_date():
        return LIB
    os.makedirs(BUILD, exist_ok=True)
    extra = ["-Xptxas", "-v"] if ptxas_info else []
    srcs = [os.path.join(CSRC, s) for s in SOURCES]
    with cf.ThreadPoolExecutor(max_workers=min(8, os.cpu_count() or 1)) as ex:
        results = list(ex.map(lambda s: _compile(s, extra), srcs))
    if verbose:
        for _, err in results:
            if err.strip():
                print(err, file=sys.stderr)
    objs = [o for o, _ in results]
    tmp = LIB + ".tmp"
    cmd = [NVCC] + ARCH + ["-shared", "-o", tmp] + objs + ["-lcudart"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    build(verbose=True, force="--force" in sys.argv, ptxas_info="--ptxas" in sys.argv)
    print(LIB)
