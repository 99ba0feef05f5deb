"""Builds the GB300 extension in-tree (no cmake, no setuptools).

  _build/librockstar_gb300.so  - CUDA kernels + C ABI (nvcc, sm_103a only)
  _build/libsynth.so           - seeded synthetic snapshot generator (gcc)

Translation units are compiled in parallel; outputs are only rebuilt when a
source or header is newer.
"""
import concurrent.futures as cf
import glob
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
OUT = os.path.join(HERE, "_build")
INC = os.path.join(ROOT, "include")
ARCH = "-gencode=arch=compute_103a,code=sm_103a"
NVCC_FLAGS = ["-O3", "-lineinfo", "-std=c++17", ARCH, "--fmad=false", "-Xcompiler", "-fPIC",
              "-Xptxas", "-O3", "--expt-relaxed-constexpr", "-I", INC, "-I", CSRC]
LIB = os.path.join(OUT, "librockstar_gb300.so")
SYNTH = os.path.join(OUT, "libsynth.so")


def _nvcc():
    for c in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", shutil.which("nvcc")):
        if c and os.path.exists(c):
            return c
    raise RuntimeError("nvcc not found")


def _newest(paths):
    return max(os.path.getmtime(p) for p in paths)


def _compile(src, deps):
    obj = os.path.join(OUT, os.path.basename(src) + ".o")
    if os.path.exists(obj) and os.path.getmtime(obj) >= _newest([src] + deps):
        return obj
    cmd = [_nvcc(), *NVCC_FLAGS, "-c", src, "-o", obj + ".tmp"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("nvcc failed for %s:\n%s" % (src, r.stderr[-6000:]))
    os.replace(obj + ".tmp", obj)
    return obj


def build(verbose=False):
    os.makedirs(OUT, exist_ok=True)
    headers = glob.glob(os.path.join(CSRC, "*.cuh")) + glob.glob(os.path.join(INC, "*.h"))
    srcs = sorted(glob.glob(os.path.join(CSRC, "*.cu")))
    with cf.ThreadPoolExecutor(max_workers=min(8, len(srcs))) as ex:
        objs = list(ex.map(lambda s: _compile(s, headers), srcs))
    if not (os.path.exists(LIB) and os.path.getmtime(LIB) >= _newest(objs)):
        tmp = LIB + ".tmp%d" % os.getpid()
        cmd = [_nvcc(), ARCH, "-shared", "-o", tmp, *objs, "-lcudart"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("link failed:\n" + r.stderr[-4000:])
        os.replace(tmp, LIB)
    ssrc = os.path.join(CSRC, "synth.c")
    if not (os.path.exists(SYNTH) and os.path.getmtime(SYNTH) >= os.path.getmtime(ssrc)):
        tmp = SYNTH + ".tmp%d" % os.getpid()
        subprocess.check_call(["gcc", "-O2", "-fopenmp", "-fPIC", "-shared", "-std=c99",
                               "-D_DEFAULT_SOURCE", "-ffp-contract=off", "-o", tmp, ssrc, "-lm"])
        os.replace(tmp, SYNTH)
    if verbose:
        print("built", LIB, SYNTH)
    return LIB


if __name__ == "__main__":
    build(verbose=True)
    sys.exit(0)
