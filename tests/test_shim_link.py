"""The reference-side shim (mpi-rockstar_gb300/shim/gpu_shim.c) as a
maintainer would build it: compiled against the reference's own headers
with its build flags (the record layouts are asserted equal to the C ABI's
at compile time), linked with the reference's own objects and the GB300
library, and run through the reference's error path.  Needs the reference
checkout and its objects (oracle/_ref, built by __graft_entry__.build());
skipped where they are absent."""
import glob
import os
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SHIM = os.path.join(ROOT, "mpi-rockstar_gb300", "shim", "gpu_shim.c")
LIBDIR = os.path.join(ROOT, "mpi-rockstar_gb300", "_build")
REF_OBJ = os.path.join(ROOT, "oracle", "_ref", "obj")
FLAGS = ["-std=gnu99", "-fopenmp", "-fexceptions", "-D_DEFAULT_SOURCE",
         "-D_POSIX_C_SOURCE=200809L", "-DOUTPUT_RVMAX", "-DOUTPUT_NFW_CHI2",
         "-DOUTPUT_INERTIA_TENSOR", "-Werror=implicit-function-declaration"]


def ref_src():
    import __graft_entry__ as ge
    return ge.ref_src()


def compile_shim(tmp_path, src_dir):
    obj = tmp_path / "gpu_shim.o"
    r = subprocess.run(["gcc", "-c", *FLAGS, "-I", src_dir, "-I", os.path.join(ROOT, "include"),
                        "-I", os.path.join(ROOT, "oracle", "ref"), SHIM, "-o", str(obj)],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-3000:]
    return obj


def test_shim_compiles(tmp_path):
    src = ref_src()
    if not src:
        pytest.skip("reference sources not present")
    compile_shim(tmp_path, src)


def test_shim_links_and_aborts_without_gpu(tmp_path):
    """Linked into a reference build; without a GPU rockstar_gpu() must end
    in the reference's rockstar_abort (never a silent CPU fallback)."""
    src = ref_src()
    objs = sorted(glob.glob(os.path.join(REF_OBJ, "**", "*.o"), recursive=True))
    lib = os.path.join(LIBDIR, "librockstar_gb300.so")
    if not src or not objs or not os.path.exists(lib):
        pytest.skip("reference objects or the library not built")
    shim = compile_shim(tmp_path, src)
    exe = tmp_path / "shim_driver"
    r = subprocess.run(["gcc", *FLAGS, "-I", src, "-I", os.path.join(ROOT, "oracle", "ref"),
                        os.path.join(ROOT, "tests", "shim", "shim_driver.c"), str(shim), *objs,
                        "-L", LIBDIR, "-lrockstar_gb300", "-Wl,-rpath," + LIBDIR, "-lstdc++",
                        "-lm", "-o", str(exe)], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-3000:]
    # an internal-format particle file, read through the shim before the FOF
    import importlib.util
    spec = importlib.util.spec_from_file_location("layouts_only", os.path.join(
        ROOT, "mpi-rockstar_gb300", "layouts.py"))
    L = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(L)
    import ctypes
    import numpy as np
    q = np.zeros(300, L.PARTICLE)
    q["id"] = np.arange(300) * 3
    cfg = L.config_struct(L.Config(scale_now=0.5, box_size=75.0))
    rbin = str(tmp_path / "q.rbin")
    so = ctypes.CDLL(lib)
    assert so.rsg_write_internal(rbin.encode(), ctypes.c_void_p(q.ctypes.data),
                                 ctypes.c_int64(300), ctypes.c_int64(0), ctypes.c_int64(0),
                                 ctypes.byref(cfg)) == 0
    run = subprocess.run([str(exe), rbin], capture_output=True, text=True, timeout=300)
    assert "internal: 300 particles, id sum 134550, scale 0.500000, box 75.000" in run.stdout
    try:
        import torch
        has_gpu = torch.cuda.is_available()
    except ImportError:
        has_gpu = False
    if has_gpu:
        assert run.returncode == 0, run.stdout + run.stderr
        assert "groups" in run.stdout and "halos" in run.stdout
    else:
        assert run.returncode == 42, run.stdout + run.stderr
        assert "rockstar_abort(1)" in run.stdout
        assert "no CUDA device" in run.stderr
