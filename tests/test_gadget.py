"""Particle input: the GADGET-2 reader and the id sort, against the
reference's own load_particles_gadget2 (src/io/io_gadget.c) and its id sort
(src/mpi_main.cpp:2021-2024) through the fixtures of
tests/golden/make_gadget_golden.py.  The synthetic files are rebuilt from
tests/gadget_files.py byte for byte (checked by hash)."""
import ctypes
import ctypes.util
import hashlib
import os
import struct

import numpy as np
import pytest

import gadget_files as GF
from conftest import ROOT

GOLD = os.path.join(ROOT, "tests", "golden")
REF_LIB = os.path.join(ROOT, "oracle", "_ref", "libref_rockstar.so")
NAMES = sorted(GF.SPECS)
FIELDS = ("om", "ol", "h0", "box_size", "total_particles", "scale_now", "particle_mass",
          "avg_particle_spacing")
CRITICAL_DENSITY = 2.77519737e11  # src/universal_constants.h:5


def check_cfg(cfg, want):
    """All values exact except AVG_PARTICLE_SPACING = cbrt(PARTICLE_MASS /
    (Om * CRITICAL_DENSITY)) (src/io/io_gadget.c:172): the C library's cbrt
    is accurate to a few ulps, not correctly rounded, and the x86-64 and
    AArch64 builds of glibc give results up to two ulps apart for some
    arguments, so that value must equal this machine's cbrt of the same
    argument (what the reference computes here) and lie within four ulps of
    the stored one."""
    got = [float(cfg[k]) for k in FIELDS]
    assert got[:-1] == want[:-1]
    libm = ctypes.CDLL(ctypes.util.find_library("m"))
    libm.cbrt.restype = ctypes.c_double
    libm.cbrt.argtypes = [ctypes.c_double]
    assert got[-1] == libm.cbrt(got[6] / (got[0] * CRITICAL_DENSITY))
    assert abs(got[-1] - want[-1]) <= 4 * np.spacing(want[-1])


def fixture(name):
    return np.load(os.path.join(GOLD, "gadget_%s.npz" % name))


def rebuild(tmp_path, name):
    path = str(tmp_path / (name + ".g2"))
    GF.write(path, name)
    z = fixture(name)
    assert hashlib.sha256(open(path, "rb").read()).hexdigest() == str(z["sha256"])
    return path, z


@pytest.mark.parametrize("name", NAMES)
def test_files_rebuild_identically(tmp_path, name):
    rebuild(tmp_path, name)


@pytest.mark.skipif(not os.path.exists(REF_LIB), reason="reference oracle not built")
@pytest.mark.parametrize("name", NAMES)
def test_reference_reader_gives_fixture(tmp_path, name):
    from oracle import refcall
    path, z = rebuild(tmp_path, name)
    parts, cfg = refcall.load_gadget2(path, particle_mass=float(z["particle_mass_in"]),
                                      **GF.reader_kwargs(name))
    assert parts.view(np.uint8).tobytes() == z["particles"].tobytes()
    check_cfg(cfg, z["cfg"].tolist())


@pytest.mark.gpu
@pytest.mark.parametrize("name", NAMES)
def test_read_gadget2(rk, tmp_path, name):
    """Same particle bytes (file order, rescaled) and configuration values as
    the reference's reader."""
    path, z = rebuild(tmp_path, name)
    c = rk.Config(particle_mass=float(z["particle_mass_in"]), box_size=1.0, total_particles=1)
    parts, cfg = rk.read_gadget2(path, c, **GF.reader_kwargs(name))
    assert parts.view(np.uint8).tobytes() == z["particles"].tobytes()
    check_cfg(cfg, z["cfg"].tolist())


@pytest.mark.gpu
@pytest.mark.parametrize("name", NAMES)
def test_sort_by_id(rk, name):
    z = fixture(name)
    parts = z["particles"].view(rk.PARTICLE)
    got = rk.sort_by_id(parts)
    assert got.view(np.uint8).tobytes() == z["sorted"].tobytes()
    assert rk.sort_by_id(parts[:0]).size == 0 and rk.sort_by_id(parts[:1]).tobytes() == parts[:1].tobytes()


@pytest.mark.gpu
def test_sort_by_id_negative_and_equal_ids(rk):
    """Signed order, and equal ids keep their input order (stable)."""
    rng = np.random.default_rng(3)
    p = np.zeros(5000, rk.PARTICLE)
    p["id"] = rng.integers(-50, 50, len(p))
    p["pos"][:, 0] = np.arange(len(p))
    got = rk.sort_by_id(p)
    want = p[np.argsort(p["id"], kind="stable")]
    assert got.tobytes() == want.tobytes()


@pytest.mark.gpu
def test_read_gadget2_errors(rk, tmp_path):
    c = rk.Config(particle_mass=2.5e10, box_size=1.0, total_particles=1)
    path, z = rebuild(tmp_path, "v0_le_id4_f4")
    raw = open(path, "rb").read()
    # truncated in the ID block
    bad = str(tmp_path / "cut.g2")
    open(bad, "wb").write(raw[:-100])
    with pytest.raises(rk.RockstarError) as e:
        rk.read_gadget2(bad, c)
    assert e.value.code == -7
    # a curved cosmology (Om + Ol != 1): the reference stops
    curved = bytearray(raw)
    curved[4 + 136:4 + 144] = struct.pack("<d", 0.5)
    bad2 = str(tmp_path / "curved.g2")
    open(bad2, "wb").write(bytes(curved))
    with pytest.raises(rk.RockstarError) as e:
        rk.read_gadget2(bad2, c)
    assert e.value.code == -5
    with pytest.raises(rk.RockstarError) as e:
        rk.read_gadget2(str(tmp_path / "missing.g2"), c)
    assert e.value.code == -7


@pytest.mark.skipif(not os.path.exists(REF_LIB), reason="reference oracle not built")
def test_bench_input_port_equals_reference(tmp_path):
    """The CPU restatement bench.py times beside the device reader reads its
    file as the reference's reader does."""
    import sys
    sys.path.insert(0, ROOT)
    import bench
    from oracle import refcall
    rk_dtype = np.dtype([("id", "<i8"), ("pos", "<f4", (6,))])
    for n in (1, 4321):
        path = str(tmp_path / ("io%d.g2" % n))
        bench.io_write_gadget(path, n)
        got = bench.io_cpu_read(path, n, rk_dtype)
        want, cfg = refcall.load_gadget2(path, particle_mass=1e9)
        assert got.tobytes() == want.view(np.uint8).tobytes()
        assert cfg["scale_now"] == bench.IO_SCALE and cfg["total_particles"] == n
