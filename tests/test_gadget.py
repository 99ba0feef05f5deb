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
    w = parts.copy()
    rk.sort_by_id(w, inplace=True)
    assert w.tobytes() == z["sorted"].tobytes()


def test_sort_by_id_inplace_needs_a_particle_array(rk):
    p = np.zeros(10, rk.PARTICLE)
    with pytest.raises(ValueError):
        rk.sort_by_id(p[::2], inplace=True)
    with pytest.raises(ValueError):
        rk.sort_by_id(p.tolist(), inplace=True)


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


@pytest.mark.gpu
@pytest.mark.parametrize("name", NAMES)
def test_read_gadget2_device(rk, tmp_path, name):
    """The records left in device memory are the reference reader's."""
    path, z = rebuild(tmp_path, name)
    c = rk.Config(particle_mass=float(z["particle_mass_in"]), box_size=1.0, total_particles=1)
    d, cfg = rk.read_gadget2_device(path, c, **GF.reader_kwargs(name))
    assert d.cpu().numpy().tobytes() == z["particles"].tobytes()
    check_cfg(cfg, z["cfg"].tolist())
    rk.sort_by_id_device(d)
    assert d.cpu().numpy().tobytes() == z["sorted"].tobytes()


@pytest.mark.gpu
def test_sort_by_id_id_ranges(rk):
    """Ids over the whole int64 range, and all ids equal (order kept)."""
    rng = np.random.default_rng(5)
    p = np.zeros(3000, rk.PARTICLE)
    p["id"] = rng.integers(np.iinfo(np.int64).min, np.iinfo(np.int64).max, len(p),
                           dtype=np.int64, endpoint=True)
    p["id"][:2] = [np.iinfo(np.int64).min, np.iinfo(np.int64).max]
    p["pos"][:, 0] = np.arange(len(p))
    assert rk.sort_by_id(p).tobytes() == p[np.argsort(p["id"], kind="stable")].tobytes()
    p["id"] = 77
    assert rk.sort_by_id(p).tobytes() == p.tobytes()


@pytest.mark.gpu
def test_input_staging_large(rk, tmp_path):
    """Transfers of many staging chunks on several threads: a 40 MB file read
    to the host and to the device, and a 96 MB id sort, against the CPU
    restatement bench.py times."""
    import sys
    import torch
    sys.path.insert(0, ROOT)
    import bench
    n = 1_250_001
    path = str(tmp_path / "big.g2")
    bench.io_write_gadget(path, n)
    want = bench.io_cpu_read(path, n, rk.PARTICLE)
    c = rk.Config(particle_mass=1e9, box_size=1.0, total_particles=1)
    got, cfg = rk.read_gadget2(path, c)
    assert got.tobytes() == want.tobytes() and cfg["total_particles"] == n
    d, _ = rk.read_gadget2_device(path, c)
    assert d.cpu().numpy().tobytes() == want.tobytes()
    order = np.argsort(want["id"], kind="stable")
    big = np.concatenate([want, want[::-1], want[:500_000]])
    big["id"][n:] = -big["id"][n:]
    assert rk.sort_by_id(big).tobytes() == big[np.argsort(big["id"], kind="stable")].tobytes()
    rk.sort_by_id_device(d)
    assert d.cpu().numpy().tobytes() == want[order].tobytes()
    # a file cut inside the position payload
    raw = open(path, "rb").read()
    cut = str(tmp_path / "cut.g2")
    open(cut, "wb").write(raw[: 300 + 12 * n // 2])
    with pytest.raises(rk.RockstarError) as e:
        rk.read_gadget2_device(cut, c)
    assert e.value.code == -7
    torch.cuda.synchronize()


def write_plain_gadget(path, parts, box, particle_mass):
    """An untagged little-endian GADGET-2 file of type-1 particles at a = 1
    (velocities unscaled), float coordinates and 8-byte ids."""
    n = len(parts)
    npart = [0, n, 0, 0, 0, 0]
    hdr = struct.pack("<6I6ddd2i6I2i4d2i6ii", *npart, 0, particle_mass / 1e10, 0, 0, 0, 0,
                      1.0, 0.0, 0, 0, *npart, 0, 1, box, 0.3, 0.7, 0.7, *([0] * 9))
    with open(path, "wb") as f:
        for blob in (hdr.ljust(256, b"\0"), parts["pos"][:, :3].astype("<f4").tobytes(),
                     parts["pos"][:, 3:].astype("<f4").tobytes(), parts["id"].astype("<i8").tobytes()):
            f.write(struct.pack("<I", len(blob)) + blob + struct.pack("<I", len(blob)))


@pytest.mark.gpu
def test_file_to_halos_on_device(rk, tmp_path):
    """A clustered snapshot: file -> device records -> device id sort ->
    rsg_path_device gives the same particles, groups and halos as the host
    reader, the host sort and an upload."""
    import torch
    p, box, mp, _ = rk.synth(2, 0.125, 11)
    rng = np.random.default_rng(4)
    p = p[rng.permutation(len(p))]
    path = str(tmp_path / "clustered.g2")
    write_plain_gadget(path, p, box, mp)
    c = rk.Config(particle_mass=mp, box_size=box, total_particles=len(p))
    d, cfg = rk.read_gadget2_device(path, c)
    rk.sort_by_id_device(d)
    n = d.numel() // rk.PARTICLE.itemsize
    assert n == len(p)
    run_cfg = rk.Config(particle_mass=cfg["particle_mass"], box_size=cfg["box_size"],
                        total_particles=int(cfg["total_particles"]))
    host_sorted = rk.sort_by_id(rk.read_gadget2(path, c)[0])
    assert host_sorted.tobytes() == p[np.argsort(p["id"], kind="stable")].tobytes()
    a = rk.DevicePath(n, run_cfg)
    ra = a.run(d.data_ptr())
    up = torch.from_numpy(host_sorted.view(np.uint8).copy()).cuda()
    b = rk.DevicePath(n, run_cfg)
    rb = b.run(up.data_ptr())
    assert ra == rb and ra[1] > 0 and ra[2] > 0
    for x, y in zip(a.results(), b.results()):
        assert x.tobytes() == y.tobytes()
