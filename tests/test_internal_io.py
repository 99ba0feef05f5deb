"""The reference's internal particle format: rsg_write_internal against the
bytes of the reference's own output_particles_internal, rsg_read_internal
and rsg_read_internal_device against its load_particles_internal
(src/io/io_internal.c:43-100), through the fixtures of
tests/golden/make_internal_golden.py.  The host variants are file I/O with
no device step, so they are checked here on the CPU."""
import os
import struct

import numpy as np
import pytest

from conftest import ROOT

GOLD = os.path.join(ROOT, "tests", "golden")
REF_LIB = os.path.join(ROOT, "oracle", "_ref", "libref_rockstar.so")
NAMES = ("rbin_777", "rbin_empty")
FIELDS = ("scale_now", "om", "ol", "h0", "box_size", "particle_mass")


def fixture(name):
    return np.load(os.path.join(GOLD, "internal_%s.npz" % name))


def config(rk, values):
    c = rk.Config()
    for k, v in zip(FIELDS, values):
        setattr(c, k, float(v))
    return c


@pytest.mark.parametrize("name", NAMES)
def test_write_internal_equals_reference_bytes(rk, tmp_path, name):
    z = fixture(name)
    path = str(tmp_path / "out.rbin")
    parts = z["particles"].view(rk.PARTICLE)
    rk.write_internal(path, parts, config(rk, z["cfg_in"]), int(z["snap"]), int(z["chunk"]))
    assert open(path, "rb").read() == z["raw_file"].tobytes()


@pytest.mark.parametrize("name", NAMES)
def test_read_internal_equals_reference(rk, tmp_path, name):
    z = fixture(name)
    path = str(tmp_path / "in.rbin")
    z["raw_file"].tofile(path)
    got, cfg = rk.read_internal(path, rk.Config())
    assert got.tobytes() == z["particles"].tobytes()
    assert [cfg[k] for k in FIELDS] == z["cfg_out"].tolist()


@pytest.mark.skipif(not os.path.exists(REF_LIB), reason="reference oracle not built")
def test_reference_reads_what_the_library_writes(rk, tmp_path):
    from oracle import refcall
    rng = np.random.default_rng(9)
    p = np.zeros(5000, rk.PARTICLE)
    p["id"] = rng.permutation(5000)
    p["pos"] = rng.normal(0, 30, (5000, 6))
    c = config(rk, [0.25, 0.31, 0.69, 0.68, 100.0, 3.3e8])
    path = str(tmp_path / "lib.rbin")
    rk.write_internal(path, p, c, 7, 2)
    got, cfg = refcall.load_internal(path)
    assert got.tobytes() == p.tobytes()
    assert cfg == rk.read_internal(path, rk.Config())[1]


def test_read_internal_large_parallel(rk, tmp_path):
    """Many 8 MiB chunks read by several threads."""
    n = 1_500_017
    p = np.zeros(n, rk.PARTICLE)
    p["id"] = np.arange(n, dtype=np.int64) * 5 - 7
    p["pos"] = np.arange(6 * n, dtype=np.float32).reshape(n, 6)
    path = str(tmp_path / "big.rbin")
    rk.write_internal(path, p, rk.Config(), 1, 0)
    assert os.path.getsize(path) == 256 + 32 * n
    got, _ = rk.read_internal(path, rk.Config())
    assert got.tobytes() == p.tobytes()


def test_read_internal_errors(rk, tmp_path):
    z = fixture("rbin_777")
    raw = z["raw_file"].tobytes()
    cases = {
        "cut.rbin": raw[:-1],                                  # truncated records
        "short.rbin": raw[:100],                               # truncated header
        "magic.rbin": b"\0" * 8 + raw[8:],                     # not a Rockstar file
        "ids.rbin": raw[:88] + struct.pack("<q", 1) + raw[96:],  # a halo catalogue's ids
    }
    for fname, data in cases.items():
        path = str(tmp_path / fname)
        open(path, "wb").write(data)
        with pytest.raises(rk.RockstarError) as e:
            rk.read_internal(path, rk.Config())
        assert e.value.code == -7, fname
    with pytest.raises(rk.RockstarError) as e:
        rk.read_internal(str(tmp_path / "missing.rbin"), rk.Config())
    assert e.value.code == -7


@pytest.mark.gpu
@pytest.mark.parametrize("name", NAMES)
def test_read_internal_device(rk, tmp_path, name):
    """The records in device memory are the reference reader's."""
    z = fixture(name)
    path = str(tmp_path / "in.rbin")
    z["raw_file"].tofile(path)
    d, cfg = rk.read_internal_device(path, rk.Config())
    assert d.cpu().numpy().tobytes() == z["particles"].tobytes()
    assert [cfg[k] for k in FIELDS] == z["cfg_out"].tolist()


@pytest.mark.gpu
def test_read_internal_device_large(rk, tmp_path):
    n = 1_500_017
    p = np.zeros(n, rk.PARTICLE)
    p["id"] = n - np.arange(n, dtype=np.int64)
    p["pos"] = np.arange(6 * n, dtype=np.float32).reshape(n, 6)
    path = str(tmp_path / "big.rbin")
    rk.write_internal(path, p, rk.Config(), 1, 0)
    d, _ = rk.read_internal_device(path, rk.Config())
    assert d.cpu().numpy().tobytes() == p.tobytes()
    rk.sort_by_id_device(d)
    assert d.cpu().numpy().tobytes() == p[::-1].tobytes()


def test_internal_io_arguments(rk, tmp_path):
    import ctypes as C
    z = fixture("rbin_777")
    path = str(tmp_path / "in.rbin")
    z["raw_file"].tofile(path)
    st = rk.config_struct(rk.Config())
    n = np.zeros(1, np.int64)
    buf = np.zeros(10, rk.PARTICLE)
    # too few places for the file's particles
    rc = rk.lib().rsg_read_internal(path.encode(), C.byref(st), buf.ctypes.data, len(buf),
                                    n.ctypes.data)
    assert rc == -1 and n[0] == 777
    # an unwritable destination
    with pytest.raises(rk.RockstarError) as e:
        rk.write_internal(str(tmp_path / "no" / "dir" / "x.rbin"), buf, rk.Config())
    assert e.value.code == -7
