"""Catalogue output: the reference's halo filter (_should_print) and its ascii
and binary halo catalogues (src/io/meta_io.c:266-371,
src/io/io_internal.c:16-41,118-186), written by the library from halos,
links and particles, and the binary catalogue read back (load_binary_halos,
src/io/io_internal.c:199-225).  Checked against the oracle's restatement of
the same functions on any machine, and against the reference's own
output_binary and load_binary_halos where the reference is built
(oracle/_ref).  Host code: no GPU needed."""
import os
import struct

import numpy as np
import pytest

from conftest import ROOT

REF_LIB = os.path.join(ROOT, "oracle", "_ref", "libref_rockstar.so")
CASES = [(1, 0.05), (2, 1 / 32)]


def _case(rk, oracle, cfg_id, scale):
    p, box, mp, _ = rk.synth(cfg_id, scale)
    c = rk.Config(particle_mass=mp, box_size=box, total_particles=len(p))
    oracle.setup(c)
    fp, off, sz = oracle.fof(p)
    parts, halos, extra = oracle.find_subs(fp, off, sz)
    return c, box, parts, halos, extra


def _bounds(box):
    # a sub-box: some halos fall outside it
    return np.array([0.1 * box, 0.0, 0.2 * box, 0.8 * box, box, 0.9 * box], np.float32)


@pytest.mark.parametrize("cfg_id,scale", CASES)
def test_should_print(rk, oracle, cfg_id, scale):
    c, box, parts, h, e = _case(rk, oracle, cfg_id, scale)
    for b in (None, _bounds(box)):
        a = rk.should_print(h, c, b)
        assert np.array_equal(a, oracle.should_print(h, b))
        assert 0 < a.sum() < len(a)  # the filter takes some halos and drops others
    # ALWAYS_PRINT_FLAG (src/groupies.h:12) overrides the size and boundness
    # cuts, but not the bounds
    drop = np.flatnonzero(~rk.should_print(h, c))
    h2 = h.copy()
    h2["flags"][drop] |= 16
    assert rk.should_print(h2, c).all()
    assert np.array_equal(rk.should_print(h2, c, _bounds(box)), oracle.should_print(h2, _bounds(box)))


@pytest.mark.parametrize("cfg_id,scale", CASES)
def test_ascii_matches_oracle(rk, oracle, tmp_path, cfg_id, scale):
    c, box, parts, h, e = _case(rk, oracle, cfg_id, scale)
    for k, (b, np_, off) in enumerate([(None, len(parts), 0), (_bounds(box), 0, 1000)]):
        ours, ref = tmp_path / ("a%d.list" % k), tmp_path / ("b%d.list" % k)
        rk.write_ascii(str(ours), h, e, c, id_offset=off, bounds=b, num_p=np_)
        oracle.write_ascii(str(ref), h, e, id_offset=off, bounds=b, num_p=np_)
        got, want = ours.read_bytes(), ref.read_bytes()
        assert got == want
        lines = got.decode().splitlines()
        rows = [ln for ln in lines if not ln.startswith("#")]
        assert len(rows) == int(rk.should_print(h, c, b).sum())
        assert rows[0].split()[0] == str(off)  # ids count from id_offset
        assert len(rows[0].split()) == len(lines[0].split())  # one value per column


@pytest.mark.parametrize("cfg_id,scale", CASES)
def test_binary_matches_oracle(rk, oracle, tmp_path, cfg_id, scale):
    c, box, parts, h, e = _case(rk, oracle, cfg_id, scale)
    for k, b in enumerate((None, _bounds(box))):
        ours, ref = tmp_path / ("a%d.bin" % k), tmp_path / ("b%d.bin" % k)
        rk.write_binary(str(ours), h, parts, c, id_offset=5, snap=3, chunk=1, bounds=b)
        oracle.write_binary(str(ref), h, parts, id_offset=5, snap=3, chunk=1, bounds=b)
        assert ours.read_bytes() == ref.read_bytes()


@pytest.mark.skipif(not os.path.exists(REF_LIB), reason="reference oracle not built")
@pytest.mark.parametrize("cfg_id,scale", CASES)
def test_binary_matches_reference(rk, oracle, tmp_path, cfg_id, scale):
    """The same bytes as the reference's own output_binary."""
    from oracle import refcall
    c, box, parts, h, e = _case(rk, oracle, cfg_id, scale)
    refcall.setup(c)
    for k, b in enumerate((None, _bounds(box))):
        ours, ref = tmp_path / ("a%d.bin" % k), tmp_path / ("r%d.bin" % k)
        rk.write_binary(str(ours), h, parts, c, id_offset=5, snap=3, chunk=1, bounds=b)
        refcall.output_binary(str(ref), h, parts, id_offset=5, snap=3, chunk=1, bounds=b)
        assert ours.read_bytes() == ref.read_bytes()


def test_binary_layout(rk, oracle, tmp_path):
    """Header fields, halo records and particle ids of the binary file."""
    c, box, parts, h, e = _case(rk, oracle, 1, 0.05)
    path = tmp_path / "h.bin"
    rk.write_binary(str(path), h, parts, c, id_offset=7, snap=12, chunk=2)
    raw = path.read_bytes()
    magic, snap, chunk = struct.unpack_from("<Qqq", raw, 0)
    scale, om, ol, h0 = struct.unpack_from("<4f", raw, 24)
    bounds = struct.unpack_from("<6f", raw, 40)
    nh, npart = struct.unpack_from("<qq", raw, 64)
    box_size, pmass = struct.unpack_from("<2f", raw, 80)
    ptype, rev = struct.unpack_from("<qi", raw, 88)
    version = raw[100:112].split(b"\0")[0]
    add_flag = struct.unpack_from("<i", raw, 112)[0]
    assert (magic, snap, chunk) == (0xfadedacec0c0d0d0, 12, 2)
    assert (ptype, rev, version, add_flag) == (1, 2, b"1.0.0RC", 5)
    assert np.isclose(box_size, box) and np.isclose(om, c.om)
    keep = rk.should_print(h, c)
    assert nh == keep.sum() and npart == h["num_p"][keep].sum()
    assert len(raw) == 256 + nh * h.dtype.itemsize + npart * 8
    recs = np.frombuffer(raw, h.dtype, nh, 256)
    assert np.array_equal(recs["id"], 7 + np.arange(nh))
    assert np.array_equal(recs["p_start"], np.concatenate([[0], np.cumsum(recs["num_p"])[:-1]]))
    ids = np.frombuffer(raw, np.int64, npart, 256 + nh * h.dtype.itemsize)
    want = np.concatenate([parts["id"][s:s + n] for s, n in
                           zip(h["p_start"][keep], h["num_p"][keep])])
    assert np.array_equal(ids, want)
    pos = h["pos"][keep][:, :3]
    # extent of the printed halos; the running min/max start from halo 0
    lo = np.minimum(pos.min(0), h["pos"][0, :3])
    hi = np.maximum(pos.max(0), h["pos"][0, :3])
    assert np.array_equal(np.array(bounds, np.float32), np.concatenate([lo, hi]))


def test_empty_and_bad_arguments(rk, oracle, tmp_path):
    c, box, parts, h, e = _case(rk, oracle, 1, 0.05)
    empty = h[:0]
    rk.write_binary(str(tmp_path / "e.bin"), empty, parts, c)
    oracle.write_binary(str(tmp_path / "o.bin"), empty, parts)
    assert (tmp_path / "e.bin").read_bytes() == (tmp_path / "o.bin").read_bytes()
    assert len((tmp_path / "e.bin").read_bytes()) == 256
    rk.write_ascii(str(tmp_path / "e.list"), empty, e[:0], c)
    oracle.write_ascii(str(tmp_path / "o.list"), empty, e[:0])
    assert (tmp_path / "e.list").read_bytes() == (tmp_path / "o.list").read_bytes()
    # a halo whose particles lie outside the given particle array
    bad = h.copy()
    keep = np.flatnonzero(rk.should_print(h, c))
    bad["p_start"][keep[0]] = len(parts)
    with pytest.raises(rk.RockstarError) as ex:
        rk.write_binary(str(tmp_path / "x.bin"), bad, parts, c)
    assert ex.value.code == -1
    with pytest.raises(rk.RockstarError) as ex:
        rk.write_ascii(str(tmp_path / "no" / "such" / "dir.list"), h, e, c)
    assert ex.value.code == -7


def _canon_nan(h):
    # NaN payloads differ between the GPU and a host CPU (0/0 gives a
    # different bit pattern, printed "nan" or "-nan"); the catalogue compare
    # is about the writer and the values, so NaNs are made one pattern
    h = h.copy()
    for name in h.dtype.names:
        a = h[name]
        if a.dtype.kind == "f":
            a[np.isnan(a)] = np.float32("nan")
    return h


@pytest.mark.gpu
@pytest.mark.parametrize("cfg_id,scale", CASES)
def test_catalog_from_gpu_path(rk, oracle, tmp_path, cfg_id, scale):
    """End to end: the 3D FOF and the plain substructure form on the GPU, then
    the catalogues, against the oracle's path and writers."""
    c, box, parts, h, e = _case(rk, oracle, cfg_id, scale)
    p, _, _, _ = rk.synth(cfg_id, scale)
    fp, off, sz = rk.rockstar_fof(p, c)
    gparts, gh, ge = rk.find_subs(fp, off, sz, c)
    assert gparts.tobytes() == parts.tobytes()
    gh, h = _canon_nan(gh), _canon_nan(h)
    rk.write_ascii(str(tmp_path / "g.list"), gh, ge, c, num_p=len(gparts))
    oracle.write_ascii(str(tmp_path / "o.list"), h, e, num_p=len(parts))
    assert (tmp_path / "g.list").read_bytes() == (tmp_path / "o.list").read_bytes()
    rk.write_binary(str(tmp_path / "g.bin"), gh, gparts, c)
    oracle.write_binary(str(tmp_path / "o.bin"), h, parts)
    assert (tmp_path / "g.bin").read_bytes() == (tmp_path / "o.bin").read_bytes()


@pytest.mark.parametrize("cfg_id,scale", CASES)
def test_read_binary_round_trip(rk, oracle, tmp_path, cfg_id, scale):
    """rsg_read_binary returns what rsg_write_binary wrote: the printable
    halos (id and p_start rewritten), their particles' ids, the header and
    the configuration values read_binary_header_config sets."""
    c, box, parts, h, e = _case(rk, oracle, cfg_id, scale)
    path = str(tmp_path / "c.bin")
    rk.write_binary(path, h, parts, c, id_offset=7, snap=4, chunk=2)
    hdr, hh, ids, cfg = rk.read_binary(path, rk.Config())
    keep = rk.should_print(h, c)
    kept = h[keep]
    assert hdr.magic == 0xfadedacec0c0d0d0 and hdr.snap == 4 and hdr.chunk == 2
    assert hdr.num_halos == len(kept) == len(hh) and hdr.particle_type == 1
    assert np.array_equal(hh["id"], np.arange(len(kept)) + 7)
    starts = np.concatenate([[0], np.cumsum(kept["num_p"])[:-1]])
    assert np.array_equal(hh["p_start"], starts)
    for f in ("num_p", "m", "r", "vmax", "pos"):
        assert hh[f].tobytes() == kept[f].tobytes()
    want = np.concatenate([parts["id"][s:s + n] for s, n in zip(kept["p_start"], kept["num_p"])])
    assert np.array_equal(ids, want)
    assert cfg["box_size"] == float(np.float32(c.box_size))
    assert cfg["particle_mass"] == float(np.float32(c.particle_mass))


@pytest.mark.skipif(not os.path.exists(REF_LIB), reason="reference oracle not built")
@pytest.mark.parametrize("cfg_id,scale", CASES)
def test_read_binary_matches_reference(rk, oracle, tmp_path, cfg_id, scale):
    """The same header, halos, ids and configuration values as the
    reference's load_binary_halos on the reference's own output_binary."""
    from oracle import refcall
    c, box, parts, h, e = _case(rk, oracle, cfg_id, scale)
    path = str(tmp_path / "r.bin")
    refcall.output_binary(path, h, parts, id_offset=3, snap=9, chunk=0, bounds=_bounds(box))
    rhdr, rh, rids, rcfg = refcall.load_binary(path)
    hdr, hh, ids, cfg = rk.read_binary(path, rk.Config())
    assert bytes(hdr) == rhdr.tobytes()
    assert hh.tobytes() == rh.tobytes() and np.array_equal(ids, rids)
    assert cfg == rcfg


def test_read_binary_errors(rk, tmp_path):
    c = rk.Config()
    good = str(tmp_path / "empty.bin")
    rk.write_binary(good, np.zeros(0, rk.HALO), np.zeros(0, rk.PARTICLE), c)
    hdr, hh, ids, _ = rk.read_binary(good, c)
    assert hdr.num_halos == 0 and len(hh) == 0 and len(ids) == 0
    raw = open(good, "rb").read()
    cases = {
        "short.bin": raw[:200],
        "magic.bin": b"\1" + raw[1:],
        "count.bin": raw[:64] + struct.pack("<q", 3) + raw[72:],  # 3 halos announced, none stored
        "neg.bin": raw[:72] + struct.pack("<q", -1) + raw[80:],
    }
    for name, data in cases.items():
        path = str(tmp_path / name)
        open(path, "wb").write(data)
        with pytest.raises(rk.RockstarError) as ex:
            rk.read_binary(path, c)
        assert ex.value.code == -7, name


@pytest.mark.parametrize("cfg_id,scale", CASES)
def test_particles_table_matches_oracle(rk, oracle, tmp_path, cfg_id, scale):
    """output_full_particles: filtered and unfiltered, every particle or
    every n-th id, with and without bounds; same bytes and same ids."""
    c, box, parts, h, e = _case(rk, oracle, cfg_id, scale)
    assert (e["child"] > -1).any()  # the recursion over children is exercised
    opts = [dict(), dict(unfiltered=1), dict(every_n=7, id_offset=100),
            dict(bounds=_bounds(box), num_p=0, strict_so_masses=1)]
    for k, kw in enumerate(opts):
        ours, ref = tmp_path / ("a%d.particles" % k), tmp_path / ("b%d.particles" % k)
        kw.setdefault("num_p", len(parts))
        ids = rk.write_particles(str(ours), h, e, parts, c, **kw)
        want = oracle.write_particles(str(ref), h, e, parts, **kw)
        assert ours.read_bytes() == ref.read_bytes()
        assert np.array_equal(ids, want)
        assert np.array_equal(ids > -1, rk.should_print(h, c, kw.get("bounds")))


def test_particles_table_bad_links(rk, oracle, tmp_path):
    c, box, parts, h, e = _case(rk, oracle, 1, 0.05)
    parent = int(np.flatnonzero(e["child"] > -1)[0])
    for bad in ("loop", "range"):
        e2 = e.copy()
        if bad == "loop":
            e2["child"][e["child"][parent]] = parent
        else:
            e2["next_cochild"][e["child"][parent]] = len(h) + 5
        with pytest.raises(rk.RockstarError) as ex:
            rk.write_particles(str(tmp_path / "x.particles"), h, e2, parts, c, unfiltered=1)
        assert ex.value.code == -1
