"""Deterministic synthetic GADGET-2 snapshot files for the input tests.

Test infrastructure: writes a file in the layout the reference's reader takes
(src/io/io_gadget.c, src/io/io_gadget.h:8-27): Fortran records (a 4-byte
length before and after), the 256-byte header, then the POS, VEL and ID
blocks, each block optionally preceded by a tag record (variant 1: a 4-byte
tag; variant 2: the tag and the next record's length), in either byte order.
The same spec gives the same bytes on every machine, so a device-side test
can rebuild the file whose reference reading is stored as a fixture."""
import struct

import numpy as np

# name: (variant, big-endian, id bytes, coordinate bytes, particles per type,
#        header mass of type 1, redshift, flags); the halo type is 1
SPECS = {
    "v0_le_id4_f4": (0, False, 4, 4, [37, 1500, 0, 0, 11, 3], 0.0, 0.5, {}),
    "v2_be_id8_f8": (2, True, 8, 8, [5, 1203, 17, 0, 0, 0], 0.082, 1.0, {}),
    "v1_le_id8_f4": (1, False, 8, 4, [0, 777, 0, 40, 0, 0], 0.0, 0.0, {}),
    "v2_le_id4_f4_all": (2, False, 4, 4, [20, 400, 0, 0, 9, 0], 0.05, 2.0,
                         {"skip_non_halo": 0}),
    "v0_be_id4_f8_lgadget": (0, True, 4, 8, [0, 900, 3, 0, 0, 0], 0.0, 1.5,
                             {"lgadget": 1, "rescale_particle_mass": 1,
                              "length_conversion": 1e-3}),
}


def _arrays(spec, seed):
    variant, be, idb, cb, npart, m1, z, flags = spec
    rng = np.random.default_rng(seed)
    n = int(sum(npart))
    box = 75.0
    pos = rng.uniform(0, box, (n, 3))
    vel = rng.normal(0, 300.0, (n, 3))
    ids = rng.permutation(np.arange(1, n + 1, dtype=np.int64) * 7 + (1 << 33 if idb == 8 else 0))
    if idb == 4:
        ids = ids % (1 << 32)
    return pos, vel, ids, box


def header_bytes(spec, box, big):
    variant, be, idb, cb, npart, m1, z, flags = spec
    e = ">" if big else "<"
    masses = [0.0, m1, 0.0, 0.0, 0.0, 0.0]
    a = 1.0 / (1.0 + z)
    total_low = list(npart)
    total_hw = [0] * 6
    if flags.get("lgadget"):  # LGADGET keeps the high word in the next type's field
        total_low = list(npart)
        total_low[2] = 0
    h = struct.pack(e + "6I", *npart)
    h += struct.pack(e + "6d", *masses)
    h += struct.pack(e + "dd", a, z)
    h += struct.pack(e + "ii", 0, 0)
    h += struct.pack(e + "6I", *total_low)
    h += struct.pack(e + "ii", 0, 1)
    h += struct.pack(e + "dddd", box, 0.3, 0.7, 0.7)
    h += struct.pack(e + "ii", 0, 0)
    h += struct.pack(e + "6i", *total_hw)
    h += struct.pack(e + "i", 0)
    h += b"\0" * (256 - len(h))
    assert len(h) == 256
    return h


def write(path, name, seed=1):
    spec = SPECS[name]
    variant, big, idb, cb, npart, m1, z, flags = spec
    e = ">" if big else "<"
    pos, vel, ids, box = _arrays(spec, seed)
    out = bytearray()

    def rec(payload):
        out.extend(struct.pack(e + "I", len(payload)))
        out.extend(payload)
        out.extend(struct.pack(e + "I", len(payload)))

    def tag(t, nxt):
        if variant == 1:
            rec(t.ljust(4, b" ")[:4])
        elif variant == 2:
            rec(t.ljust(4, b" ")[:4] + struct.pack(e + "I", nxt + 8))

    hdr = header_bytes(spec, box, big)
    tag(b"HEAD", len(hdr))
    rec(hdr)
    ct = (">" if big else "<") + ("f8" if cb == 8 else "f4")
    for t, arr in ((b"POS ", pos), (b"VEL ", vel)):
        b = arr.astype(ct).tobytes()
        tag(t, len(b))
        rec(b)
    it = (">" if big else "<") + ("u8" if idb == 8 else "u4")
    b = ids.astype(it).tobytes()
    tag(b"ID  ", len(b))
    rec(b)
    with open(path, "wb") as f:
        f.write(bytes(out))
    return flags


def reader_kwargs(name):
    """Keyword arguments of the reader for a spec (its flags)."""
    return dict(SPECS[name][7])
