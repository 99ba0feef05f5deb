"""Generates the fixtures of the reference's internal particle format.

Run in a checkout where the reference sources are present (oracle/_ref is
built from them by oracle/ref/Makefile, which compiles src/io/io_internal.c):

    python tests/golden/make_internal_golden.py

For each case it writes a particle set with the reference's own
output_particles_internal(snap, chunk, 1) and reads the file back with its
load_particles_internal (src/io/io_internal.c:52-100), and stores,
compressed: the file's bytes, the particles and configuration given to the
writer, and the particles and configuration values the reader returns.
"""
import os
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle import refcall  # noqa: E402
from oracle import layouts as L  # noqa: E402

CASES = {
    # name: (particles, seed, snap, chunk, configuration given to the writer)
    "rbin_777": (777, 3, 61, 5, {"scale_now": 0.6123456789, "om": 0.3089, "ol": 0.6911,
                                 "h0": 0.6774, "box_size": 62.5, "particle_mass": 1.234567e9}),
    "rbin_empty": (0, 0, 0, 0, {"scale_now": 1.0, "om": 0.3, "ol": 0.7, "h0": 0.7,
                                "box_size": 40.0, "particle_mass": 1e9}),
}


def particles(n, seed):
    rng = np.random.default_rng(seed)
    p = np.zeros(n, L.PARTICLE)
    p["id"] = rng.integers(-(1 << 40), 1 << 40, n)
    p["pos"][:, :3] = rng.uniform(0, 62.5, (n, 3))
    p["pos"][:, 3:] = rng.normal(0, 250.0, (n, 3))
    return p


def main():
    assert refcall.available(), "oracle/_ref not built (run __graft_entry__.build())"
    with tempfile.TemporaryDirectory() as d:
        for name, (n, seed, snap, chunk, cfg) in CASES.items():
            path = os.path.join(d, name + ".rbin")
            p = particles(n, seed)
            refcall.output_particles_internal(path, p, cfg, snap, chunk)
            raw = np.fromfile(path, np.uint8)
            got, cfg_out = refcall.load_internal(path)
            assert got.tobytes() == p.tobytes()
            np.savez_compressed(
                os.path.join(HERE, "internal_%s.npz" % name), raw_file=raw,
                particles=p.view(np.uint8), snap=np.array(snap), chunk=np.array(chunk),
                cfg_in=np.array([cfg[k] for k in refcall.INTERNAL_CFG_FIELDS]),
                cfg_out=np.array([cfg_out[k] for k in refcall.INTERNAL_CFG_FIELDS]))
            print(name, n, len(raw), cfg_out)


if __name__ == "__main__":
    main()
