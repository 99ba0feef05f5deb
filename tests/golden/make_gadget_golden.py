"""Generates the GADGET-2 input fixtures from the reference's own reader.

Run in a checkout where the reference sources are present (oracle/_ref is
built from them by oracle/ref/Makefile, including src/io/io_gadget.c and
src/io/io_util.c):

    python tests/golden/make_gadget_golden.py

For every synthetic file of tests/gadget_files.SPECS it stores, compressed:
the SHA-256 of the file (so a test can check that it rebuilt the same
bytes), the particles as load_particles_gadget2 returns them (file order,
rescaled), the same particles sorted by id as the reference sorts them before
halo finding (std::sort by id, src/mpi_main.cpp:2021-2024; the ids are
distinct, so the order is unique), and the configuration values the reader
sets.
"""
import hashlib
import os
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "tests"))

import gadget_files as GF  # noqa: E402
from oracle import refcall  # noqa: E402

PARTICLE_MASS_IN = 2.5e10  # PARTICLE_MASS before the reader runs


def main():
    assert refcall.available(), "oracle/_ref not built (run __graft_entry__.build())"
    with tempfile.TemporaryDirectory() as d:
        for name in GF.SPECS:
            path = os.path.join(d, name + ".g2")
            GF.write(path, name)
            digest = hashlib.sha256(open(path, "rb").read()).hexdigest()
            parts, cfg = refcall.load_gadget2(path, particle_mass=PARTICLE_MASS_IN,
                                              **GF.reader_kwargs(name))
            order = np.argsort(parts["id"], kind="stable")
            assert len(np.unique(parts["id"])) == len(parts)
            np.savez_compressed(os.path.join(HERE, "gadget_%s.npz" % name),
                                sha256=np.array(digest), particles=parts.view(np.uint8),
                                sorted=parts[order].view(np.uint8),
                                cfg=np.array([cfg[k] for k in refcall.GADGET_CFG_FIELDS]),
                                particle_mass_in=np.array(PARTICLE_MASS_IN))
            print(name, len(parts), cfg)


if __name__ == "__main__":
    main()
