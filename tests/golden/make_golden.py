"""Generates the golden fixtures from the reference's own hot-path sources.

Run in a checkout where the reference sources are present (it builds
oracle/_ref/libref_rockstar.so from them with oracle/ref/Makefile):

    python tests/golden/make_golden.py

For each case it stores, compressed: the hash of the generated input (so a
test can verify its regenerated input is the same), the reference's 3D FOF
partition (smallest member id per particle, -1 outside groups), and for
find_subs run on the reference's own FOF groups: every halo record, its
extra_halo_info links, and the halo of every particle (-1 for none).
"""
import hashlib
import importlib.util
import os
import subprocess
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

CASES = [("c1_q", 1, 0.25), ("c2_s", 2, 1 / 32), ("c1_tiny", 1, 0.02),
         ("c3_t", 3, 0.001), ("c5_t", 5, 0.002)]
SEED = 20261203


def load_pkg():
    d = os.path.join(ROOT, "mpi-rockstar_gb300")
    spec = importlib.util.spec_from_file_location(
        "mpi_rockstar_gb300", os.path.join(d, "__init__.py"), submodule_search_locations=[d])
    m = importlib.util.module_from_spec(spec)
    sys.modules["mpi_rockstar_gb300"] = m
    spec.loader.exec_module(m)
    return m


def input_hash(p):
    return hashlib.sha256(p.tobytes()).hexdigest()


def halo_of_particle(parts, H, n):
    lab = np.full(n, -1, np.int32)
    for i, h in enumerate(H):
        if h["num_p"] > 0:
            lab[parts["id"][h["p_start"]:h["p_start"] + h["num_p"]]] = i
    return lab


def canon(parts, off, sz, n):
    lab = np.full(n, -1, np.int64)
    for o, s in zip(off, sz):
        g = parts["id"][o:o + s]
        lab[g] = g.min()
    return lab


def main(names=None):
    """Writes every case, or only those named on the command line."""
    rk = load_pkg()
    rk.build()
    subprocess.check_call(["make", "-s", "-C", os.path.join(ROOT, "oracle", "ref")])
    from oracle import refcall
    for name, cfg, scale in CASES:
        if names and name not in names:
            continue
        p, box, mp, _ = rk.synth(cfg, scale, SEED)
        c = rk.Config(particle_mass=mp, box_size=box, total_particles=len(p))
        refcall.setup(c)
        fp, off, sz = refcall.fof(p)
        parts, H, E = refcall.find_subs(fp, off, sz)
        np.savez_compressed(
            os.path.join(HERE, name + ".npz"),
            cfg=cfg, scale=scale, seed=SEED, n=len(p), input_sha=input_hash(p),
            box=box, mp=mp,
            fof_label=canon(fp, off, sz, len(p)).astype(np.int32),
            fof_order=fp["id"].astype(np.int32), fof_off=off, fof_sz=sz,
            halos=H.view(np.uint8).reshape(len(H), -1), extra=E.view(np.uint8).reshape(len(E), -1),
            halo_of=halo_of_particle(parts, H, len(p)))
        print(name, len(p), "groups", len(off), "halos", len(H))


if __name__ == "__main__":
    main(sys.argv[1:])
