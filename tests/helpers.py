"""Shared helpers for the parity tests (no GPU needed to import)."""
import numpy as np


def canon_partition(parts, off, sz):
    """Group membership as a canonical label per particle id: the smallest id
    in the particle's group, or -1 for particles in no group."""
    ids = parts["id"]
    lab = np.full(int(ids.max()) + 1 if len(ids) else 0, -1, np.int64)
    for o, s in zip(off, sz):
        g = ids[o:o + s]
        lab[g] = g.min()
    return lab


def config_for(mod, box, mp, n):
    return mod.Config(particle_mass=mp, box_size=box, total_particles=n)
