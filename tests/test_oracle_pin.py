"""Pins the C restatement (oracle/rockstar_oracle.c) to the reference's own
sources compiled as-is (oracle/_ref): identical bytes for FOF, particle
permutations, halos and links.  Skipped where the reference checkout (and
so oracle/_ref) is absent."""
import os

import numpy as np
import pytest

from conftest import ROOT

REF_LIB = os.path.join(ROOT, "oracle", "_ref", "libref_rockstar.so")
pytestmark = pytest.mark.skipif(not os.path.exists(REF_LIB), reason="reference oracle not built")


def _cfg(rk, p, box, mp):
    return rk.Config(particle_mass=mp, box_size=box, total_particles=len(p))


@pytest.mark.parametrize("cfg,scale", [(1, 0.05), (1, 0.25), (2, 1 / 32), (3, 0.001),
                                       (4, 1 / 4096), (5, 0.002)])
def test_restatement_equals_reference(rk, oracle, cfg, scale):
    from oracle import refcall
    p, box, mp, _ = rk.synth(cfg, scale)
    c = _cfg(rk, p, box, mp)
    assert refcall.setup(c) == oracle.setup(c)
    assert np.array_equal(refcall.thresholds(), oracle.thresholds())
    a = refcall.fof(p)
    b = oracle.fof(p)
    for x, y in zip(a, b):
        assert np.array_equal(x, y)
    ra = refcall.find_subs(*a)
    rb = oracle.find_subs(*b)
    assert np.array_equal(ra[0], rb[0])
    assert ra[1].tobytes() == rb[1].tobytes()
    for f in ("child", "next_cochild", "prev_cochild", "sub_of", "ph", "max_metric"):
        assert np.array_equal(ra[2][f], rb[2][f])


def test_restatement_duplicates(rk, oracle):
    from oracle import refcall
    p, box, mp, _ = rk.synth(1, 0.05)
    p = p.copy()
    p["pos"][10] = p["pos"][11]
    p["id"][500] = p["id"][501]
    c = _cfg(rk, p, box, mp)
    refcall.setup(c)
    oracle.setup(c)
    for x, y in zip(refcall.fof(p), oracle.fof(p)):
        assert np.array_equal(x, y)


def test_potential_equals_reference(rk, oracle):
    """compute_potential (Barnes-Hut) on a random particle set."""
    from oracle import refcall
    rng = np.random.default_rng(5)
    po = np.zeros(3000, rk.POTENTIAL)
    po["pos"][:, :3] = rng.normal(size=(3000, 3)).astype(np.float32) * 0.3
    c = rk.Config()
    refcall.setup(c)
    oracle.setup(c)
    a = refcall.compute_potential(po)
    b = oracle.compute_potential(po)
    assert np.array_equal(a["pe"], b["pe"])
