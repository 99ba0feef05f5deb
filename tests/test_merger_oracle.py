"""The merger tree's descendant rule (src/merger.c:45-101), restated in the
oracle as a sort-based join, against the reference's own merger.c compiled
into oracle/_ref.  Test infrastructure for the temporal row: the device
path is not built."""
import os

import numpy as np
import pytest

from conftest import ROOT

REF_LIB = os.path.join(ROOT, "oracle", "_ref", "libref_rockstar.so")


def catalogue(rng, nh, pool, mean_np, start_id, overlap=False):
    """nh halos with consecutive ids from start_id, each listing a random
    draw of particle ids from pool (with repeats across halos)."""
    from oracle import layouts as L
    h = np.zeros(nh, L.HALO)
    sizes = rng.poisson(mean_np, nh)
    sizes[rng.random(nh) < 0.1] = 0
    h["id"] = start_id + np.arange(nh)
    h["num_p"] = sizes
    h["p_start"] = np.concatenate([[0], np.cumsum(sizes)[:-1]])
    ids = rng.choice(pool, int(sizes.sum()))
    if overlap and nh > 3:  # two halos listing the same range
        h["p_start"][3] = h["p_start"][1]
        h["num_p"][3] = h["num_p"][1]
    return h, ids.astype(np.int64)


@pytest.mark.skipif(not os.path.exists(REF_LIB), reason="reference oracle not built")
@pytest.mark.parametrize("seed", [1, 2, 3])
def test_descendants_equal_reference(seed):
    from oracle import refcall, restatement
    rng = np.random.default_rng(seed)
    pool = rng.choice(np.arange(-5000, 200000), 6000, replace=False)
    h1, p1 = catalogue(rng, 400, pool, 30, 0)
    h2, p2 = catalogue(rng, 300, pool, 40, 10_000, overlap=True)
    got = restatement.descendants(h1, p1, h2, p2)
    want = refcall.descendants(h1, p1, h2, p2)
    assert np.array_equal(got, want)
    assert (got > -1).any() and (got == -1).any()


def test_descendant_rule_cases():
    """Ties go to the smaller id; a later listing of a particle replaces an
    earlier one; halos without matches keep -1."""
    from oracle import layouts as L
    from oracle import restatement
    h2 = np.zeros(3, L.HALO)
    h2["id"] = [7, 3, 9]
    h2["num_p"] = [2, 2, 1]
    h2["p_start"] = [0, 2, 4]
    p2 = np.array([100, 101, 102, 103, 101], np.int64)  # 101: halo 7, then halo 9
    h1 = np.zeros(3, L.HALO)
    h1["num_p"] = [4, 1, 2]
    h1["p_start"] = [0, 4, 5]
    p1 = np.array([100, 102, 103, 101, 555, 100, 102], np.int64)
    got = restatement.descendants(h1, p1, h2, p2)
    # halo 0: 100 -> 7, 102 -> 3, 103 -> 3, 101 -> 9: id 3 twice
    # halo 1: no match; halo 2: 7 once, 3 once: the smaller, 3
    assert got.tolist() == [3, -1, 3]
    if os.path.exists(REF_LIB):
        from oracle import refcall
        assert refcall.descendants(h1, p1, h2, p2).tolist() == [3, -1, 3]
