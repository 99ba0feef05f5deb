"""3D FOF on the GPU against the C restatement of the reference (which is
itself pinned bit-exact to the reference sources): kd-tree permutations
element for element, and rockstar()'s whole output -- the permuted particle
array (its union-find labels decide the order through the partition sort)
and the group offsets and sizes -- byte for byte."""
import numpy as np
import pytest

from helpers import canon_partition

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("dim,leaf", [(3, 20), (6, 40), (3, 10)])
@pytest.mark.parametrize("cfg,scale", [(1, 0.05), (2, 1 / 64)])
def test_tree_permutation(rk, oracle, dim, leaf, cfg, scale):
    p, box, mp, _ = rk.synth(cfg, scale)
    a = rk.tree_order(p, dim, leaf)
    b = oracle.tree_order(p, dim, leaf)
    assert np.array_equal(a["id"], b["id"])


def test_tree_degenerate(rk, oracle):
    """Coincident coordinates and repeated values on split dimensions."""
    rng = np.random.default_rng(3)
    p = np.zeros(5000, rk.PARTICLE)
    p["id"] = np.arange(5000)
    p["pos"] = rng.integers(0, 4, size=(5000, 6)).astype(np.float32)
    p["pos"][:700] = 1.0
    for dim, leaf in [(3, 20), (6, 40)]:
        assert np.array_equal(rk.tree_order(p, dim, leaf)["id"],
                              oracle.tree_order(p, dim, leaf)["id"])


@pytest.mark.parametrize("cfg,scale", [(1, 0.25), (1, 1.0), (2, 1 / 16), (3, 0.005),
                                       (4, 1 / 2048), (5, 0.004)])
def test_fof_partition(rk, oracle, cfg, scale):
    p, box, mp, _ = rk.synth(cfg, scale)
    c = rk.Config(particle_mass=mp, box_size=box, total_particles=len(p))
    oracle.setup(c)
    ro = oracle.fof(p)
    rg = rk.rockstar_fof(p, c)
    assert len(rg[0]) == len(ro[0])
    assert len(rg[1]) == len(ro[1])
    assert np.array_equal(canon_partition(*rg), canon_partition(*ro))
    # the reference's permutation and group table, byte for byte
    assert rg[0].tobytes() == ro[0].tobytes()
    assert np.array_equal(rg[1], ro[1]) and np.array_equal(rg[2], ro[2])


def test_fof_duplicates(rk, oracle):
    """Duplicate positions / ids are removed as src/rockstar.c:379-396 does."""
    p, box, mp, _ = rk.synth(1, 0.05)
    p = p.copy()
    p["pos"][10] = p["pos"][11]
    p["pos"][200] = p["pos"][3000]
    p["id"][500] = p["id"][501]
    c = rk.Config(particle_mass=mp, box_size=box, total_particles=len(p))
    oracle.setup(c)
    ro = oracle.fof(p)
    rg = rk.rockstar_fof(p, c)
    assert len(rg[0]) == len(ro[0]) < len(p)
    assert rg[0].tobytes() == ro[0].tobytes()
    assert np.array_equal(rg[1], ro[1]) and np.array_equal(rg[2], ro[2])


def test_fof_empty_and_tiny(rk, oracle):
    c = rk.Config()
    oracle.setup(c)
    for n in (0, 1, 2, 15):
        p = np.zeros(n, rk.PARTICLE)
        p["id"] = np.arange(n)
        p["pos"][:, :3] = np.linspace(0, 0.01, n)[:, None]
        out, off, sz = rk.rockstar_fof(p, c)
        assert len(out) == n
        assert (len(off) == 1) == (n >= 10)
        ro = oracle.fof(p)
        assert out.tobytes() == ro[0].tobytes() and np.array_equal(off, ro[1])


@pytest.mark.parametrize("n_groups", [1, 40])
def test_fof_small_groups_interleaved(rk, oracle, n_groups):
    """Clumps of 2 to 30 particles: groups below MIN_HALO_PARTICLES stay in
    the permuted array between the kept ones, as the partition sort leaves
    them, and only the kept ones are listed."""
    rng = np.random.default_rng(11 + n_groups)
    sizes = rng.integers(2, 31, size=n_groups)
    centres = rng.uniform(1, 39, size=(n_groups, 3))
    pos = np.concatenate([cen + rng.normal(0, 0.004, size=(k, 3)) for cen, k in zip(centres, sizes)]
                         + [rng.uniform(0, 40, size=(3000, 3))])
    p = np.zeros(len(pos), rk.PARTICLE)
    p["id"] = np.arange(len(pos))
    p["pos"][:, :3] = pos.astype(np.float32)
    p["pos"][:, 3:] = rng.normal(0, 100, size=(len(pos), 3)).astype(np.float32)
    c = rk.Config(particle_mass=1e9, box_size=40.0, total_particles=len(p))
    oracle.setup(c)
    ro = oracle.fof(p)
    rg = rk.rockstar_fof(p, c)
    assert rg[0].tobytes() == ro[0].tobytes()
    assert np.array_equal(rg[1], ro[1]) and np.array_equal(rg[2], ro[2])
    assert (rg[2] >= c.min_halo_particles).all()


@pytest.mark.parametrize("cfg_id,scale,parts", [(2, 0.25, 4), (3, 0.01, 7)])
def test_fof_chunked_later_lists(rk, cfg_id, scale, parts, monkeypatch):
    """A later-dense list larger than its buffer is built and walked in
    chunks of particles; the groups must be the same bytes as with the whole
    list (RSG_FOF_LIST_ENTRIES caps the buffer)."""
    p, box, mp, _ = rk.synth(cfg_id, scale)
    cfg = rk.Config(particle_mass=mp, box_size=box, total_particles=len(p))
    whole = rk.rockstar_fof(p, cfg)
    ne = rk.last_stats()["dense_pairs"]
    assert ne > 4 * (1 << 17)
    monkeypatch.setenv("RSG_FOF_LIST_ENTRIES", str(ne // parts))
    chunked = rk.rockstar_fof(p, cfg)
    assert rk.last_stats()["dense_pairs"] == ne
    for a, b in zip(whole, chunked):
        assert a.tobytes() == b.tobytes()
    monkeypatch.setenv("RSG_FOF_LIST_ENTRIES", "1000")
    with pytest.raises(rk.RockstarError) as e:
        rk.rockstar_fof(p, cfg)
    assert e.value.code == -4


@pytest.mark.parametrize("cfg_id,scale", [(2, 0.25), (3, 0.01)])
def test_fof_seed_loop_forms(rk, cfg_id, scale):
    """The seed frontiers run as a device-side graph loop; with per-launch
    timing selected the same steps run host-driven.  Both give the same
    groups, byte for byte, in the same number of steps."""
    p, box, mp, _ = rk.synth(cfg_id, scale)
    cfg = rk.Config(particle_mass=mp, box_size=box, total_particles=len(p))
    graph = rk.rockstar_fof(p, cfg)
    st = rk.last_stats()
    assert st["dense"] > 1000 and st["dense_pairs"] > st["dense"] and st["seed_steps"] > 2
    rk.profile_select("6k_kahnE")  # the step kernel alone (mangled name)
    try:
        host = rk.rockstar_fof(p, cfg)
        launches, ms = rk.profile_read()
    finally:
        rk.profile_select("")
    assert rk.last_stats()["seed_steps"] == st["seed_steps"] == launches
    assert rk.last_stats()["dense_pairs"] == st["dense_pairs"]
    for a, b in zip(graph, host):
        assert a.tobytes() == b.tobytes()
