"""The C ABI library loads and exports every function declared in
include/*.h (no GPU calls)."""
import ctypes
import glob
import os
import re

import numpy as np
import pytest

from conftest import ROOT


def declared_functions():
    names = set()
    for h in glob.glob(os.path.join(ROOT, "include", "*.h")):
        src = re.sub(r"/\*.*?\*/", "", open(h).read(), flags=re.S)
        for m in re.finditer(r"^\s*(?:const\s+)?[\w ]+?[\s\*]+(rsg_\w+)\s*\(", src, re.M):
            names.add(m.group(1))
    return names


def test_exports_every_declared_symbol(rk):
    lib = ctypes.CDLL(rk.LIB)
    names = declared_functions()
    assert {"rsg_rockstar_fof", "rsg_find_subs", "rsg_find_subs_batch",
            "rsg_path_device", "rsg_config_setup"} <= names
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing


def test_config_setup_matches_oracle(rk, oracle):
    """AVG_PARTICLE_SPACING and the density thresholds, host side."""
    import numpy as np
    c = rk.Config(particle_mass=2.03e10, box_size=80.0, total_particles=2097152)
    st = rk.setup_config(c)
    sp = oracle.setup(c)
    th = oracle.thresholds()
    assert st.avg_particle_spacing == sp
    assert np.array_equal(np.array(list(st.particle_thresh_dens)), th[:5])
    assert (st.particle_rvir_dens, st.particle_rvir_dens_z0, st.dynamical_time) == tuple(th[5:8])


def test_errors_without_gpu(rk):
    """Without a GPU every compute entry fails with a code, never silently."""
    import numpy as np
    import torch
    if torch.cuda.is_available():
        return
    p = np.zeros(10, rk.PARTICLE)
    try:
        rk.rockstar_fof(p, rk.Config())
    except rk.RockstarError as e:
        assert e.code in (-2, -3)
    else:
        raise AssertionError("expected an error without a GPU")


def test_isolated_groups_workload(rk):
    """The precision study's snapshot: one group per lattice cell, every
    particle at least 0.5 Mpc/h inside its cell, so no two groups can link."""
    p, box, mp, ng = rk.synth(3, 0.002)
    assert ng == 400 and mp == 1e9
    side = int(np.ceil(ng ** (1 / 3) - 1e-9))
    cell = box / side
    x = p["pos"][:, :3].astype(np.float64)
    f = x - np.floor(x / cell) * cell
    assert f.min() >= 0.5 - 1e-4 and f.max() <= cell - 0.5 + 1e-4
    # every occupied cell is one of the first ng cells in x-fastest order
    c = np.floor(x / cell).astype(np.int64)
    idx = c[:, 0] + side * (c[:, 1] + side * c[:, 2])
    assert idx.max() < ng and len(np.unique(idx)) == ng


def test_tuning_parameters(rk):
    """rsg_set_tuning / rsg_get_tuning: names, ranges, errors (host only)."""
    old = rk.get_tuning()
    assert set(old) == set(rk.TUNING_NAMES)
    try:
        rk.set_tuning("seg_max", 4096)
        assert rk.get_tuning("seg_max") == 4096
        with pytest.raises(rk.RockstarError) as e:
            rk.set_tuning("seg_max", 10)
        assert e.value.code == -1
        with pytest.raises(rk.RockstarError):
            rk.set_tuning("no_such_parameter", 1)
        with pytest.raises(rk.RockstarError):
            rk.set_tuning("bh_huge", 100)  # must stay above the warp kernels' node size
    finally:
        for k, v in old.items():
            rk.set_tuning(k, v)


def test_bench_parses_profile_table():
    """bench.py reads rsg_profile_table's lines (name, launches, total ms,
    gap ms) to pick the kernel whose roofline it reports."""
    import bench
    rows = bench.parse_table("_ZN3rsg4k_nnEPKv\t10\t12.5\t0.02\n_ZN3rsg6k_kahnEv\t3\t1.0\t0.5\n")
    assert rows == [("k_nn", 10, 12.5), ("k_kahn", 3, 1.0)]
