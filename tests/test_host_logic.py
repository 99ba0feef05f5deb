"""Host-side logic without a GPU: the autotuner's search and the precision
study's comparison."""
import numpy as np


class FakeTuning:
    """Stands in for the library's tuning calls; the step time is a known
    function of the parameters."""

    def __init__(self, names):
        self.v = {k: 1 for k in names}

    def get_tuning(self, name=None):
        return dict(self.v) if name is None else self.v[name]

    def set_tuning(self, name, value):
        self.v[name] = value


def test_autotune_coordinate_descent(rk):
    from mpi_rockstar_gb300 import autotune
    fake = FakeTuning(autotune.CANDIDATES)
    for k, c in autotune.CANDIDATES.items():
        fake.v[k] = c[2]  # the defaults sit in the middle of each candidate list
    best_of = {"bh_chunk": 4096, "seg_max": 65536}

    def step_ms():
        ms = 100.0
        for k, v in best_of.items():
            ms += 0.0 if fake.v[k] == v else 5.0  # 5% per wrong parameter
        return ms

    res = autotune.autotune(fake, None, None, step_ms=step_ms)
    assert res["default_ms"] == 110.0 and res["best_ms"] == 100.0
    for k, c in autotune.CANDIDATES.items():
        assert res["best"][k] == best_of.get(k, c[2]), k
    assert fake.get_tuning() == res["best"]  # left set


def test_autotune_ignores_noise(rk):
    """Gains below min_gain keep the current value."""
    from mpi_rockstar_gb300 import autotune
    fake = FakeTuning(autotune.CANDIDATES)
    for k, c in autotune.CANDIDATES.items():
        fake.v[k] = c[2]
    start = dict(fake.v)
    res = autotune.autotune(fake, None, None, min_gain=0.01,
                            step_ms=lambda: 100.0 - 0.5 * (fake.v["bp_big"] != start["bp_big"]))
    assert res["best"] == start


def _runs(rk):
    """Two forms over the same 3 halos / 4 records: form 0 moves one
    potential by 1% and flips one bound flag and one halo's status."""
    h = np.zeros(3, rk.HALO)
    h["m"] = [10.0, 20.0, 30.0]
    h["mgrav"] = [8.0, 18.0, 30.0]
    h["r"] = [1.0, 2.0, 3.0]
    h["vmax"] = [5.0, 6.0, 7.0]
    q = np.zeros(4, rk.POTENTIAL)
    q["pos"][:, 0] = [1, 2, 3, 4]
    q["pe"] = [1.0, 2.0, 3.0, 4.0]
    q["ke"] = [0.5, 2.01, 1.0, -1.0]  # the last is potential-only
    h0, q0 = h.copy(), q.copy()
    q0["pe"][1] = 2.02                 # now pe >= ke: bound
    h0["mgrav"][0] = 4.0               # 4 <= 0.5 * 10: dropped from the output
    return {3: {"halos": h, "records": q, "kernel_ms": 1.0, "wall_s": 0.1},
            0: {"halos": h0, "records": q0, "kernel_ms": 0.5, "wall_s": 0.1},
            "groups": 1, "particles": 4}


def test_precision_compare(rk):
    from mpi_rockstar_gb300 import precision
    cfg = rk.Config(particle_mass=1.0, unbound_threshold=0.5)
    res = precision.compare(_runs(rk), cfg, ref=3, forms=(0,))
    e = res["forms"]["0"]
    assert np.isclose(e["potential_rel"]["max"], 0.01)
    assert e["bound_flag_flips"] == 1          # only records with ke >= 0 count
    assert e["output_status_flips"] == 1
    assert np.isclose(e["mvir_rel"]["max"], 0.5)
    assert e["vmax_rel"]["max"] == 0.0
    assert res["halos"] == 3 and res["records"] == 4
