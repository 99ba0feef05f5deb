"""Potential forms 2 (FP32 plain sums) and 3 (FP64 direct sum), and the
precision study on the isolated-groups workload (mpi-rockstar_gb300/precision.py).

Tolerances:
  form 3 against a numpy FP64 direct sum: 1e-12 relative (both FP64; only the
    summation order differs);
  form 1 against form 0 (same tree, FP32 Kahan arithmetic): 1e-5 relative,
    the batched precision form's stated bound;
  form 2 against form 0: 1e-4 relative (uncompensated FP32 sums);
  Barnes-Hut (forms 0-2) against the direct sum: median below 1e-2, the
    opening-angle error of the reference's walk."""
import numpy as np
import pytest

from test_gpu_potential import direct_fp64, nfw_like

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("n,seed,dup", [(3000, 11, 0), (4000, 12, 30)])
def test_direct_form_equals_fp64_sum(rk, n, seed, dup):
    po = nfw_like(n, seed, dup=dup).view(rk.POTENTIAL)
    cfg = rk.Config(particle_mass=1e9, force_res=0.003)
    a = rk.compute_potential(po, cfg, form=0)
    d = rk.compute_potential(po, cfg, form=3)
    assert np.array_equal(a["pos"], d["pos"])          # same permutation
    ref = direct_fp64(d, cfg.particle_mass, cfg.force_res)
    rel = np.abs(d["pe"] - ref) / ref
    assert rel.max() <= 1e-12, rel.max()


def test_plain_fp32_form(rk):
    po = nfw_like(30000, 13).view(rk.POTENTIAL)
    cfg = rk.Config(particle_mass=1e9, force_res=0.003)
    a = rk.compute_potential(po, cfg, form=0)
    k = rk.compute_potential(po, cfg, form=1)
    p = rk.compute_potential(po, cfg, form=2)
    assert np.array_equal(a["pos"], p["pos"])
    ek = np.abs(k["pe"] - a["pe"]) / a["pe"]
    ep = np.abs(p["pe"] - a["pe"]) / a["pe"]
    assert ek.max() <= 1e-5 and ep.max() <= 1e-4, (ek.max(), ep.max())
    # compensation is what the batched form pays for: it must not be worse
    assert np.median(ek) <= np.median(ep)


def test_potential_form_setter(rk):
    prev = rk.set_potential_form(2)
    try:
        assert rk.set_potential_form(3) == 2
        with pytest.raises(rk.RockstarError):
            rk.set_potential_form(4)
    finally:
        rk.set_potential_form(prev)


def test_precision_study_isolated_groups(rk):
    from mpi_rockstar_gb300 import precision
    p, box, mp, ng = rk.synth(3, 0.005)
    cfg = rk.Config(particle_mass=mp, box_size=box, total_particles=len(p))
    runs = precision.run_forms(rk, p, cfg)
    res = precision.compare(runs, cfg)
    print(res)
    assert res["halos"] >= ng // 2
    h3 = runs[3]["halos"]
    for f in (0, 1, 2):
        h = runs[f]["halos"]
        # everything before the potentials is form-independent
        for k in ("num_p", "m", "pos", "p_start"):
            assert np.array_equal(h[k], h3[k]), (f, k)
        e = res["forms"][str(f)]
        assert e["potential_rel"]["median"] < 1e-2
    v1, v2 = res["forms"]["1"]["vs_form0"], res["forms"]["2"]["vs_form0"]
    assert v1["potential_rel"]["max"] <= 1e-5
    assert v2["potential_rel"]["max"] <= 1e-4
    # FP32 arithmetic moves no halo across the output threshold
    assert v1["output_status_flips"] == 0
    # a tenth of every group moves above its escape speed
    assert res["reference_unbound_records_frac"] >= 0.05
