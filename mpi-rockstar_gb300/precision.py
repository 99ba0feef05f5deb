"""Potential and unbinding precision study on the isolated-groups workload.

The batched path runs over one snapshot once per potential form
(rsg_set_potential_form):

  0  Barnes-Hut with the reference's FP64 arithmetic (src/potential.c:133-192)
  1  Barnes-Hut with FP32 terms and Kahan-compensated FP32 sums (batched default)
  2  Barnes-Hut with FP32 terms and plain FP32 sums
  3  FP64 direct sum over all pairs (the precision reference)

Everything before the potentials (3D FOF, 6D hierarchy, assignment, the
potential sets) is independent of the form, so the halos and the potential
records of the runs correspond one to one.  Each form is compared with
form 3 on:

  potentials    per record |pe_f - pe_3| / pe_3
  bound flags   records of a halo's own particles whose bound state
                (pe >= ke, src/properties.c unbinding) differs
  halos         bound fraction mgrav / m, Mvir (mgrav, the bound mass that
                BOUND_PROPS reports), Rvir (r), Vmax (vmax), and the halos whose
                output status flips (m * UNBOUND_THRESHOLD >= mgrav drops a
                halo, src/io/meta_io.c:276-286)

and forms 1 and 2 also with form 0, which shares their tree and opening
rule, so that difference is the FP32 arithmetic alone.
"""
import time

import numpy as np


def _rel(a, b):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    d = np.abs(a - b)
    s = np.abs(b)
    out = np.zeros_like(d)
    nz = s > 0
    out[nz] = d[nz] / s[nz]
    out[~nz & (d > 0)] = np.inf
    return out


def _stats(x):
    x = np.asarray(x, np.float64)
    if x.size == 0:
        return {"n": 0}
    return {"n": int(x.size), "median": float(np.median(x)),
            "p99": float(np.quantile(x, 0.99)), "max": float(x.max())}


def run_forms(rk, parts, cfg, forms=(3, 0, 1, 2)):
    """The batched path over `parts` once per form.  Returns {form: dict with
    halos, records (potential records, last_potentials order) and the device
    time of the potential kernels}."""
    p, off, sz = rk.rockstar_fof(parts, cfg)
    out = {}
    prev = rk.set_potential_form(1)
    rk.keep_potentials(True)
    try:
        for f in forms:
            rk.set_potential_form(f)
            rk.profile_select("k_bh_walk" if f != 3 else "k_direct64")
            t0 = time.perf_counter()
            _, h, _ = rk.find_subs(p, off, sz, cfg, batched=True)
            wall = time.perf_counter() - t0
            launches, ms = rk.profile_read()
            out[f] = {"halos": h, "records": rk.last_potentials(), "kernel_ms": ms,
                      "launches": launches, "wall_s": wall}
    finally:
        rk.profile_select("")
        rk.keep_potentials(False)
        rk.set_potential_form(prev)
    out["groups"] = len(off)
    out["particles"] = int(sz.sum())
    return out


def compare(runs, cfg, ref=3, forms=(0, 1, 2)):
    """Error statistics of each form against `ref` (see the module text)."""
    R = runs[ref]
    hr, pr = R["halos"], R["records"]
    own = pr["ke"] >= 0
    bound_r = pr["pe"] >= pr["ke"]
    res = {"groups": runs["groups"], "particles": runs["particles"], "halos": len(hr),
           "records": len(pr), "reference_form": ref, "forms": {}}
    ut = cfg.unbound_threshold
    mp = cfg.particle_mass

    def status(h):
        return ~((h["m"] * ut >= h["mgrav"]) | ((h["mgrav"] < 1.5 * mp) & (ut > 0)))

    keep_r = status(hr)
    for f in forms:
        F = runs[f]
        h, q = F["halos"], F["records"]
        if len(h) != len(hr) or len(q) != len(pr):
            raise RuntimeError("form %d: %d halos / %d records, reference %d / %d"
                               % (f, len(h), len(q), len(hr), len(pr)))
        if not np.array_equal(q["pos"], pr["pos"]):
            raise RuntimeError("form %d: potential records in a different order" % f)
        pe = _rel(q["pe"], pr["pe"])
        flips = (q["pe"] >= q["ke"]) != bound_r
        ok = hr["m"] > 0
        bf_f = np.where(ok, h["mgrav"] / np.where(ok, h["m"], 1), 0)
        bf_r = np.where(ok, hr["mgrav"] / np.where(ok, hr["m"], 1), 0)
        e = {"potential_rel": _stats(pe),
             "bound_flag_flips": int(flips[own].sum()),
             "bound_flag_flip_frac": float(flips[own].mean()) if own.any() else 0.0,
             "bound_fraction_abs": _stats(np.abs(bf_f - bf_r)[ok]),
             "mvir_rel": _stats(_rel(h["mgrav"], hr["mgrav"])[ok]),
             "rvir_rel": _stats(_rel(h["r"], hr["r"])[ok]),
             "vmax_rel": _stats(_rel(h["vmax"], hr["vmax"])[ok]),
             "output_status_flips": int((status(h) != keep_r).sum()),
             "kernel_ms": F["kernel_ms"], "wall_s": F["wall_s"]}
        if f in (1, 2) and 0 in runs and ref != 0:
            h0, q0 = runs[0]["halos"], runs[0]["records"]
            e["vs_form0"] = {
                "potential_rel": _stats(_rel(q["pe"], q0["pe"])),
                "bound_flag_flips": int(((q["pe"] >= q["ke"]) != (q0["pe"] >= q0["ke"]))[own].sum()),
                "mvir_rel": _stats(_rel(h["mgrav"], h0["mgrav"])[ok]),
                "rvir_rel": _stats(_rel(h["r"], h0["r"])[ok]),
                "vmax_rel": _stats(_rel(h["vmax"], h0["vmax"])[ok]),
                "output_status_flips": int((status(h) != status(h0)).sum())}
        res["forms"][str(f)] = e
    res["reference_kernel_ms"] = R["kernel_ms"]
    bf = np.where(hr["m"] > 0, hr["mgrav"] / np.where(hr["m"] > 0, hr["m"], 1), 0)
    res["reference_bound_fraction_median"] = float(np.median(bf)) if len(bf) else 0.0
    res["reference_unbound_records_frac"] = float((~bound_r[own]).mean()) if own.any() else 0.0
    return res
