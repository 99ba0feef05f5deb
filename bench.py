"""Benchmark of the halo-finding hot path: 3D FOF -> 6D phase-space FOF
hierarchy -> particle assignment -> potentials / unbinding -> properties.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference]

One step is the whole path over one synthetic snapshot.  The default
workload is the 512^3 snapshot (134,217,728 particles, 500 Mpc/h, 200,000
NFW hosts with subhalos, 45% background; csrc/synth.c workload 4), the
configuration the metric is quoted on.  Under torchrun every rank processes
its own snapshot (seed + rank): replicas, no exchange, so scaling is weak.

value   : particles/s of the batched form with the particles already in HBM
          (rsg_path_device), timed per step with CUDA events; L2 is flushed
          between steps.  The plain drop-in is timed beside it.
e2e     : the same metric through the C ABI with host buffers
          (rsg_rockstar_fof + rsg_find_subs_batch on a pinned array), copies
          included.
parity  : on a bounded sample of the workload, the plain form against the
          oracle (bit for bit) and the batched form's membership; on the full
          workload the batched form against the plain one (config.tolerance).
roofline: the dominant kernel (by device time in the launch list), timed
          with CUDA events on its stream during the timed steps.
cpu_baseline: the C restatement of the reference (oracle/) on one host core
          over the same bounded sample.
"""
import argparse
import json
import math
import os
import struct
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)
METRIC = "particles/s through FOF+6D+unbind+props, batched vs plain on GB300 @ stated tol"
SEED = 20261203
# bounded samples of each workload (same density and structure, smaller box):
# the CPU baseline and the oracle parity check run on SAMPLE_SCALE, the
# reference arm times REF_SCALE per step
SAMPLE_SCALE = {1: 0.25, 2: 0.125, 3: 0.005, 4: 1 / 64, 5: 0.02}
REF_SCALE = {1: 1.0, 2: 1.0, 3: 0.05, 4: 1 / 32, 5: 0.1}
# Algorithmic (compulsory) bytes of ONE launch of a kernel, from the work
# counters the library reports for the step (rsg_last_stats): every input
# record read once, every output written once; node data held in L2 is not
# counted.  Kernels without an entry get no roofline figure.
ALGO_BYTES = {
    # 6D FOF: each level's particles read once (24 B of the 32 B record), one
    # union-find parent written (4 B)
    "k_fof6_w": lambda st, L: 28.0 * st["items_6d"] / max(L, 1),
    # assignment: position read, label read and written
    "k_asc_assign_p": lambda st, L: 32.0 * st["items_6d"] / max(L, 1),
    # basic halo properties: two passes over the halo's positions
    "k_basic_props": lambda st, L: 48.0 * st["items_6d"] / max(L, 1),
    # norm_sd: positions read and written back
    "k_norm_par": lambda st, L: 48.0 * st["items_6d"] / max(L, 1),
    "k_norm_warp": lambda st, L: 48.0 * st["items_6d"] / max(L, 1),
    # next-closest search: sample position read, distance written
    "k_nn": lambda st, L: 28.0 * st["samples_6d"] / max(L, 1),
    # median selection: every sample distance read once
    "k_target_par": lambda st, L: 4.0 * st["samples_6d"] / max(L, 1),
    # later-dense lists: positions of the dense particles in both launches,
    # every entry (one per dense pair) written once
    "k_llist_w": lambda st, L: (32.0 * st["dense"] + 4.0 * st["dense_pairs"]) / max(L, 1),
    # seed frontiers: every list entry read, its pending count updated
    "k_kahn": lambda st, L: 12.0 * st["dense_pairs"] / max(L, 1),
    # potentials: record read (48 B), potential written (8 B)
    "k_bh_walk": lambda st, L: 56.0 * st["pot_records"] / max(L, 1),
    # property scans: record read, kinetic energy written
    "k_halo_scans_blk": lambda st, L: 52.0 * st["kept_big"],
    "k_halo_scans_list": lambda st, L: 52.0 * st["kept_small"],
}


# DRAM bytes per work unit from one ncu capture (dram__bytes_read.sum +
# dram__bytes_write.sum of the captured launch over the units it processed),
# scaled to the timed launches by their units
NCU_TRAFFIC = {
    "k_fof6_w": ((137.976064e6 + 95.008e6) / 2309888.0, "items_6d",
                 "one ncu capture of the level-0 launch on workload 4 at 1/32 scale, "
                 "scaled by particles"),
}
# Instruction issue of the search kernels from the same captures: the share
# of cycles an instruction issued and the lanes active per instruction.  For
# a tree walk their product -- the share of the SM's lane-issue capacity
# doing work -- says more than an HBM fraction.
NCU_ISSUE = {
    "k_fof6_w": (0.774138, 27.75),
    "k_nn": (0.662851, 4.62),
    "k_bh_walk": (0.698618, 19.11),
    "k_llist_w": (0.642338, 14.73),
    "k_kahn": (0.219013, 27.52),
}
NCU_ISSUE_SOURCE = "ncu, workload 4 at 1/32 scale, one launch per kernel"


def short_name(mangled):
    """rsg kernel name from its mangled symbol (_ZN3rsg<len><name>...)."""
    import re
    m = re.match(r"_ZN3rsg(\d+)", mangled)
    if not m:
        return mangled
    k = int(m.group(1))
    return mangled[m.end():m.end() + k]


def parse_table(txt):
    rows = []
    for line in txt.splitlines():
        parts = line.split("\t")  # name, launches, total ms[, gap before ms]
        if len(parts) >= 3:
            rows.append((short_name(parts[0]), int(parts[1]), float(parts[2])))
    return rows


def load_pkg():
    import importlib.util
    d = os.path.join(ROOT, "mpi-rockstar_gb300")
    if "mpi_rockstar_gb300" in sys.modules:
        return sys.modules["mpi_rockstar_gb300"]
    spec = importlib.util.spec_from_file_location(
        "mpi_rockstar_gb300", os.path.join(d, "__init__.py"), submodule_search_locations=[d])
    m = importlib.util.module_from_spec(spec)
    sys.modules["mpi_rockstar_gb300"] = m
    spec.loader.exec_module(m)
    return m


def peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            return json.load(f), "measured"
    except OSError:
        return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0}, "fallback"


class Clocks:
    """nvidia-smi sampling during the timed region."""

    def __init__(self, dev):
        self.f = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)
        q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
        try:
            self.p = subprocess.Popen(["nvidia-smi", "-i", str(dev), "--query-gpu=" + q,
                                       "--format=csv,noheader,nounits", "-lms", "200"],
                                      stdout=self.f, stderr=subprocess.DEVNULL)
        except OSError:
            self.p = None

    def stop(self):
        if self.p is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.p.terminate()
        self.p.wait()
        self.f.seek(0)
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in self.f.read().splitlines():
            parts = [x.strip() for x in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                mx = float(parts[2])
            except ValueError:
                continue
            for nm, v in zip(names, parts[5:9]):
                if v.lower() == "active":
                    reasons.add(nm)
        os.unlink(self.f.name)
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": mx,
                "reasons": sorted(reasons), "samples": len(sm)}


def cpu_baseline_port(rk, cfg_id, scale):
    """The oracle restatement on one core over a bounded sample: workload
    `cfg_id` at `scale` (same density and structure), the whole path.
    Returns the baseline entry and the sample with the oracle's output, which
    the parity check compares the GPU with."""
    from oracle import restatement as O
    O.build()
    p, box, mp, _ = rk.synth(cfg_id, scale, SEED)
    c = rk.Config(particle_mass=mp, box_size=box, total_particles=len(p))
    O.setup(c)
    t0 = time.perf_counter()
    fp, off, sz = O.fof(p)
    t1 = time.perf_counter()
    ro = O.find_subs(fp, off, sz)
    t2 = time.perf_counter()
    entry = {"value": len(p) / (t2 - t0), "unit": "particles/s", "cores": 1, "kind": "port",
             "sample": "workload %d at scale %g (%d particles), full path, one step, 1 thread"
                       % (cfg_id, scale, len(p)),
             "fof_s": round(t1 - t0, 3), "find_subs_s": round(t2 - t1, 3)}
    return entry, (p, c, fp, off, sz, ro)


HALO_INT = ("num_p", "num_child_particles", "n_core", "flags")


def _halo_labels(parts, halos, nid):
    """Halo index of every particle id (-1: in no halo)."""
    lab = np.full(nid, -1, np.int64)
    n = np.clip(halos["num_p"], 0, None).astype(np.int64)
    keep = np.flatnonzero(n > 0)
    cnt = n[keep]
    if not len(cnt):
        return lab
    first = np.concatenate([[0], np.cumsum(cnt)[:-1]])
    pos = np.repeat(halos["p_start"][keep].astype(np.int64) - first, cnt) + np.arange(cnt.sum())
    lab[parts["id"][pos]] = np.repeat(keep, cnt)
    return lab


def catalogue_compare(pa, ha, pb, hb, tol=1e-4):
    """Two halo catalogues of the same particles: particles outside halos
    with identical members on both sides, and matched halos with a float
    field beyond `tol` (relative) or a different integer field."""
    nid = int(max(pa["id"].max(initial=0), pb["id"].max(initial=0))) + 1
    la, lb = _halo_labels(pa, ha, nid), _halo_labels(pb, hb, nid)
    inside = (la >= 0) | (lb >= 0)
    w = len(hb) + 1
    uk, cnt = np.unique((la[inside] + 1) * w + (lb[inside] + 1), return_counts=True)
    A, B = uk // w - 1, uk % w - 1
    sa = np.bincount(la[la >= 0], minlength=len(ha))
    sb = np.bincount(lb[lb >= 0], minlength=len(hb))
    ok = (A >= 0) & (B >= 0)
    ok[ok] &= (cnt[ok] == sa[A[ok]]) & (cnt[ok] == sb[B[ok]])
    mA, mB = A[ok], B[ok]
    over = np.zeros(len(mA), bool)
    for f in ha.dtype.names:
        if ha.dtype[f].base.kind != "f":
            continue
        x = ha[f][mA].astype(np.float64).reshape(len(mA), -1)
        y = hb[f][mB].astype(np.float64).reshape(len(mB), -1)
        same = (x == y) | (np.isnan(x) & np.isnan(y))
        den = np.maximum(np.abs(x), np.abs(y))
        with np.errstate(invalid="ignore", divide="ignore"):
            e = np.where(same, 0.0, np.abs(x - y) / np.where(den > 0, den, 1.0))
        over |= (e > tol).any(axis=1)
    for f in HALO_INT:
        over |= ha[f][mA] != hb[f][mB]
    return {"membership_diff_particles": int(cnt[~ok].sum()),
            "halos_with_particles": [int((sa > 0).sum()), int((sb > 0).sum())],
            "halos_matched": int(len(mA)), "halos_over_1e-4": int(over.sum())}


def canon_nan(a):
    b = a.copy()
    for f in b.dtype.names:
        if b.dtype[f].base.kind == "f":
            v = b[f]
            v[np.isnan(v)] = np.nan
    return b


def sample_parity(rk, sample):
    """The GPU path (rsg_path_device, both forms) on the CPU baseline's
    sample against the oracle's output for it."""
    import torch
    p, c, fp, off, sz, ro = sample
    d_in = torch.from_numpy(p.view(np.uint8).reshape(-1)).cuda()
    out = {"sample_particles": len(p)}
    for form, batched in (("plain", False), ("batched", True)):
        path = rk.DevicePath(len(p), c, batched=batched)
        path.run(d_in.data_ptr())
        parts, h, e = path.results()
        cmp = catalogue_compare(ro[0], ro[1], parts, h)
        if not batched:
            exact = (parts.tobytes() == ro[0].tobytes()
                     and canon_nan(h).tobytes() == canon_nan(ro[1]).tobytes()
                     and all(np.array_equal(e[f], ro[2][f]) for f in e.dtype.names
                             if f != "_pad"))
            out["plain_vs_oracle"] = "bit-identical" if exact else "differs"
            cmp["bit_identical"] = exact
        out[form] = cmp
        cmp["near_threshold_pairs"] = rk.last_stats()["near_6d"]
        del path
    torch.cuda.empty_cache()
    return out


# ---- reference arm: the oracle port over all host cores -------------------
_REF_CFG = None


def _ref_init(cfg_fields):
    global _REF_CFG
    sys.path.insert(0, ROOT)
    from oracle import layouts as OL
    from oracle import restatement as O
    O.build()
    _REF_CFG = OL.Config(**cfg_fields)
    O.setup(_REF_CFG)


def _ref_worker(args):
    from oracle import restatement as O
    parts, off, sz = args
    out, h, e = O.find_subs(parts, off, sz)
    return len(h)


def pool_find_subs(pool, ncores, fp, off, sz):
    """find_subs over the groups on the pool's processes, groups dealt
    largest first to the least loaded process (as the reference's dynamic
    OpenMP loop hands them out); returns the number of halos."""
    order = np.argsort(-sz, kind="stable")
    chunks = [[] for _ in range(ncores)]
    load = np.zeros(ncores)
    for g in order:
        k = int(np.argmin(load))
        chunks[k].append(g)
        load[k] += float(sz[g]) * np.log2(float(sz[g]) + 2)
    jobs = []
    for ch in chunks:
        if not ch:
            continue
        ch = np.array(sorted(ch))
        parts = np.concatenate([fp[off[g]:off[g] + sz[g]] for g in ch])
        o = np.concatenate([[0], np.cumsum(sz[ch])[:-1]])
        jobs.append((parts, o, sz[ch]))
    return sum(pool.map(_ref_worker, jobs))


def reference_arm(args, rk):
    """The reference's algorithm on the host cores: the C restatement (pinned
    bit-exact to the reference's sources) with the FOF serial, as rockstar()
    runs it, and find_subs over the groups on one process per core, largest
    groups first, as the reference's dynamic OpenMP loop deals them."""
    import dataclasses
    import multiprocessing as mp_
    from concurrent.futures import ProcessPoolExecutor
    from oracle import layouts as OL
    from oracle import restatement as O
    O.build()
    rscale = args.ref_scale if args.ref_scale else REF_SCALE.get(args.cfg, 1.0) * args.scale
    p, box, mp, _ = rk.synth(args.cfg, rscale, SEED)
    n_full = rk.synth_count(args.cfg, args.scale, SEED)
    fields = {f.name: getattr(rk.Config(particle_mass=mp, box_size=box, total_particles=len(p)),
                              f.name) for f in dataclasses.fields(OL.Config)}
    O.setup(OL.Config(**fields))
    ncores = os.cpu_count() or 1
    pool = ProcessPoolExecutor(ncores, mp_context=mp_.get_context("spawn"),
                               initializer=_ref_init, initargs=(fields,))

    def step():
        fp, off, sz = O.fof(p)  # serial, as rockstar() is in the reference
        return pool_find_subs(pool, ncores, fp, off, sz)

    for _ in range(args.warmup):
        step()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        step()
    dt = (time.perf_counter() - t0) / args.steps
    pool.shutdown()
    v = len(p) / dt
    line = {"impl": "reference", "metric": METRIC, "value": v, "unit": "particles/s",
            "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": dt * 1e3, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32+f64", "data": "synthetic",
            "config": {"workload": "synthetic workload %d at scale %g: %d particles"
                                   % (args.cfg, args.scale, n_full),
                       "particles": n_full, "sample_particles": len(p), "host_cores": ncores},
            "cpu_baseline": {"value": v, "unit": "particles/s", "cores": ncores, "kind": "port",
                             "sample": "workload %d at scale %g (%d particles, same density and "
                                       "structure) per step; FOF serial, find_subs over the "
                                       "groups on %d processes" % (args.cfg, rscale, len(p),
                                                                   ncores)},
            "e2e": {"value": v, "unit": "particles/s", "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def cpu_table(rk, specs, repeats):
    """The reference's CPU path per workload, as the reference arm runs it:
    the C restatement with the FOF serial and find_subs over the groups on
    one process per host core (largest first); best of `repeats`.  One JSON
    line per workload (the table of the benchmark spec)."""
    import multiprocessing as mp_
    from concurrent.futures import ProcessPoolExecutor
    import dataclasses
    from oracle import layouts as OL
    from oracle import restatement as O
    O.build()
    ncores = os.cpu_count() or 1
    for cfg_id, scale in specs:
        p, box, mp, _ = rk.synth(cfg_id, scale, SEED)
        fields = {f.name: getattr(rk.Config(particle_mass=mp, box_size=box,
                                            total_particles=len(p)), f.name)
                  for f in dataclasses.fields(OL.Config)}
        O.setup(OL.Config(**fields))
        pool = ProcessPoolExecutor(ncores, mp_context=mp_.get_context("spawn"),
                                   initializer=_ref_init, initargs=(fields,))
        best_f = best_s = None
        for _ in range(repeats):
            t0 = time.perf_counter()
            fp, off, sz = O.fof(p)
            t1 = time.perf_counter()
            pool_find_subs(pool, ncores, fp, off, sz)
            t2 = time.perf_counter()
            best_f = min(best_f or 1e30, t1 - t0)
            best_s = min(best_s or 1e30, t2 - t1)
        pool.shutdown()
        print(json.dumps({"workload": cfg_id, "scale": scale, "particles": len(p),
                          "groups": len(sz), "host_cores": ncores, "fof_s": round(best_f, 3),
                          "find_subs_s": round(best_s, 3),
                          "particles_per_s": len(p) / (best_f + best_s),
                          "repeats": repeats}), flush=True)


def precision_study(rk, scale, forms):
    """Potential forms against the first of `forms` (normally 3, the FP64
    direct sum) on the isolated-groups workload (mpi-rockstar_gb300/precision.py)."""
    from mpi_rockstar_gb300 import precision
    rk.build()
    p, box, mp, ng = rk.synth(3, scale, SEED)
    cfg = rk.Config(particle_mass=mp, box_size=box, total_particles=len(p))
    t0 = time.time()
    runs = precision.run_forms(rk, p, cfg, forms)
    res = precision.compare(runs, cfg, ref=forms[0], forms=forms[1:])
    res.update({"workload": "isolated groups (potential/unbinding precision study)",
                "scale": scale, "planted_groups": ng, "study_s": round(time.time() - t0, 1)})
    print(json.dumps(res))


def profile_only(rk, cfg_id, scale, warmup):
    """The batched path alone: `warmup` steps, then one step whose launches
    are timed with CUDA events (the small case an ncu capture runs)."""
    import torch
    rk.build()
    p, box, mp, _ = rk.synth(cfg_id, scale, SEED)
    cfg = rk.Config(particle_mass=mp, box_size=box, total_particles=len(p))
    d_in = torch.from_numpy(p.view(np.uint8).reshape(-1)).cuda()
    path = rk.DevicePath(len(p), cfg, batched=True)
    for _ in range(warmup):
        path.run(d_in.data_ptr())
    torch.cuda.synchronize()
    rk.profile_select("*")
    t0 = time.perf_counter()
    res = path.run(d_in.data_ptr())
    torch.cuda.synchronize()
    ms = (time.perf_counter() - t0) * 1e3
    rows = [l.split("\t") for l in rk.profile_table().strip().splitlines()]
    rk.profile_select("")
    print(json.dumps({"workload": "synthetic workload %d at scale %g: %d particles"
                      % (cfg_id, scale, len(p)), "warmup": warmup,
                      "step_ms_with_events": ms, "halos": res[2],
                      "launches": {r[0]: int(r[1]) for r in rows},
                      "kernel_ms": {r[0]: float(r[2]) for r in rows[:12]}}))


IO_BOX, IO_SCALE = 250.0, 0.5  # box (Mpc/h) and scale factor of the input file


def io_write_gadget(path, n):
    """A GADGET-2 file of n type-1 particles: tagged variant (8-byte block
    tags), little-endian, float coordinates, 8-byte ids in a random order,
    header mass 1e-3 (1e7 Msun/h)."""
    rng = np.random.default_rng(SEED)
    pos = rng.uniform(0, IO_BOX, (n, 3)).astype("<f4")
    vel = rng.normal(0, 300.0, (n, 3)).astype("<f4")
    ids = (rng.permutation(n).astype("<i8") + 1) * 3
    a = IO_SCALE
    npart = [0, n, 0, 0, 0, 0]
    hdr = struct.pack("<6I6ddd2i6I2i4d2i6ii", *npart, 0, 1e-3, 0, 0, 0, 0, a, 1 / a - 1, 0, 0,
                      *npart, 0, 1, IO_BOX, 0.3, 0.7, 0.7, 0, 0, 0, 0, 0, 0, 0, 0, 0)
    with open(path, "wb") as f:
        for tag, blob in ((b"HEAD", hdr.ljust(256, b"\0")), (b"POS ", pos.tobytes()),
                          (b"VEL ", vel.tobytes()), (b"ID  ", ids.tobytes())):
            f.write(struct.pack("<I4sII", 8, tag, len(blob) + 8, 8))
            f.write(struct.pack("<I", len(blob)) + blob + struct.pack("<I", len(blob)))


def io_cpu_read(path, n, particle_dtype):
    """One-thread numpy restatement of load_particles_gadget2
    (src/io/io_gadget.c:200-254) for the file of io_write_gadget: positions
    as stored (length conversion 1), velocities times sqrt(a) in double
    rounded to float, ids as stored."""
    o = 16 + 264  # HEAD tag record, header record
    out = np.zeros(n, particle_dtype)
    for k in range(2):
        o += 16 + 4  # block tag record, record marker
        blk = np.fromfile(path, "<f4", 3 * n, offset=o).reshape(n, 3)
        fac = 1.0 if k == 0 else math.sqrt(IO_SCALE)
        out["pos"][:, 3 * k:3 * k + 3] = (blk.astype(np.float64) * fac).astype(np.float32)
        o += 12 * n + 4
    out["id"] = np.fromfile(path, "<i8", n, offset=o + 16 + 4)
    return out


def io_table(rk, n, reps=3):
    """Particle input at n particles: the file of io_write_gadget read by
    rsg_read_gadget2 (host records, device assembly, records back to the
    host), then rsg_sort_particles_by_id on the file-order records (host ->
    device radix sort -> host), each best of `reps` after one untimed call.
    Beside each: the one-thread numpy restatement of the reference's reader
    and of its id sort (std::sort by id, src/mpi_main.cpp:2021-2024; here
    numpy's stable sort), with the outputs compared byte for byte.  The file
    is written first, so reads come from the page cache.  One JSON line."""
    fd, path = tempfile.mkstemp(suffix=".gadget2")
    os.close(fd)

    def best(fn):
        fn()
        ts = []
        for _ in range(reps):
            t0 = time.perf_counter()
            out = fn()
            ts.append(time.perf_counter() - t0)
        return min(ts), out

    try:
        io_write_gadget(path, n)
        file_bytes = os.path.getsize(path)
        t_cpu_read, p_cpu = best(lambda: io_cpu_read(path, n, rk.PARTICLE))
        t_cpu_sort, s_cpu = best(lambda: p_cpu[np.argsort(p_cpu["id"], kind="stable")])
        import torch
        torch.cuda.set_device(0)
        rk.build()
        cfg = rk.Config(particle_mass=1e9, box_size=IO_BOX, total_particles=n)
        t_read, (p_gpu, _) = best(lambda: rk.read_gadget2(path, cfg))
        # in place, as the reference sorts p; each call gets the file order
        work = np.empty_like(p_gpu)
        ts = []
        for r in range(reps + 1):  # the first one untimed
            np.copyto(work, p_gpu)
            t0 = time.perf_counter()
            rk.sort_by_id(work, inplace=True)
            if r:
                ts.append(time.perf_counter() - t0)
        t_sort, s_gpu = min(ts), work
        t_dread, (d_gpu, _) = best(lambda: rk.read_gadget2_device(path, cfg))
        d_read_ok = d_gpu.cpu().numpy().tobytes() == p_cpu.tobytes()
        pristine = d_gpu.clone()
        ts = []
        for r in range(reps + 1):  # the first one untimed
            d_gpu.copy_(pristine)
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            rk.sort_by_id_device(d_gpu)
            torch.cuda.synchronize()
            if r:
                ts.append(time.perf_counter() - t0)
        t_dsort = min(ts)
        d_sort_ok = d_gpu.cpu().numpy().tobytes() == s_cpu.tobytes()
        del d_gpu, pristine
        # the internal format (the records verbatim after a 256-byte header):
        # the reference's single fread restated as one np.fromfile
        rk.write_internal(path, s_cpu, cfg)
        t_icpu, i_cpu = best(lambda: np.fromfile(path, rk.PARTICLE, offset=256))
        t_ihost, (i_host, _) = best(lambda: rk.read_internal(path, cfg))
        t_idev, (i_dev, _) = best(lambda: rk.read_internal_device(path, cfg))
        internal = {"cpu_port_s": t_icpu, "host_s": t_ihost, "device_s": t_idev,
                    "device_particles_per_s": n / t_idev,
                    "identical": i_host.tobytes() == i_cpu.tobytes() == s_cpu.tobytes()
                    and i_dev.cpu().numpy().tobytes() == s_cpu.tobytes()}
        del i_dev
    finally:
        os.unlink(path)
    rec_bytes = n * rk.PARTICLE.itemsize
    hbm = peaks()[0]["hbm_gbs"]
    print(json.dumps({
        "workload": "GADGET-2 file, %d particles (%d bytes), tagged variant, float "
                    "coordinates, 8-byte ids in random order" % (n, file_bytes),
        "reader": {"particles_per_s": n / t_read, "s": t_read,
                   "cpu_port_particles_per_s": n / t_cpu_read, "cpu_port_s": t_cpu_read,
                   "h2d_bytes": n * (12 + 12 + 8), "d2h_bytes": rec_bytes,
                   "identical": p_gpu.tobytes() == p_cpu.tobytes()},
        "id_sort": {"particles_per_s": n / t_sort, "s": t_sort,
                    "cpu_port_particles_per_s": n / t_cpu_sort, "cpu_port_s": t_cpu_sort,
                    "h2d_bytes": rec_bytes, "d2h_bytes": rec_bytes,
                    "identical": s_gpu.tobytes() == s_cpu.tobytes(),
                    "sorted": bool(np.all(np.diff(s_gpu["id"]) > 0))},
        "device_resident": {
            "reader_to_device_s": t_dread, "reader_to_device_particles_per_s": n / t_dread,
            "reader_identical": d_read_ok,
            "id_sort_device_s": t_dsort, "id_sort_device_particles_per_s": n / t_dsort,
            "id_sort_identical": d_sort_ok,
            "id_sort_roofline": {"bound": "hbm", "algorithmic_bytes": 2 * rec_bytes,
                                 "achieved_gbs": 2 * rec_bytes / t_dsort / 1e9, "peak_gbs": hbm,
                                 "frac": 2 * rec_bytes / t_dsort / 1e9 / hbm,
                                 "note": "records read and written once; host-timed call "
                                         "including the id-range read-back"}},
        "internal_format": internal,
        "cpu_port": {"cores": 1, "kind": "port",
                     "what": "numpy restatement of the reader; numpy stable sort for the id sort"},
        "reps": reps}))


def run_autotune(rk, cfg_id, scale):
    """Size-class thresholds by measurement (mpi-rockstar_gb300/autotune.py)."""
    from mpi_rockstar_gb300 import autotune
    rk.build()
    p, box, mp, _ = rk.synth(cfg_id, scale, SEED)
    cfg = rk.Config(particle_mass=mp, box_size=box, total_particles=len(p))
    res = autotune.autotune(rk, p, cfg, log=lambda m: print(m, file=sys.stderr, flush=True))
    workload = "synthetic workload %d at scale %g: %d particles" % (cfg_id, scale, len(p))
    autotune.save(res, rk.TUNING_FILE, workload)
    print(json.dumps({"workload": workload, "best": res["best"], "default": res["default"],
                      "best_ms": res["best_ms"], "default_ms": res["default_ms"],
                      "trials": len(res["trials"])}))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--cfg", type=int, default=4,
                    help="synthetic workload (csrc/synth.c); 4 is the 512^3 snapshot")
    ap.add_argument("--scale", type=float, default=1.0)
    ap.add_argument("--plain-steps", type=int, default=1,
                    help="timed steps of the plain form (after one untimed step) on workloads "
                         "above 2^23 particles; smaller ones use --steps/--warmup")
    ap.add_argument("--sample-scale", type=float, default=None,
                    help="scale of the bounded sample the CPU baseline and the oracle parity "
                         "check run on (default: per workload, about 10-20 s of CPU work)")
    ap.add_argument("--ref-scale", type=float, default=None,
                    help="scale of the sample each reference-arm step runs on")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--kernel-table", default="",
                    help="write per-kernel CUDA-event times of one extra (untimed) step of "
                         "each form to this file")
    ap.add_argument("--precision-study", action="store_true",
                    help="instead of the bench line: the potential precision study on the "
                         "isolated-groups workload at --scale, one JSON line")
    ap.add_argument("--autotune", action="store_true",
                    help="instead of the bench line: tune the batched form's size-class "
                         "thresholds on the workload (--cfg, --scale) and write them to "
                         "mpi-rockstar_gb300/tuning.json, which later runs apply")
    ap.add_argument("--profile-only", action="store_true",
                    help="instead of the bench line: --warmup batched steps, then one step "
                         "with CUDA events around every launch; prints the step time and "
                         "each kernel's launches (the command the ncu captures run)")
    ap.add_argument("--cpu-table", default="",
                    help="instead of the bench line: the reference's CPU path (FOF serial, "
                         "find_subs on every host core) per workload, best of 3, for "
                         "'cfg:scale,cfg:scale,...'; one JSON line each")
    ap.add_argument("--io-table", type=int, default=0,
                    help="instead of the bench line: particle input (GADGET-2 reader and id "
                         "sort) at this many particles against a one-thread CPU restatement; "
                         "one JSON line")
    ap.add_argument("--precision-forms", default="3,0,1,2",
                    help="potential forms of the study; the first is the reference "
                         "(3: FP64 direct sum, O(n^2) per group)")
    args = ap.parse_args()
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rk = load_pkg()
    if args.precision_study:
        if rank == 0:
            precision_study(rk, args.scale, [int(f) for f in args.precision_forms.split(",")])
        return
    if args.autotune:
        if rank == 0:
            run_autotune(rk, args.cfg, args.scale)
        return
    if args.profile_only:
        if rank == 0:
            profile_only(rk, args.cfg, args.scale, args.warmup)
        return
    if args.io_table:
        if rank == 0:
            io_table(rk, args.io_table)
        return
    if args.cpu_table:
        if rank == 0:
            specs = [(int(a), float(b)) for a, b in
                     (x.split(":") for x in args.cpu_table.split(","))]
            cpu_table(rk, specs, 3)
        return
    if args.impl == "reference":
        if rank == 0:
            reference_arm(args, rk)
        return
    # CPU baseline first: no GPU context exists yet
    cpu, sample = None, None
    if rank == 0 and world >= 1 and not args.no_cpu_baseline and args.gpus == 1:
        sscale = args.sample_scale or SAMPLE_SCALE.get(args.cfg, 0.1) * args.scale
        cpu, sample = cpu_baseline_port(rk, args.cfg, min(sscale, args.scale))
    import torch
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    rk.build()
    tuned = rk.load_tuning()  # size-class thresholds from a committed autotune run, if any
    p, box, mp, _ = rk.synth(args.cfg, args.scale, SEED + rank)
    n = len(p)
    cfg = rk.Config(particle_mass=mp, box_size=box, total_particles=n)
    raw = torch.from_numpy(p.view(np.uint8).reshape(-1))
    d_in = raw.cuda()
    flush = torch.empty(256 << 20, dtype=torch.uint8, device="cuda")

    def event_table(path):
        """One untimed step with CUDA events around every kernel."""
        torch.cuda.synchronize()
        rk.profile_select("*")
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record()
        path.run(d_in.data_ptr())
        e1.record()
        torch.cuda.synchronize()
        tab = rk.profile_table()
        rk.profile_select("")
        return e0.elapsed_time(e1), tab

    def timed(path, steps, prof, warmup=None):
        for _ in range(args.warmup if warmup is None else warmup):
            path.run(d_in.data_ptr())
        torch.cuda.synchronize()
        if dist:
            dist.barrier()
        if prof:
            rk.profile_select(prof)
        l0 = rk.launch_count()
        times, res = [], None
        for _ in range(steps):
            flush.fill_(1)  # L2 flush between steps (outside the step's events)
            torch.cuda.synchronize()
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record()
            res = path.run(d_in.data_ptr())
            e1.record()
            torch.cuda.synchronize()
            times.append(e0.elapsed_time(e1))
        launches = rk.launch_count() - l0
        kl, kms = rk.profile_read() if prof else (0, 0.0)
        rk.profile_select("")
        return float(np.mean(times)), res, launches, kl, kms

    # plain drop-in (the reference's results bit for bit), then the batched form;
    # on the large workloads the plain form gets one untimed and --plain-steps
    # timed steps (it is reported beside the headline, not as it)
    big = n > (1 << 23)
    plain_steps = args.plain_steps if big else args.steps
    plain_path = rk.DevicePath(n, cfg, batched=False)
    plain_ms, plain_res, plain_launches, _, _ = timed(plain_path, plain_steps, None,
                                                      1 if big else None)
    batched_path = rk.DevicePath(n, cfg, batched=True)
    batched_path.run(d_in.data_ptr())
    # the dominant kernel of the batched step, by device time
    tab_ms, tab = event_table(batched_path)
    rows = parse_table(tab)
    top = rows[0][0] if rows else None
    clocks = Clocks(local)
    step_ms, res, launches, kl, kms = timed(batched_path, args.steps, top)
    clk = clocks.stop()
    stats = rk.last_stats()
    # the batched form's output against the plain form's on the full workload
    # (the plain form is pinned bit for bit to the oracle by the tests and by
    # the sample check below)
    tol = None
    if rank == 0:
        pa, ha, _ = plain_path.results()
        pb, hb, _ = batched_path.results()
        tol = catalogue_compare(pa, ha, pb, hb)
        tol["near_threshold_pairs"] = stats["near_6d"]
        tol["against"] = "plain form on the same snapshot"
        del pa, ha, pb, hb
    if dist:
        t = torch.tensor([step_ms], device="cuda")
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        step_ms = float(t.item())
        dist.barrier()
    value = n * world / (step_ms * 1e-3)

    if args.kernel_table and rank == 0:
        # the batched table above and one extra step of the plain form
        with open(args.kernel_table, "w") as f:
            f.write("# form batched: step %.3f ms (events around every kernel)\n" % tab_ms)
            f.write(tab)
            if n <= (1 << 22):  # the plain form's table: one more plain step
                pms, ptab = event_table(plain_path)
                f.write("# form plain: step %.3f ms (events around every kernel)\n" % pms)
                f.write(ptab)

    # e2e through the C ABI with pinned host buffers: the reference's two
    # calls (rockstar(), then find_subs over the groups) on the caller's
    # array, which both permute in place as the reference does; the array is
    # refilled from the snapshot before each step, outside the timed region.
    pin = torch.empty(n * 32, dtype=torch.uint8, pin_memory=True)
    host = pin.numpy().view(rk.PARTICLE)
    e2e_t = []
    h2d = d2h = 0
    for it in range(3):
        pin.copy_(raw)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        fp, off, sz = rk.rockstar_fof(host, cfg, inplace=True)
        parts, halos, extra = rk.find_subs(fp, off, sz, cfg, batched=True, inplace=True)
        e2e_t.append(time.perf_counter() - t0)
        h2d = n * 32 + len(fp) * 32 + 16 * len(off)
        d2h = len(fp) * 32 + 16 * len(off) + len(fp) * 32 + len(halos) * (312 + 48)
    e2e_v = n * world / min(e2e_t)
    # the same two calls on pageable memory, as the reference's malloc'd p
    # arrives through the drop-in (large pageable buffers take the library's
    # staging threads)
    pageable = np.empty(n, rk.PARTICLE)
    e2e_pg = []
    for it in range(2):
        np.copyto(pageable.view(np.uint8), p.view(np.uint8))
        t0 = time.perf_counter()
        fp, off, sz = rk.rockstar_fof(pageable, cfg, inplace=True)
        rk.find_subs(fp, off, sz, cfg, batched=True, inplace=True)
        e2e_pg.append(time.perf_counter() - t0)
    del pageable

    parity = None
    if sample is not None:
        del plain_path
        torch.cuda.empty_cache()
        parity = sample_parity(rk, sample)
        parity["oracle"] = "C restatement of the reference (oracle/), same sample"

    pk, pk_kind = peaks()
    roof = None
    if kl:
        avg_ms = kms / kl
        per_step = kl / max(args.steps, 1)
        model = ALGO_BYTES.get(top)
        algo = model(stats, per_step) if model else None
        ach = algo / (avg_ms * 1e-3) / 1e9 if algo else None
        peak = float(pk["hbm_gbs"])
        share = None
        if rows:
            share = sum(r[2] for r in rows if r[0] == top) / tab_ms
        traffic, tsrc = None, None
        if top in NCU_TRAFFIC:
            per_unit, unit_key, tsrc = NCU_TRAFFIC[top]
            traffic = per_unit * stats[unit_key] / max(per_step, 1)
        roof = {"kernel": top, "bound": "hbm", "achieved": ach, "peak": peak, "unit": "GB/s",
                "frac": (ach / peak) if ach else None, "traffic": traffic,
                "traffic_source": tsrc,
                "algorithmic_bytes_per_launch": algo, "launches": kl, "avg_ms": avg_ms,
                "share_of_step": share,
                "issue": ({"issue_active": NCU_ISSUE[top][0],
                           "lanes_per_instruction": NCU_ISSUE[top][1],
                           "issue_x_lanes": NCU_ISSUE[top][0] * NCU_ISSUE[top][1] / 32.0,
                           "source": NCU_ISSUE_SOURCE} if top in NCU_ISSUE else None),
                "peak_kind": "measured copy (MEASURED_PEAKS.json hbm_gbs)"
                             if pk_kind == "measured" else "fallback 6.8 TB/s"}
    line = {"metric": METRIC, "value": value, "unit": "particles/s", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": step_ms,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f32+f64", "data": "synthetic",
            "config": {"workload": "synthetic workload %d: %d particles, %.0f Mpc/h box"
                                   % (args.cfg, n, box),
                       "particles": n, "groups": res[1], "halos": res[2],
                       "l2": "flushed between steps (256 MiB write)", "form": "batched",
                       "plain_particles_per_s": n * world / (plain_ms * 1e-3),
                       "plain_ms_per_step": plain_ms, "plain_halos": plain_res[2],
                       "plain_steps": plain_steps,
                       "batched_over_plain": plain_ms / step_ms,
                       "tolerance": tol,
                       "plain_gpu_launches": plain_launches,
                       "tuning": rk.get_tuning(),
                       "tuning_source": "mpi-rockstar_gb300/tuning.json" if tuned else "defaults"},
            "e2e_pageable": {"value": n * world / min(e2e_pg), "unit": "particles/s",
                             "what": "the e2e calls on a pageable (malloc'd) particle array, "
                                     "best of 2"},
            "e2e": {"value": e2e_v, "unit": "particles/s", "h2d_bytes_per_step": h2d,
                    "d2h_bytes_per_step": d2h},
            "gpu_launches": launches, "roofline": roof, "cpu_baseline": cpu, "parity": parity,
            "work": stats,
            "clocks": clk, "peak_source": pk_kind}
    if rank == 0:
        print(json.dumps(line), flush=True)
    if dist:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
