"""Autotuner for the batched form's size-class thresholds and chunk sizes.

The parameters are those of rsg_set_tuning (include/rockstar_gb300.h):
where the particle assignment switches to Morton-ordered buckets, where a
Barnes-Hut node takes the chunked pass and the chunk it uses, the potential
set copy segment, and the chunk sizes of the chunked norm_sd and basic
properties.  They change speed only, never a choice, so any value is valid.

The search is a coordinate descent: each parameter in turn takes every
candidate value while the others stay fixed, and the value with the lowest
median step time is kept when it beats the current one by more than
`min_gain` (step-to-step noise is about 1%).  Passes repeat until one
changes nothing, at most `passes` times.  A step is one batched
rsg_path_device call on device-resident particles, timed on the host around
the call (the call returns after its stream has drained).
"""
import json
import time

CANDIDATES = {
    "asc_bucket_min": (32, 64, 128, 256, 512),
    "bh_huge": (16384, 32768, 65536, 131072, 262144),
    "bh_chunk": (4096, 8192, 16384, 32768, 65536),
    "seg_max": (2048, 4096, 8192, 16384, 65536),
    "norm_chunk": (1024, 2048, 4096, 8192, 16384),
    "bp_big": (4096, 8192, 16384, 32768, 65536),
    "bp_chunk": (1024, 2048, 4096, 8192, 16384),
}


def _median(v):
    v = sorted(v)
    return v[len(v) // 2]


def device_step(rk, parts, cfg, reps):
    """A function timing the median of `reps` batched steps on device-resident
    particles (one warm-up step first)."""
    import numpy as np
    import torch

    d_in = torch.from_numpy(np.ascontiguousarray(parts).view(np.uint8).reshape(-1)).cuda()
    path = rk.DevicePath(len(parts), cfg, batched=True)
    path.run(d_in.data_ptr())  # warm-up: arena growth, module load

    def step_ms():
        ts = []
        for _ in range(reps):
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            path.run(d_in.data_ptr())
            ts.append((time.perf_counter() - t0) * 1e3)
        return _median(ts)

    return step_ms


def autotune(rk, parts, cfg, reps=5, passes=2, min_gain=0.01, names=None, log=None,
             step_ms=None):
    """Tunes on one workload (`parts`, a PARTICLE array, and its Config), or
    with any `step_ms()` timer.  Leaves the best values set and returns
    {"best", "default", "best_ms", "default_ms", "trials"}."""
    names = list(names or CANDIDATES)
    trials = []
    if step_ms is None:
        step_ms = device_step(rk, parts, cfg, reps)
    default = rk.get_tuning()
    cur = dict(default)
    cur_ms = step_ms()
    default_ms = cur_ms
    trials.append({"values": dict(cur), "ms": cur_ms})
    for _ in range(passes):
        changed = False
        for name in names:
            best_v, best_ms = cur[name], cur_ms
            for v in CANDIDATES[name]:
                if v == cur[name]:
                    continue
                rk.set_tuning(name, v)
                ms = step_ms()
                trials.append({"param": name, "value": v, "ms": ms})
                if log:
                    log("%s=%d: %.2f ms (current %.2f)" % (name, v, ms, cur_ms))
                if ms < best_ms * (1.0 - min_gain):
                    best_v, best_ms = v, ms
            rk.set_tuning(name, best_v)
            if best_v != cur[name]:
                cur[name], changed = best_v, True
                cur_ms = step_ms()  # re-measure with the new value in place
        if not changed:
            break
    return {"best": cur, "default": default, "best_ms": cur_ms, "default_ms": default_ms,
            "trials": trials}


def save(result, path, workload):
    out = dict(result)
    out["workload"] = workload
    with open(path, "w") as f:
        json.dump(out, f, indent=1)
