"""rsg_rockstar_fof_noalloc: the allocation-free 3D FOF of one chunk, for
callers that run halo finding inside a simulation step on the GPU that holds
the simulation and cannot let a library cudaMalloc or cudaFree mid-step.

Two consecutive calls on caller-owned device buffers must each return what
the allocating entry point rsg_rockstar_fof returns for the same particles
(identical bytes: the FOF is integer/index work, so the tolerance is zero),
and the second call must leave the device's free memory unchanged.  The
file's name keeps it last in collection, so the calls also run after every
other test has used the library in this process; one test repeats them in a
fresh process, where the first call loads the library's code and scratch
array and the second must take nothing.  Calls that overlap from two host
threads get RSG_ERR_BUSY and leave their outputs alone."""
import json
import os
import subprocess
import sys
import threading

import numpy as np
import pytest

CASES = [(1, 0.25), (2, 1 / 32)]   # 65536 particles each: the entry's limit


def test_rejects_oversize_chunk(rk):
    """Checked on the host before any CUDA call (runs without a GPU)."""
    st = rk.setup_config(rk.Config())
    n = rk.NOALLOC_MAX_PARTICLES + 1
    with pytest.raises(rk.RockstarError) as e:
        rk.rockstar_fof_noalloc(16, n, st, 16 + 32 * n, 64, 64, n, 0)
    assert e.value.code == -4 and str(rk.NOALLOC_MAX_PARTICLES) in str(e.value)


def test_rejects_overlapping_buffers(rk):
    st = rk.setup_config(rk.Config())
    with pytest.raises(rk.RockstarError) as e:
        rk.rockstar_fof_noalloc(4096, 100, st, 4096 + 32 * 50, 64, 64, 100, 0)
    assert e.value.code == -1 and "overlap" in str(e.value)


@pytest.mark.gpu
@pytest.mark.parametrize("cfg_id,scale", CASES)
def test_noalloc_matches_rockstar_fof(rk, cfg_id, scale):
    import torch
    p, box, mp, _ = rk.synth(cfg_id, scale)
    n = len(p)
    assert n <= rk.NOALLOC_MAX_PARTICLES
    cfg = rk.Config(particle_mass=mp, box_size=box, total_particles=n)
    ref_p, ref_off, ref_sz = rk.rockstar_fof(p, cfg)

    st = rk.setup_config(cfg)
    dev = torch.device("cuda", 0)
    d_in = torch.from_numpy(p.view(np.uint8).copy()).to(dev)
    d_out = torch.empty(n * rk.PARTICLE.itemsize, dtype=torch.uint8, device=dev)
    cap = n // 2 + 1
    d_off = torch.empty(cap, dtype=torch.int64, device=dev)
    d_sz = torch.empty(cap, dtype=torch.int64, device=dev)
    stream = torch.cuda.Stream(device=dev)
    torch.cuda.synchronize()

    free = []
    for call in range(2):
        d_out.fill_(0xAB)
        d_off.fill_(-7)
        d_sz.fill_(-7)
        torch.cuda.synchronize()
        free.append(torch.cuda.mem_get_info(dev)[0])
        num_p, nf = rk.rockstar_fof_noalloc(d_in.data_ptr(), n, st, d_out.data_ptr(),
                                            d_off.data_ptr(), d_sz.data_ptr(), cap,
                                            stream.cuda_stream)
        torch.cuda.synchronize()
        free.append(torch.cuda.mem_get_info(dev)[0])
        got = d_out[: num_p * rk.PARTICLE.itemsize].cpu().numpy().view(rk.PARTICLE)
        assert num_p == len(ref_p), call
        assert nf == len(ref_off), call
        assert got.tobytes() == ref_p.tobytes(), call
        assert np.array_equal(d_off[:nf].cpu().numpy(), ref_off), call
        assert np.array_equal(d_sz[:nf].cpu().numpy(), ref_sz), call
    # the second call allocates nothing (2 MiB: the granularity of the count)
    assert abs(free[3] - free[2]) <= (2 << 20), free
    # input untouched
    assert d_in.cpu().numpy().tobytes() == p.tobytes()


@pytest.mark.gpu
def test_noalloc_group_capacity(rk):
    """Too small max_fofs is an error, reported after the groups are known."""
    import torch
    p, box, mp, _ = rk.synth(1, 0.05)
    n = len(p)
    st = rk.setup_config(rk.Config(particle_mass=mp, box_size=box, total_particles=n))
    dev = torch.device("cuda", 0)
    d_in = torch.from_numpy(p.view(np.uint8).copy()).to(dev)
    d_out = torch.empty_like(d_in)
    d_off = torch.empty(1, dtype=torch.int64, device=dev)
    d_sz = torch.empty(1, dtype=torch.int64, device=dev)
    with pytest.raises(rk.RockstarError) as e:
        rk.rockstar_fof_noalloc(d_in.data_ptr(), n, st, d_out.data_ptr(), d_off.data_ptr(),
                                d_sz.data_ptr(), 1, 0)
    assert e.value.code == -1 and "max_fofs" in str(e.value)


@pytest.mark.gpu
def test_noalloc_overlapping_calls_are_refused(rk):
    """Two host threads call at once on one device, each with its own output
    buffers: each call returns RSG_OK with rsg_rockstar_fof's bytes, or
    RSG_ERR_BUSY with its outputs untouched."""
    import torch
    p, box, mp, _ = rk.synth(2, 1 / 32)
    n = len(p)
    cfg = rk.Config(particle_mass=mp, box_size=box, total_particles=n)
    ref_p, ref_off, ref_sz = rk.rockstar_fof(p, cfg)
    st = rk.setup_config(cfg)
    dev = torch.device("cuda", 0)
    d_in = torch.from_numpy(p.view(np.uint8).copy()).to(dev)
    cap = n // 2 + 1
    bufs = [(torch.empty(n * 32, dtype=torch.uint8, device=dev),
             torch.empty(cap, dtype=torch.int64, device=dev),
             torch.empty(cap, dtype=torch.int64, device=dev),
             torch.cuda.Stream(device=dev)) for _ in range(2)]
    outcomes = []
    for rep in range(6):
        for out, off, sz, _ in bufs:
            out.fill_(0xAB)
            off.fill_(-7)
            sz.fill_(-7)
        torch.cuda.synchronize()
        res = [None, None]
        go = threading.Barrier(2)

        def call(k):
            out, off, sz, stream = bufs[k]
            torch.cuda.set_device(dev)
            go.wait()
            try:
                res[k] = rk.rockstar_fof_noalloc(d_in.data_ptr(), n, st, out.data_ptr(),
                                                 off.data_ptr(), sz.data_ptr(), cap,
                                                 stream.cuda_stream)
            except rk.RockstarError as e:
                res[k] = e.code
        th = [threading.Thread(target=call, args=(k,)) for k in range(2)]
        for t in th:
            t.start()
        for t in th:
            t.join()
        torch.cuda.synchronize()
        for k, (out, off, sz, _) in enumerate(bufs):
            if res[k] == -6:  # RSG_ERR_BUSY: nothing written
                assert (out == 0xAB).all() and (off == -7).all() and (sz == -7).all()
            else:
                num_p, nf = res[k]
                got = out[: num_p * 32].cpu().numpy().view(rk.PARTICLE)
                assert got.tobytes() == ref_p.tobytes()
                assert np.array_equal(off[:nf].cpu().numpy(), ref_off)
                assert np.array_equal(sz[:nf].cpu().numpy(), ref_sz)
        outcomes.append(tuple(r if isinstance(r, int) else 0 for r in res))
    assert all(o.count(0) >= 1 for o in outcomes), outcomes  # one call always runs


FRESH = r"""
import json, sys
import numpy as np
sys.path.insert(0, sys.argv[1]); sys.path.insert(0, sys.argv[1] + "/tests")
from conftest import load_pkg
import torch
rk = load_pkg()
p, box, mp, _ = rk.synth(1, 0.25)
n = len(p)
cfg = rk.Config(particle_mass=mp, box_size=box, total_particles=n)
st = rk.setup_config(cfg)
dev = torch.device("cuda", 0)
d_in = torch.from_numpy(p.view(np.uint8).copy()).to(dev)
d_out = torch.empty(n * 32, dtype=torch.uint8, device=dev)
cap = n // 2 + 1
d_off = torch.empty(cap, dtype=torch.int64, device=dev)
d_sz = torch.empty(cap, dtype=torch.int64, device=dev)
torch.cuda.synchronize()
free, outs = [], []
for call in range(2):
    free.append(torch.cuda.mem_get_info(dev)[0])
    num_p, nf = rk.rockstar_fof_noalloc(d_in.data_ptr(), n, st, d_out.data_ptr(),
                                        d_off.data_ptr(), d_sz.data_ptr(), cap, 0)
    torch.cuda.synchronize()
    free.append(torch.cuda.mem_get_info(dev)[0])
    outs.append((d_out[: num_p * 32].cpu().numpy().tobytes(), d_off[:nf].cpu().numpy(),
                 d_sz[:nf].cpu().numpy()))
ref_p, ref_off, ref_sz = rk.rockstar_fof(p, cfg)
same = all(o[0] == ref_p.tobytes() and np.array_equal(o[1], ref_off)
           and np.array_equal(o[2], ref_sz) for o in outs)
print(json.dumps({"free": free, "same": bool(same)}))
"""


@pytest.mark.gpu
def test_noalloc_in_fresh_process(rk):
    """In a process that has not used the library: the first call may take
    device memory once (the library's code and the scratch array load); the
    second takes none, and both equal rsg_rockstar_fof."""
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    r = subprocess.run([sys.executable, "-c", FRESH, root], capture_output=True, text=True,
                       timeout=600)
    assert r.returncode == 0, r.stderr[-3000:]
    res = json.loads(r.stdout.strip().splitlines()[-1])
    free = res["free"]
    assert res["same"]
    assert abs(free[3] - free[2]) <= (2 << 20), free
