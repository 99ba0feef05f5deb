"""rsg_rockstar_fof_noalloc: the allocation-free 3D FOF of one chunk.

Two consecutive calls on caller-owned device buffers must each return what
the allocating entry point rsg_rockstar_fof returns for the same particles
(identical bytes: the FOF is integer/index work, so the tolerance is zero),
and the second call must leave the device's free memory unchanged.  The
file's name keeps it last in collection, so the calls also run after every
other test has used the library in this process."""
import ctypes as C

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
