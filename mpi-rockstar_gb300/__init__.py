"""GB300 halo-finding hot path: host-side mirror of the reference interface.

The compute runs in the CUDA library _build/librockstar_gb300.so (kernels for
sm_103a behind the C ABI of include/rockstar_gb300.h); this module only
moves numpy arrays across that ABI with ctypes.  There is no CPU fallback:
if the library cannot be loaded every call raises, and without a GPU every
call that computes or moves data to the device raises.

Function names follow the reference calls they replace:
  rockstar_fof      <- rockstar(NULL, 1)            src/rockstar.c:53-128
  find_subs         <- find_subs() over all groups  src/groupies.c:669-708
                       as the loop of src/mpi_main.cpp:1363-1389 runs it
  compute_potential <- compute_potential()          src/potential.c:183-192
  compute_kinetic_energy <- compute_kinetic_energy() src/potential.c:194-211
  should_print, write_ascii, write_binary, write_particles
                    <- _should_print, output_ascii, output_binary,
                       output_full_particles        src/io/meta_io.c:266-461,
                                                    src/io/io_internal.c:118-186
  read_binary       <- load_binary_halos()          src/io/io_internal.c:199-225
  read_gadget2      <- load_particles_gadget2()     src/io/io_gadget.c:200-254
  read_internal, write_internal
                    <- load_particles_internal(), output_particles_internal()
                                                    src/io/io_internal.c:52-100
  sort_by_id        <- the std::sort by id          src/mpi_main.cpp:2021-2024
The *_device variants keep the records in device memory.  The file-format
calls that need no conversion (the catalogue writers and readers, the
internal-format host reader and writer) are host I/O with no device step.
"""
import ctypes as C
import os

import numpy as np

from .layouts import PARTICLE, HALO, EXTRA, POTENTIAL, Config, config_struct  # noqa: F401

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "_build", "librockstar_gb300.so")
SYNTH = os.path.join(HERE, "_build", "libsynth.so")


class RockstarError(RuntimeError):
    """A library call failed; carries the RSG_ERR_* code."""

    def __init__(self, code, msg):
        super().__init__("rockstar_gb300 error %d: %s" % (code, msg))
        self.code = code


def build():
    from . import builder
    return builder.build()


_lib = None


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB):
            raise RockstarError(-3, "CUDA extension not built: %s (call build())" % LIB)
        h = C.CDLL(LIB)
        vp, i64 = C.c_void_p, C.c_int64
        h.rsg_version.restype = C.c_int
        h.rsg_last_error.restype = C.c_char_p
        h.rsg_config_setup.argtypes = [vp]
        h.rsg_rockstar_fof.argtypes = [vp, vp, vp, vp, vp, i64, vp]
        h.rsg_debug_tree_order.argtypes = [vp, i64, C.c_int, C.c_int]
        h.rsg_debug_hierarchy.restype = i64
        h.rsg_debug_hierarchy.argtypes = [vp, vp, vp, i64]
        h.rsg_path_device.argtypes = [vp, i64, vp, vp, vp, vp, vp, vp, i64, vp, C.c_int32]
        h.rsg_find_subs_batch.argtypes = [vp, i64, vp, vp, i64, vp, vp, vp, i64, vp]
        h.rsg_launch_count.restype = i64
        h.rsg_profile_select.argtypes = [C.c_char_p]
        h.rsg_profile_read.argtypes = [vp, vp]
        h.rsg_last_stats.argtypes = [vp, C.c_int32]
        h.rsg_compute_potential.argtypes = [vp, i64, vp, C.c_int32]
        h.rsg_compute_kinetic_energy.argtypes = [vp, i64, vp, vp, C.c_float, vp]
        h.rsg_profile_table.restype = i64
        h.rsg_profile_table.argtypes = [C.c_char_p, i64]
        h.rsg_find_subs.argtypes = [vp, i64, vp, vp, i64, vp, vp, vp, i64, vp]
        h.rsg_rockstar_fof_noalloc.argtypes = [vp, i64, vp, vp, vp, vp, vp, i64, vp, vp]
        h.rsg_set_potential_form.restype = C.c_int32
        h.rsg_set_potential_form.argtypes = [C.c_int32]
        h.rsg_debug_keep_potentials.argtypes = [C.c_int32]
        h.rsg_keep_halo_records.restype = C.c_int32
        h.rsg_keep_halo_records.argtypes = [C.c_int32]
        h.rsg_halo_records.restype = i64
        h.rsg_halo_records.argtypes = [vp, i64, vp, vp, i64]
        h.rsg_set_tuning.restype = C.c_int32
        h.rsg_set_tuning.argtypes = [C.c_char_p, i64]
        h.rsg_get_tuning.restype = C.c_int32
        h.rsg_get_tuning.argtypes = [C.c_char_p, vp]
        h.rsg_debug_potentials.restype = i64
        h.rsg_debug_potentials.argtypes = [vp, i64]
        h.rsg_read_gadget2.argtypes = [C.c_char_p, vp, vp, vp, i64, vp]
        h.rsg_sort_particles_by_id.argtypes = [vp, i64]
        h.rsg_read_gadget2_device.argtypes = [C.c_char_p, vp, vp, vp, i64, vp]
        h.rsg_sort_particles_by_id_device.argtypes = [vp, i64]
        h.rsg_read_internal.argtypes = [C.c_char_p, vp, vp, i64, vp]
        h.rsg_read_binary.argtypes = [C.c_char_p, vp, vp, vp, i64, vp, i64]
        h.rsg_read_internal_device.argtypes = [C.c_char_p, vp, vp, i64, vp]
        h.rsg_write_internal.argtypes = [C.c_char_p, vp, i64, i64, i64, vp]
        h.rsg_should_print.argtypes = [vp, vp, vp]
        h.rsg_count_halos_to_print.restype = i64
        h.rsg_count_halos_to_print.argtypes = [vp, i64, vp, vp]
        h.rsg_write_ascii.argtypes = [C.c_char_p, vp, vp, i64, vp, vp]
        h.rsg_write_particles.argtypes = [C.c_char_p, vp, vp, i64, vp, i64, vp, i64, i64, vp,
                                          vp]
        h.rsg_write_binary.argtypes = [C.c_char_p, vp, i64, vp, i64, vp, vp]
        for name, args in _EXTRA_SIGS.items():
            if hasattr(h, name):
                getattr(h, name).argtypes = args
        _lib = h
    return _lib


_EXTRA_SIGS = {}


def _check(rc):
    if rc != 0:
        raise RockstarError(rc, lib().rsg_last_error().decode(errors="replace"))


def setup_config(cfg):
    """Returns a filled rsg_config struct (ctypes) for a layouts.Config."""
    st = config_struct(cfg)
    _check(lib().rsg_config_setup(C.byref(st)))
    return st


def rockstar_fof(parts, cfg, inplace=False):
    """3D FOF of an id-sorted particle array.  Returns (particles, offsets,
    sizes): the permuted/deduplicated particles and each group's range.
    With inplace=True the caller's (contiguous PARTICLE) array is permuted in
    place, as rsg_rockstar_fof does, and the returned particles are a view
    of its first num_p records."""
    st = setup_config(cfg)
    if inplace:
        if not (isinstance(parts, np.ndarray) and parts.dtype == PARTICLE
                and parts.flags.c_contiguous and parts.flags.writeable):
            raise ValueError("inplace needs a writeable contiguous PARTICLE array")
        pa = parts
    else:
        pa = np.array(parts, dtype=PARTICLE, copy=True)
    n = np.array([len(pa)], np.int64)
    cap = len(pa) // 2 + 1
    off = np.zeros(cap, np.int64)
    sz = np.zeros(cap, np.int64)
    nf = np.zeros(1, np.int64)
    _check(lib().rsg_rockstar_fof(pa.ctypes.data, n.ctypes.data, C.byref(st), off.ctypes.data,
                                  sz.ctypes.data, cap, nf.ctypes.data))
    k = int(nf[0])
    if inplace:
        return pa[:n[0]], off[:k].copy(), sz[:k].copy()
    return pa[:n[0]].copy(), off[:k].copy(), sz[:k].copy()


def find_subs(parts, offsets, sizes, cfg, batched=False, inplace=False):
    """Substructure + halo properties for every group.  batched=False is the
    plain drop-in (the reference's results bit for bit); batched=True the
    batched form (rsg_find_subs_batch).  Returns (particles, halos, extra);
    with inplace=True the caller's particle array is permuted in place and
    returned."""
    st = setup_config(cfg)
    if inplace:
        if not (isinstance(parts, np.ndarray) and parts.dtype == PARTICLE
                and parts.flags.c_contiguous and parts.flags.writeable):
            raise ValueError("inplace needs a writeable contiguous PARTICLE array")
        pa = parts
    else:
        pa = np.array(parts, dtype=PARTICLE, copy=True)
    off = np.ascontiguousarray(offsets, np.int64)
    sz = np.ascontiguousarray(sizes, np.int64)
    cap = int(sz.sum()) // 2 + len(sz) + 16
    h = np.zeros(cap, HALO)
    e = np.zeros(cap, EXTRA)
    nh = np.zeros(1, np.int64)
    fn = lib().rsg_find_subs_batch if batched else lib().rsg_find_subs
    _check(fn(pa.ctypes.data, len(pa), off.ctypes.data, sz.ctypes.data, len(sz),
              C.byref(st), h.ctypes.data, e.ctypes.data, cap, nh.ctypes.data))
    k = int(nh[0])
    return pa, h[:k].copy(), e[:k].copy()


def compute_potential(po, cfg, form=0):
    """Barnes-Hut potentials of one set of POTENTIAL records (permuted into
    tree order, pe filled): form 0 reference arithmetic, 1 FP32 form."""
    st = setup_config(cfg)
    q = np.array(po, dtype=POTENTIAL, copy=True)
    _check(lib().rsg_compute_potential(q.ctypes.data, len(q), C.byref(st), form))
    return q


def compute_kinetic_energy(po, vel_cen, pos_cen, scale_now, cfg):
    """compute_kinetic_energy (src/potential.c:194-211) on the GPU: a copy of
    the POTENTIAL records with ke set for every record whose ke >= 0."""
    st = setup_config(cfg)
    q = np.array(po, dtype=POTENTIAL, copy=True)
    vc = np.ascontiguousarray(vel_cen, np.float32)
    pc = np.ascontiguousarray(pos_cen, np.float32)
    _check(lib().rsg_compute_kinetic_energy(q.ctypes.data, len(q), vc.ctypes.data,
                                            pc.ctypes.data, float(scale_now), C.byref(st)))
    return q


POTENTIAL_FORMS = {0: "FP64 Barnes-Hut (reference arithmetic)",
                   1: "FP32 Barnes-Hut, Kahan-compensated sums",
                   2: "FP32 Barnes-Hut, plain sums",
                   3: "FP64 direct sum"}


def set_potential_form(form):
    """Potential form of the batched substructure form from now on
    (rsg_set_potential_form); returns the previous one."""
    r = int(lib().rsg_set_potential_form(int(form)))
    if r < 0:
        _check(r)
    return r


TUNING_NAMES = ("asc_bucket_min", "bh_huge", "bh_chunk", "seg_max", "norm_chunk", "bp_big",
                "bp_chunk")
TUNING_FILE = os.path.join(os.path.dirname(os.path.abspath(__file__)), "tuning.json")


def set_tuning(name, value):
    """One size-class threshold or chunk size of the batched form
    (rsg_set_tuning)."""
    _check(lib().rsg_set_tuning(name.encode(), int(value)))


def get_tuning(name=None):
    """The current value of one tuning parameter, or all of them as a dict."""
    if name is None:
        return {k: get_tuning(k) for k in TUNING_NAMES}
    v = np.zeros(1, np.int64)
    _check(lib().rsg_get_tuning(name.encode(), v.ctypes.data))
    return int(v[0])


def load_tuning(path=TUNING_FILE):
    """Applies the parameters of an autotune result file (the `best` dict);
    returns them, or None when the file does not exist."""
    import json
    if not os.path.exists(path):
        return None
    with open(path) as f:
        best = json.load(f)["best"]
    for k, v in best.items():
        set_tuning(k, v)
    return best


def keep_halo_records(on=True):
    """Keep, from the next calls, every halo's potential records as the
    reference's analyze_halo_generic receives them (rsg_keep_halo_records)."""
    _check(lib().rsg_keep_halo_records(1 if on else 0))


def halo_records(nh):
    """Records of the last call's nh halos: (records, first, count), halo i's
    records being records[first[i]:first[i] + count[i]] (sorted by r^2)."""
    first = np.zeros(max(nh, 1), np.int64)
    count = np.zeros(max(nh, 1), np.int64)
    k = int(lib().rsg_halo_records(None, 0, first.ctypes.data, count.ctypes.data, nh))
    if k < 0:
        _check(k)
    out = np.zeros(k, POTENTIAL)
    r = int(lib().rsg_halo_records(out.ctypes.data if k else None, k, first.ctypes.data,
                                   count.ctypes.data, nh))
    if r < 0:
        _check(r)
    return out, first[:nh].copy(), count[:nh].copy()


def keep_potentials(on=True):
    """Keep the potential records of each later find_subs / path call (test
    hook); last_potentials() returns them."""
    lib().rsg_debug_keep_potentials(1 if on else 0)


def last_potentials():
    """POTENTIAL records of the last call made after keep_potentials(True):
    sorted by halo (index in the halo output, stored in the `_pad` field),
    potential-only records (ke < 0) after a halo's own, then by radius."""
    k = int(lib().rsg_debug_potentials(None, 0))
    out = np.zeros(k, POTENTIAL)
    if k:
        lib().rsg_debug_potentials(out.ctypes.data, k)
    return out


def debug_hierarchy():
    """(level, size, target_r) of every subgroup node of the last find_subs."""
    cap = 1 << 22
    lv = np.zeros(cap, np.int32)
    n = np.zeros(cap, np.int32)
    tr = np.zeros(cap, np.float32)
    k = lib().rsg_debug_hierarchy(lv.ctypes.data, n.ctypes.data, tr.ctypes.data, cap)
    k = min(k, cap)
    return lv[:k].copy(), n[:k].copy(), tr[:k].copy()


def tree_order(parts, dim, leaf):
    """kd-tree build permutation computed on the GPU (test hook)."""
    pa = np.array(parts, dtype=PARTICLE, copy=True)
    _check(lib().rsg_debug_tree_order(pa.ctypes.data, len(pa), dim, leaf))
    return pa


_synth = None


def _synth_lib():
    global _synth
    if _synth is None:
        h = C.CDLL(SYNTH)
        h.synth_count.restype = C.c_int64
        h.synth_count.argtypes = [C.c_int, C.c_double, C.c_uint64]
        h.synth_generate.argtypes = [C.c_int, C.c_double, C.c_uint64, C.c_void_p, C.c_int64,
                                     C.c_void_p, C.c_void_p, C.c_void_p]
        _synth = h
    return _synth


def synth_count(cfg_id, scale=1.0, seed=20261203):
    """Particles in synth(cfg_id, scale, seed), without generating them."""
    n = _synth_lib().synth_count(cfg_id, scale, seed)
    if n < 0:
        raise ValueError("bad synthetic workload %r scale %r" % (cfg_id, scale))
    return int(n)


def synth(cfg_id, scale=1.0, seed=20261203):
    """Seeded synthetic snapshot (see csrc/synth.c).  Returns
    (particles, box_size, particle_mass, n_structures)."""
    _synth_lib()
    n = _synth.synth_count(cfg_id, scale, seed)
    if n < 0:
        raise ValueError("bad synthetic workload %r scale %r" % (cfg_id, scale))
    p = np.zeros(n, PARTICLE)
    box = np.zeros(1)
    mp = np.zeros(1)
    nh = np.zeros(1, np.int64)
    rc = _synth.synth_generate(cfg_id, scale, seed, p.ctypes.data, n, box.ctypes.data,
                               mp.ctypes.data, nh.ctypes.data)
    if rc:
        raise ValueError("synthetic generator failed (%d)" % rc)
    return p, float(box[0]), float(mp[0]), int(nh[0])


def launch_count():
    """Kernels this library has launched in the process so far."""
    return int(lib().rsg_launch_count())


def profile_select(name):
    """Time every launch of kernels whose name contains `name` with CUDA events."""
    _check(lib().rsg_profile_select(name.encode() if name else b""))


def profile_read():
    """(launches, total device ms) of the selected kernel since the last read."""
    n = np.zeros(1, np.int64)
    t = np.zeros(1, np.float64)
    _check(lib().rsg_profile_read(n.ctypes.data, t.ctypes.data))
    return int(n[0]), float(t[0])


class GadgetOpts(C.Structure):
    """struct rsg_gadget_opts."""
    _fields_ = [("halo_particle_type", C.c_int64), ("skip_non_halo", C.c_int64),
                ("length_conversion", C.c_double), ("mass_conversion", C.c_double),
                ("rescale_particle_mass", C.c_int64), ("lightcone", C.c_int64),
                ("lgadget", C.c_int64)]


GADGET_CFG_FIELDS = ("om", "ol", "h0", "box_size", "total_particles", "scale_now",
                     "particle_mass", "avg_particle_spacing")


def read_gadget2(path, cfg, halo_particle_type=1, skip_non_halo=1, length_conversion=1.0,
                 mass_conversion=1e10, rescale_particle_mass=0, lightcone=0, lgadget=0):
    """One GADGET-2 file: (particles in file order, dict of the configuration
    values the header sets).  cfg supplies PARTICLE_MASS for a header
    without one."""
    st = config_struct(cfg)
    o = GadgetOpts(halo_particle_type, skip_non_halo, length_conversion, mass_conversion,
                   rescale_particle_mass, lightcone, lgadget)
    n = np.zeros(1, np.int64)
    _check(lib().rsg_read_gadget2(os.fsencode(path), C.byref(o), C.byref(st), None, 0,
                                  n.ctypes.data))
    pa = np.zeros(int(n[0]), PARTICLE)
    st = config_struct(cfg)
    _check(lib().rsg_read_gadget2(os.fsencode(path), C.byref(o), C.byref(st),
                                  pa.ctypes.data if len(pa) else None, len(pa), n.ctypes.data))
    return pa, {k: getattr(st, k) for k in GADGET_CFG_FIELDS}


def read_gadget2_device(path, cfg, **opts):
    """read_gadget2 with the records left on the device: (torch uint8 CUDA
    tensor of n PARTICLE records, dict of the header's configuration values);
    the tensor's data pointer feeds DevicePath.run and sort_by_id_device."""
    import torch
    st = config_struct(cfg)
    o = GadgetOpts(opts.get("halo_particle_type", 1), opts.get("skip_non_halo", 1),
                   opts.get("length_conversion", 1.0), opts.get("mass_conversion", 1e10),
                   opts.get("rescale_particle_mass", 0), opts.get("lightcone", 0),
                   opts.get("lgadget", 0))
    n = np.zeros(1, np.int64)
    _check(lib().rsg_read_gadget2_device(os.fsencode(path), C.byref(o), C.byref(st), None, 0,
                                         n.ctypes.data))
    out = torch.empty(max(int(n[0]), 1) * PARTICLE.itemsize, dtype=torch.uint8, device="cuda")
    torch.cuda.synchronize()  # the library works on its own stream
    st = config_struct(cfg)
    _check(lib().rsg_read_gadget2_device(os.fsencode(path), C.byref(o), C.byref(st),
                                         out.data_ptr(), int(n[0]), n.ctypes.data))
    return out[: int(n[0]) * PARTICLE.itemsize], {k: getattr(st, k) for k in GADGET_CFG_FIELDS}


INTERNAL_CFG_FIELDS = ("scale_now", "om", "ol", "h0", "box_size", "particle_mass")


def read_internal(path, cfg):
    """One file of the reference's internal particle format: (particles,
    dict of the configuration values its header sets)."""
    st = config_struct(cfg)
    n = np.zeros(1, np.int64)
    _check(lib().rsg_read_internal(os.fsencode(path), C.byref(st), None, 0, n.ctypes.data))
    pa = np.zeros(int(n[0]), PARTICLE)
    _check(lib().rsg_read_internal(os.fsencode(path), C.byref(st),
                                   pa.ctypes.data if len(pa) else None, len(pa), n.ctypes.data))
    return pa, {k: getattr(st, k) for k in INTERNAL_CFG_FIELDS}


def read_internal_device(path, cfg):
    """read_internal with the records left on the device: (torch uint8 CUDA
    tensor of PARTICLE records, dict of the header's values)."""
    import torch
    st = config_struct(cfg)
    n = np.zeros(1, np.int64)
    _check(lib().rsg_read_internal_device(os.fsencode(path), C.byref(st), None, 0,
                                          n.ctypes.data))
    out = torch.empty(max(int(n[0]), 1) * PARTICLE.itemsize, dtype=torch.uint8, device="cuda")
    torch.cuda.synchronize()  # the copies run on the library's streams
    _check(lib().rsg_read_internal_device(os.fsencode(path), C.byref(st), out.data_ptr(),
                                          int(n[0]), n.ctypes.data))
    return out[: int(n[0]) * PARTICLE.itemsize], {k: getattr(st, k) for k in INTERNAL_CFG_FIELDS}


def write_internal(path, parts, cfg, snap=0, chunk=0):
    """The particles in the reference's internal format
    (output_particles_internal with fraction 1)."""
    pa = np.ascontiguousarray(parts, dtype=PARTICLE)
    st = config_struct(cfg)
    _check(lib().rsg_write_internal(os.fsencode(path), pa.ctypes.data if len(pa) else None,
                                    len(pa), snap, chunk, C.byref(st)))


def sort_by_id_device(d_parts, n=None):
    """Device-resident records (a torch CUDA tensor of PARTICLE bytes, or a
    device pointer with n) sorted by id in place."""
    if n is None:
        n = d_parts.numel() // PARTICLE.itemsize
    ptr = d_parts if isinstance(d_parts, int) else d_parts.data_ptr()
    if not isinstance(d_parts, int):
        import torch
        torch.cuda.synchronize()
    _check(lib().rsg_sort_particles_by_id_device(ptr if n else None, n))


def sort_by_id(parts, inplace=False):
    """The particles sorted by id on the device: a new array, or with
    inplace=True the caller's (contiguous PARTICLE) array itself, as the
    reference's std::sort sorts p."""
    if inplace:
        if not (isinstance(parts, np.ndarray) and parts.dtype == PARTICLE
                and parts.flags.c_contiguous and parts.flags.writeable):
            raise ValueError("inplace needs a writeable contiguous PARTICLE array")
        pa = parts
    else:
        pa = np.array(parts, dtype=PARTICLE, copy=True)
    _check(lib().rsg_sort_particles_by_id(pa.ctypes.data if len(pa) else None, len(pa)))
    return pa


class CatalogOpts(C.Structure):
    """struct rsg_catalog: options of one catalogue file."""
    _fields_ = [("id_offset", C.c_int64), ("snap", C.c_int64), ("chunk", C.c_int64),
                ("bounds", C.c_void_p), ("num_p", C.c_int64), ("strict_so_masses", C.c_int64)]


def _catalog_opts(id_offset, snap, chunk, bounds, num_p, strict_so_masses):
    b = None
    if bounds is not None:
        b = np.ascontiguousarray(bounds, dtype=np.float32)
        assert b.shape == (6,)
    o = CatalogOpts(id_offset, snap, chunk, b.ctypes.data if b is not None else None, num_p,
                    strict_so_masses)
    return o, b


def should_print(halos, cfg, bounds=None):
    """_should_print of every halo (src/io/meta_io.c:266-286), as a bool array."""
    st = setup_config(cfg)
    h = np.ascontiguousarray(halos, dtype=HALO)
    o, b = _catalog_opts(0, 0, 0, bounds, 0, 0)
    bp = b.ctypes.data if b is not None else None
    out = np.zeros(len(h), bool)
    for i in range(len(h)):
        rc = lib().rsg_should_print(h[i:i + 1].ctypes.data, bp, C.byref(st))
        if rc < 0:
            _check(rc)
        out[i] = rc == 1
    n = lib().rsg_count_halos_to_print(h.ctypes.data, len(h), bp, C.byref(st))
    if n < 0:
        _check(int(n))
    assert n == int(out.sum())
    return out


def write_ascii(path, halos, extra, cfg, id_offset=0, bounds=None, num_p=0,
                strict_so_masses=0):
    """The out_<snap>.list catalogue of the printable halos (output_ascii)."""
    st = setup_config(cfg)
    h = np.ascontiguousarray(halos, dtype=HALO)
    e = np.ascontiguousarray(extra, dtype=EXTRA)
    assert len(h) == len(e)
    o, b = _catalog_opts(id_offset, 0, 0, bounds, num_p, strict_so_masses)
    _check(lib().rsg_write_ascii(os.fsencode(path), h.ctypes.data, e.ctypes.data, len(h),
                                 C.byref(o), C.byref(st)))


def write_particles(path, halos, extra, parts, cfg, id_offset=0, bounds=None, num_p=0,
                    strict_so_masses=0, unfiltered=0, every_n=0):
    """The halos_<snap>.<chunk>.particles table (output_full_particles);
    returns the ids it assigns to the halos (-1 for the unprintable ones)."""
    st = setup_config(cfg)
    h = np.ascontiguousarray(halos, dtype=HALO)
    e = np.ascontiguousarray(extra, dtype=EXTRA)
    pa = np.ascontiguousarray(parts, dtype=PARTICLE)
    assert len(h) == len(e)
    o, b = _catalog_opts(id_offset, 0, 0, bounds, num_p, strict_so_masses)
    ids = np.zeros(max(len(h), 1), np.int64)
    _check(lib().rsg_write_particles(os.fsencode(path), h.ctypes.data, e.ctypes.data, len(h),
                                     pa.ctypes.data if len(pa) else None, len(pa), C.byref(o),
                                     unfiltered, every_n, C.byref(st), ids.ctypes.data))
    return ids[:len(h)]


class BinaryHeader(C.Structure):
    """struct rsg_binary_header (the reference's binary_output_header)."""
    _fields_ = [("magic", C.c_uint64), ("snap", C.c_int64), ("chunk", C.c_int64),
                ("scale", C.c_float), ("Om", C.c_float), ("Ol", C.c_float), ("h0", C.c_float),
                ("bounds", C.c_float * 6), ("num_halos", C.c_int64),
                ("num_particles", C.c_int64), ("box_size", C.c_float),
                ("particle_mass", C.c_float), ("particle_type", C.c_int64),
                ("format_revision", C.c_int32), ("rockstar_version", C.c_char * 12),
                ("add_flag", C.c_int32), ("unused", C.c_char * 140)]


def read_binary(path, cfg):
    """A halo catalogue file (halos_<snap>.<chunk>.bin) read back, as
    load_binary_halos does: (header, halos, particle ids, dict of the
    configuration values the header sets)."""
    hdr = BinaryHeader()
    st = config_struct(cfg)
    _check(lib().rsg_read_binary(os.fsencode(path), C.byref(hdr), C.byref(st), None, 0, None, 0))
    h = np.zeros(hdr.num_halos, HALO)
    ids = np.zeros(hdr.num_particles, np.int64)
    _check(lib().rsg_read_binary(os.fsencode(path), C.byref(hdr), C.byref(st),
                                 h.ctypes.data if len(h) else None, len(h),
                                 ids.ctypes.data if len(ids) else None, len(ids)))
    return hdr, h, ids, {k: getattr(st, k) for k in INTERNAL_CFG_FIELDS}


def write_binary(path, halos, parts, cfg, id_offset=0, snap=0, chunk=0, bounds=None):
    """The halos_<snap>.<chunk>.bin catalogue: header, printable halos, the
    ids of their particles (output_binary)."""
    st = setup_config(cfg)
    h = np.ascontiguousarray(halos, dtype=HALO)
    pa = np.ascontiguousarray(parts, dtype=PARTICLE)
    o, b = _catalog_opts(id_offset, snap, chunk, bounds, 0, 0)
    _check(lib().rsg_write_binary(os.fsencode(path), h.ctypes.data, len(h), pa.ctypes.data,
                                  len(pa), C.byref(o), C.byref(st)))


STAT_NAMES = ("particles", "groups", "halos", "pot_records", "kept_big", "kept_small",
              "halos_big", "halos_small", "dense", "dense_pairs", "items_6d", "samples_6d",
              "near_6d", "seed_steps")


def last_stats():
    """Work counters of the last call on this thread (rsg_last_stats)."""
    v = np.zeros(len(STAT_NAMES), np.int64)
    _check(lib().rsg_last_stats(v.ctypes.data, len(v)))
    return dict(zip(STAT_NAMES, (int(x) for x in v)))


def profile_table():
    """Per-kernel "name\tlaunches\ttotal_ms" lines of the launches timed since
    profile_select (largest first); clears them."""
    buf = C.create_string_buffer(1 << 20)
    need = lib().rsg_profile_table(buf, 1 << 20)
    if need < 0:
        _check(int(need))
    return buf.value.decode()


NOALLOC_MAX_PARTICLES = 65536
NOALLOC_SCRATCH_BYTES = 64 << 20


def rockstar_fof_noalloc(d_in, n, cfg_struct, d_out, d_off, d_sz, max_fofs, stream=0):
    """rsg_rockstar_fof_noalloc on caller-owned device buffers (raw device
    pointers; cfg_struct from setup_config).  Returns (num_p, num_fofs)."""
    np_out = np.zeros(1, np.int64)
    nf = np.zeros(1, np.int64)
    _check(lib().rsg_rockstar_fof_noalloc(d_in, n, C.byref(cfg_struct), d_out,
                                          np_out.ctypes.data, d_off, d_sz, max_fofs,
                                          nf.ctypes.data, stream))
    return int(np_out[0]), int(nf[0])


class DevicePath:
    """The full hot path on device-resident arrays (torch CUDA tensors or raw
    device pointers): rsg_path_device."""

    def __init__(self, n, cfg, halo_cap=None, batched=False):
        import torch
        self.n = n
        self.batched = 1 if batched else 0
        self.st = setup_config(cfg)
        self.halo_cap = halo_cap or (n // 16 + 65536)
        self.out = torch.empty(n * PARTICLE.itemsize, dtype=torch.uint8, device="cuda")
        self.halos = torch.empty(self.halo_cap * HALO.itemsize, dtype=torch.uint8, device="cuda")
        self.extra = torch.empty(self.halo_cap * EXTRA.itemsize, dtype=torch.uint8, device="cuda")
        self._np = np.zeros(1, np.int64)
        self._nf = np.zeros(1, np.int64)
        self._nh = np.zeros(1, np.int64)

    def run(self, d_in_ptr):
        _check(lib().rsg_path_device(d_in_ptr, self.n, C.byref(self.st), self.out.data_ptr(),
                                     self._np.ctypes.data, self._nf.ctypes.data,
                                     self.halos.data_ptr(), self.extra.data_ptr(),
                                     self.halo_cap, self._nh.ctypes.data, self.batched))
        return int(self._np[0]), int(self._nf[0]), int(self._nh[0])

    def results(self):
        """(particles, halos, extra) of the last run, copied to the host."""
        n, nh = int(self._np[0]), int(self._nh[0])
        parts = self.out[: n * PARTICLE.itemsize].cpu().numpy().view(PARTICLE).copy()
        h = self.halos[: nh * HALO.itemsize].cpu().numpy().view(HALO).copy()
        e = self.extra[: nh * EXTRA.itemsize].cpu().numpy().view(EXTRA).copy()
        return parts, h, e
