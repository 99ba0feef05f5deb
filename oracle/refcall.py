"""ctypes access to the reference's own hot path compiled as a test oracle.

TEST INFRASTRUCTURE ONLY.  oracle/_ref/libref_rockstar.so is built by
oracle/ref/Makefile from the unmodified reference sources; it exists only
where the reference checkout is present (the development container).  The
tests use it to produce golden fixtures and to pin the C restatement in
oracle/rockstar_oracle.c; the product never imports this module.
"""
import ctypes as C
import os

import numpy as np

from . import layouts as L

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "_ref", "libref_rockstar.so")


class RefParams(C.Structure):
    _fields_ = [(k, C.c_double) for k in (
        "particle_mass", "box_size", "om", "ol", "h0", "w0", "wa",
        "fof_linking_length", "fof_fraction", "force_res", "force_res_phys_max",
        "scale_now", "initial_metric_scaling", "include_host_potential_ratio",
        "unbound_threshold")] + [(k, C.c_int64) for k in (
            "min_halo_particles", "min_halo_output_size", "bound_props",
            "shape_iterations", "weighted_shapes", "exact_ll_calc",
            "total_particles")]


def available():
    return os.path.exists(LIB)


_lib = None


def lib():
    global _lib
    if _lib is None:
        h = C.CDLL(LIB)
        vp, i64 = C.c_void_p, C.c_int64
        h.ref_setup.argtypes = [C.POINTER(RefParams)]
        h.ref_avg_particle_spacing.restype = C.c_double
        h.ref_particle_mass.restype = C.c_double
        h.ref_thresholds.argtypes = [vp]
        h.ref_sizeof_halo.restype = i64
        h.ref_sizeof_extra.restype = i64
        h.ref_sizeof_potential.restype = i64
        h.ref_fof.restype = i64
        h.ref_fof.argtypes = [vp, i64, vp, vp, vp, vp, i64]
        h.ref_find_subs.restype = i64
        h.ref_find_subs.argtypes = [vp, i64, vp, vp, i64, vp, vp, i64, C.c_int]
        h.ref_compute_potential.argtypes = [vp, i64]
        h.ref_compute_kinetic_energy.argtypes = [vp, i64, vp, vp, C.c_float]
        h.ref_time_path.restype = i64
        h.ref_time_path.argtypes = [vp, i64, C.c_int, vp, vp]
        h.ref_output_binary.argtypes = [C.c_char_p, vp, i64, vp, i64, i64, i64, i64, vp]
        h.ref_output_particles_internal.argtypes = [C.c_char_p, vp, i64, i64, i64, vp]
        h.ref_load_internal.restype = i64
        h.ref_load_internal.argtypes = [C.c_char_p, vp, i64, vp]
        h.ref_descendants.argtypes = [vp, i64, vp, i64, vp, i64, vp, i64, vp]
        h.ref_load_binary.restype = i64
        h.ref_load_binary.argtypes = [C.c_char_p, vp, vp, i64, vp, i64, vp]
        h.ref_load_gadget2.restype = i64
        h.ref_load_gadget2.argtypes = [C.c_char_p, i64, i64, C.c_double, C.c_double, i64, i64,
                                       i64, C.c_double, vp, i64, vp]
        assert h.ref_sizeof_halo() == L.HALO.itemsize
        assert h.ref_sizeof_extra() == L.EXTRA.itemsize
        assert h.ref_sizeof_potential() == L.POTENTIAL.itemsize
        _lib = h
    return _lib


def setup(cfg):
    """cfg: a layouts.Config.  Applies it to the reference's config globals."""
    q = RefParams(
        particle_mass=cfg.particle_mass, box_size=cfg.box_size, om=cfg.om,
        ol=cfg.ol, h0=cfg.h0, w0=cfg.w0, wa=cfg.wa,
        fof_linking_length=cfg.fof_linking_length, fof_fraction=cfg.fof_fraction,
        force_res=cfg.force_res, force_res_phys_max=cfg.force_res_phys_max,
        scale_now=cfg.scale_now, initial_metric_scaling=cfg.initial_metric_scaling,
        include_host_potential_ratio=cfg.include_host_potential_ratio,
        unbound_threshold=cfg.unbound_threshold,
        min_halo_particles=cfg.min_halo_particles,
        min_halo_output_size=cfg.min_halo_output_size, bound_props=cfg.bound_props,
        shape_iterations=cfg.shape_iterations, weighted_shapes=cfg.weighted_shapes,
        exact_ll_calc=cfg.exact_ll_calc, total_particles=cfg.total_particles)
    lib().ref_setup(C.byref(q))
    return lib().ref_avg_particle_spacing()


def thresholds():
    out = np.zeros(8, np.float64)
    lib().ref_thresholds(out.ctypes.data)
    return out


def fof(parts):
    """rockstar(NULL, 1) on an id-sorted particle array.
    Returns (permuted particles, offsets, sizes)."""
    parts = np.ascontiguousarray(parts, dtype=L.PARTICLE)
    n = len(parts)
    out = np.zeros(n, L.PARTICLE)
    nout = np.zeros(1, np.int64)
    cap = n // 2 + 16
    off = np.zeros(cap, np.int64)
    sz = np.zeros(cap, np.int64)
    nf = lib().ref_fof(parts.ctypes.data, n, out.ctypes.data, nout.ctypes.data,
                       off.ctypes.data, sz.ctypes.data, cap)
    return out[:nout[0]].copy(), off[:nf].copy(), sz[:nf].copy()


def find_subs(parts, off, sz, nthreads=1):
    """find_subs over every group (in place on a copy).  Returns
    (particles after find_subs, halos, extra_info)."""
    parts = np.array(parts, dtype=L.PARTICLE, copy=True)
    off = np.ascontiguousarray(off, np.int64)
    sz = np.ascontiguousarray(sz, np.int64)
    cap = int(sz.sum()) // 5 + 64 * len(sz) + 1000
    h = np.zeros(cap, L.HALO)
    e = np.zeros(cap, L.EXTRA)
    nh = lib().ref_find_subs(parts.ctypes.data, len(parts), off.ctypes.data,
                             sz.ctypes.data, len(sz), h.ctypes.data, e.ctypes.data,
                             cap, nthreads)
    if nh < 0:
        raise RuntimeError("halo capacity exceeded")
    return parts, h[:nh].copy(), e[:nh].copy()


def compute_potential(po):
    po = np.array(po, dtype=L.POTENTIAL, copy=True)
    lib().ref_compute_potential(po.ctypes.data, len(po))
    return po


def time_path(parts, nthreads):
    parts = np.ascontiguousarray(parts, dtype=L.PARTICLE)
    tf = np.zeros(1)
    ts = np.zeros(1)
    nh = lib().ref_time_path(parts.ctypes.data, len(parts), nthreads,
                             tf.ctypes.data, ts.ctypes.data)
    return float(tf[0]), float(ts[0]), int(nh)


def output_binary(path, halos, parts, id_offset=0, snap=0, chunk=0, bounds=None):
    """The reference's output_binary (src/io/io_internal.c:118-186) writing
    `halos` and the ids of their particles in `parts` to `path` (after
    setup())."""
    h = np.array(halos, dtype=L.HALO, copy=True)
    pa = np.ascontiguousarray(parts, dtype=L.PARTICLE)
    b = None if bounds is None else np.ascontiguousarray(bounds, dtype=np.float32)
    lib().ref_output_binary(os.fsencode(path), h.ctypes.data, len(h), pa.ctypes.data, len(pa),
                            id_offset, snap, chunk, b.ctypes.data if b is not None else None)


INTERNAL_CFG_FIELDS = ("scale_now", "om", "ol", "h0", "box_size", "particle_mass")


def output_particles_internal(path, parts, cfg, snap=0, chunk=0):
    """The reference's output_particles_internal(snap, chunk, 1)
    (src/io/io_internal.c:52-83) writing `parts` to `path` with the
    configuration values of the dict `cfg` (INTERNAL_CFG_FIELDS)."""
    pa = np.ascontiguousarray(parts, dtype=L.PARTICLE)
    c = np.array([cfg[k] for k in INTERNAL_CFG_FIELDS], np.float64)
    lib().ref_output_particles_internal(os.fsencode(path), pa.ctypes.data, len(pa), snap,
                                        chunk, c.ctypes.data)


def load_binary(path, max_h=1 << 20, max_ids=1 << 24):
    """The reference's load_binary_halos on one catalogue file: (the 256
    header bytes, halos, particle ids, dict of the configuration values it
    sets)."""
    hdr = np.zeros(256, np.uint8)
    h = np.zeros(max_h, L.HALO)
    ids = np.zeros(max_ids, np.int64)
    cfg = np.zeros(6, np.float64)
    nh = lib().ref_load_binary(os.fsencode(path), hdr.ctypes.data, h.ctypes.data, max_h,
                               ids.ctypes.data, max_ids, cfg.ctypes.data)
    nids = int(hdr[72:80].view(np.int64)[0])
    assert nh <= max_h and nids <= max_ids
    return hdr, h[:nh].copy(), ids[:nids].copy(), dict(zip(INTERNAL_CFG_FIELDS, cfg.tolist()))


def load_internal(path, max_p=1 << 22):
    """The reference's load_particles_internal on one file: (particles, dict
    of the configuration values read_binary_header_config sets)."""
    out = np.zeros(max_p, L.PARTICLE)
    cfg = np.zeros(6, np.float64)
    n = lib().ref_load_internal(os.fsencode(path), out.ctypes.data, max_p, cfg.ctypes.data)
    assert n <= max_p
    return out[:n].copy(), dict(zip(INTERNAL_CFG_FIELDS, cfg.tolist()))


GADGET_CFG_FIELDS = ("om", "ol", "h0", "box_size", "total_particles", "scale_now",
                     "particle_mass", "avg_particle_spacing")


def load_gadget2(path, halo_particle_type=1, skip_non_halo=1, length_conversion=1.0,
                 mass_conversion=1e10, rescale_particle_mass=0, lightcone=0, lgadget=0,
                 particle_mass=0.0, max_p=1 << 22):
    """The reference's load_particles_gadget2 on one file: (particles in file
    order, dict of the configuration values it sets)."""
    out = np.zeros(max_p, L.PARTICLE)
    cfg = np.zeros(8, np.float64)
    n = lib().ref_load_gadget2(os.fsencode(path), halo_particle_type, skip_non_halo,
                               length_conversion, mass_conversion, rescale_particle_mass,
                               lightcone, lgadget, particle_mass, out.ctypes.data, max_p,
                               cfg.ctypes.data)
    assert n <= max_p
    return out[:n].copy(), dict(zip(GADGET_CFG_FIELDS, cfg.tolist()))


def descendants(halos1, part1, halos2, part2):
    """The reference's merger-tree descendants (src/merger.c:45-101) of
    halos1 (ids in part1) among halos2 (ids in part2)."""
    h1 = np.ascontiguousarray(halos1, dtype=L.HALO)
    h2 = np.ascontiguousarray(halos2, dtype=L.HALO)
    p1 = np.ascontiguousarray(part1, dtype=np.int64)
    p2 = np.ascontiguousarray(part2, dtype=np.int64)
    out = np.zeros(max(len(h1), 1), np.int64)
    lib().ref_descendants(h1.ctypes.data, len(h1), p1.ctypes.data, len(p1), h2.ctypes.data,
                          len(h2), p2.ctypes.data, len(p2), out.ctypes.data)
    return out[:len(h1)]
