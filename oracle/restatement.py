"""ctypes access to the C restatement (oracle/rockstar_oracle.c).

TEST INFRASTRUCTURE ONLY: imported by tests/, the smoke check and the CPU
baseline of bench.py.  build() compiles the restatement with the host C
compiler into oracle/_build/liboracle.so (no FMA contraction, so float
arithmetic matches the C source exactly).
"""
import ctypes as C
import os
import subprocess

import numpy as np

from . import layouts as L

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(HERE, "rockstar_oracle.c")
LIB = os.path.join(HERE, "_build", "liboracle.so")


def build(force=False):
    if not force and os.path.exists(LIB) and os.path.getmtime(LIB) >= os.path.getmtime(SRC):
        return LIB
    os.makedirs(os.path.dirname(LIB), exist_ok=True)
    tmp = LIB + ".tmp%d" % os.getpid()
    subprocess.check_call(["gcc", "-O3", "-std=c99", "-D_DEFAULT_SOURCE", "-ffp-contract=off",
                           "-fno-math-errno", "-fPIC", "-shared", "-o", tmp, SRC, "-lm"])
    os.replace(tmp, LIB)
    return LIB


class OCfg(C.Structure):
    _fields_ = [(k, C.c_double) for k in (
        "particle_mass", "box_size", "om", "ol", "h0", "w0", "wa",
        "fof_linking_length", "fof_fraction", "force_res", "force_res_phys_max",
        "scale_now", "initial_metric_scaling", "include_host_potential_ratio",
        "unbound_threshold")] + [(k, C.c_int64) for k in (
            "min_halo_particles", "min_halo_output_size", "bound_props",
            "shape_iterations", "weighted_shapes", "exact_ll_calc",
            "total_particles")]


_lib = None


def lib():
    global _lib
    if _lib is None:
        h = C.CDLL(build())
        vp, i64 = C.c_void_p, C.c_int64
        h.oracle_setup.argtypes = [C.POINTER(OCfg)]
        h.oracle_avg_spacing.restype = C.c_double
        h.oracle_thresholds.argtypes = [vp]
        h.oracle_fof.restype = i64
        h.oracle_fof.argtypes = [vp, vp, vp, vp]
        h.oracle_free.argtypes = [vp]
        h.oracle_find_subs.restype = i64
        h.oracle_find_subs.argtypes = [vp, vp, vp, i64, vp, vp]
        h.oracle_compute_potential.argtypes = [vp, i64]
        h.oracle_kinetic_energy.argtypes = [vp, i64, vp, vp, C.c_float]
        h.oracle_should_print.argtypes = [vp, vp]
        h.oracle_write_ascii.argtypes = [C.c_char_p, vp, vp, i64, i64, vp, i64, i64]
        h.oracle_write_binary.argtypes = [C.c_char_p, vp, i64, vp, i64, i64, i64, vp]
        h.oracle_write_particles.argtypes = [C.c_char_p, vp, vp, i64, vp, i64, vp, i64, i64, i64,
                                             i64, vp]
        h.oracle_tree_order.argtypes = [vp, i64, C.c_int, C.c_int]
        h.oracle_descendants.argtypes = [vp, i64, vp, vp, i64, vp, vp]
        h.oracle_hierarchy.restype = i64
        h.oracle_hierarchy.argtypes = [vp, vp, vp, i64]
        _lib = h
    return _lib


def setup(cfg):
    q = OCfg(**{k: getattr(cfg, k) for k, _ in OCfg._fields_})
    lib().oracle_setup(C.byref(q))
    return lib().oracle_avg_spacing()


def thresholds():
    out = np.zeros(8, np.float64)
    lib().oracle_thresholds(out.ctypes.data)
    return out


def _take(ptr, n, dtype):
    if n == 0:
        lib().oracle_free(ptr)
        return np.zeros(0, dtype)
    buf = (C.c_char * (n * dtype.itemsize)).from_address(ptr)
    out = np.frombuffer(bytes(buf), dtype=dtype).copy()
    lib().oracle_free(ptr)
    return out


def fof(parts):
    """rockstar(NULL, 1): returns (permuted particles, offsets, sizes)."""
    pa = np.array(parts, dtype=L.PARTICLE, copy=True)
    n = np.array([len(pa)], np.int64)
    po, ps = C.c_void_p(), C.c_void_p()
    nf = lib().oracle_fof(pa.ctypes.data, n.ctypes.data, C.byref(po), C.byref(ps))
    off = _take(po.value, nf, np.dtype(np.int64))
    sz = _take(ps.value, nf, np.dtype(np.int64))
    return pa[:n[0]].copy(), off, sz


def find_subs(parts, off, sz):
    """find_subs over every group in order.  Returns (particles, halos, extra)."""
    pa = np.array(parts, dtype=L.PARTICLE, copy=True)
    off = np.ascontiguousarray(off, np.int64)
    sz = np.ascontiguousarray(sz, np.int64)
    hp, ep = C.c_void_p(), C.c_void_p()
    nh = lib().oracle_find_subs(pa.ctypes.data, off.ctypes.data, sz.ctypes.data, len(sz),
                                C.byref(hp), C.byref(ep))
    return pa, _take(hp.value, nh, L.HALO), _take(ep.value, nh, L.EXTRA)


def compute_potential(po):
    po = np.array(po, dtype=L.POTENTIAL, copy=True)
    lib().oracle_compute_potential(po.ctypes.data, len(po))
    return po


def tree_order(parts, dim, leaf):
    """The kd-tree build permutation of `parts` (fast3tree_init)."""
    pa = np.array(parts, dtype=L.PARTICLE, copy=True)
    lib().oracle_tree_order(pa.ctypes.data, len(pa), dim, leaf)
    return pa


def hierarchy():
    """(level, size, target_r) of every 6D FOF call of the last find_subs."""
    cap = 1 << 22
    lv = np.zeros(cap, np.int64)
    n = np.zeros(cap, np.int64)
    tr = np.zeros(cap, np.float32)
    k = min(lib().oracle_hierarchy(lv.ctypes.data, n.ctypes.data, tr.ctypes.data, cap), cap)
    return lv[:k].copy(), n[:k].copy(), tr[:k].copy()


def kinetic_energy(po, vel_cen, pos_cen, scale_now):
    """compute_kinetic_energy on a copy of the records (cosmology from setup)."""
    po = np.array(po, dtype=L.POTENTIAL, copy=True)
    vc = np.ascontiguousarray(vel_cen, np.float32)
    pc = np.ascontiguousarray(pos_cen, np.float32)
    lib().oracle_kinetic_energy(po.ctypes.data, len(po), vc.ctypes.data, pc.ctypes.data,
                                C.c_float(scale_now))
    return po


def _bounds(bounds):
    if bounds is None:
        return None, None
    b = np.ascontiguousarray(bounds, dtype=np.float32)
    return b, b.ctypes.data


def should_print(halos, bounds=None):
    """_should_print of every halo (after setup())."""
    h = np.ascontiguousarray(halos, dtype=L.HALO)
    b, bp = _bounds(bounds)
    return np.array([lib().oracle_should_print(h[i:i + 1].ctypes.data, bp) == 1
                     for i in range(len(h))], bool)


def write_ascii(path, halos, extra, id_offset=0, bounds=None, num_p=0, strict_so_masses=0):
    h = np.ascontiguousarray(halos, dtype=L.HALO)
    e = np.ascontiguousarray(extra, dtype=L.EXTRA)
    b, bp = _bounds(bounds)
    assert lib().oracle_write_ascii(os.fsencode(path), h.ctypes.data, e.ctypes.data, len(h),
                                    id_offset, bp, num_p, strict_so_masses) == 0


def write_particles(path, halos, extra, parts, id_offset=0, bounds=None, num_p=0,
                    strict_so_masses=0, unfiltered=0, every_n=0):
    """output_full_particles to `path`; returns the ids it assigns."""
    h = np.ascontiguousarray(halos, dtype=L.HALO)
    e = np.ascontiguousarray(extra, dtype=L.EXTRA)
    pa = np.ascontiguousarray(parts, dtype=L.PARTICLE)
    b, bp = _bounds(bounds)
    ids = np.zeros(max(len(h), 1), np.int64)
    assert lib().oracle_write_particles(os.fsencode(path), h.ctypes.data, e.ctypes.data, len(h),
                                        pa.ctypes.data, id_offset, bp, num_p, strict_so_masses,
                                        unfiltered, every_n, ids.ctypes.data) == 0
    return ids[:len(h)]


def write_binary(path, halos, parts, id_offset=0, snap=0, chunk=0, bounds=None):
    h = np.ascontiguousarray(halos, dtype=L.HALO)
    pa = np.ascontiguousarray(parts, dtype=L.PARTICLE)
    b, bp = _bounds(bounds)
    assert lib().oracle_write_binary(os.fsencode(path), h.ctypes.data, len(h), pa.ctypes.data,
                                     id_offset, snap, chunk, bp) == 0


def descendants(halos1, part1, halos2, part2):
    """The merger tree's descendant of every halo of halos1 (ids in part1)
    among halos2 (ids in part2), by the rule of src/merger.c:45-101."""
    h1 = np.ascontiguousarray(halos1, dtype=L.HALO)
    h2 = np.ascontiguousarray(halos2, dtype=L.HALO)
    p1 = np.ascontiguousarray(part1, dtype=np.int64)
    p2 = np.ascontiguousarray(part2, dtype=np.int64)
    out = np.zeros(max(len(h1), 1), np.int64)
    lib().oracle_descendants(h1.ctypes.data, len(h1), p1.ctypes.data, h2.ctypes.data, len(h2),
                             p2.ctypes.data, out.ctypes.data)
    return out[:len(h1)]
