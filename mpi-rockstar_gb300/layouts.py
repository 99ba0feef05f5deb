"""numpy dtypes of the C-ABI records and the hot-path configuration.

Layouts equal the reference's: src/particle.h:5-8 (32 B), src/halo.h:8-35
with OUTPUT_RVMAX/OUTPUT_NFW_CHI2/OUTPUT_INERTIA_TENSOR (312 B),
src/halo.h:37-41 (48 B), src/potential.h:7-21 (48 B).
"""
import ctypes as C
from dataclasses import dataclass, fields

import numpy as np

PARTICLE = np.dtype([("id", "<i8"), ("pos", "<f4", (6,))])
_SCALARS = ["m", "r", "child_r", "vmax_r", "mgrav", "vmax", "rvmax", "rs", "klypin_rs", "vrms"]
HALO = np.dtype(
    [("id", "<i8"), ("pos", "<f4", (6,)), ("corevel", "<f4", (3,)), ("bulkvel", "<f4", (3,))]
    + [(k, "<f4") for k in _SCALARS]
    + [("J", "<f4", (3,)), ("energy", "<f4"), ("spin", "<f4"), ("alt_m", "<f4", (4,)),
       ("Xoff", "<f4"), ("Voff", "<f4"), ("b_to_a", "<f4"), ("c_to_a", "<f4"),
       ("A", "<f4", (3,)), ("b_to_a2", "<f4"), ("c_to_a2", "<f4"), ("A2", "<f4", (3,)),
       ("bullock_spin", "<f4"), ("kin_to_pot", "<f4"), ("m_pe_b", "<f4"), ("m_pe_d", "<f4"),
       ("halfmass_radius", "<f4")]
    + [(k, "<i8") for k in ("num_p", "num_child_particles", "p_start", "desc", "flags",
                            "n_core")]
    + [("min_pos_err", "<f4"), ("min_vel_err", "<f4"), ("min_bulkvel_err", "<f4"),
       ("inertia_tensor", "<f4", (6,)), ("inertia_tensor2", "<f4", (6,)), ("chi2", "<f4")])
EXTRA = np.dtype([("child", "<i8"), ("next_cochild", "<i8"), ("prev_cochild", "<i8"),
                  ("sub_of", "<i8"), ("ph", "<i8"), ("max_metric", "<f4"), ("_pad", "<f4")])
POTENTIAL = np.dtype([("pos", "<f4", (6,)), ("r2", "<f4"), ("_pad", "<f4"), ("pe", "<f8"),
                      ("ke", "<f4"), ("flags", "<i4")])
assert PARTICLE.itemsize == 32 and HALO.itemsize == 312
assert EXTRA.itemsize == 48 and POTENTIAL.itemsize == 48


@dataclass
class Config:
    """Hot-path parameters (src/config.template.h names, lower case)."""
    particle_mass: float = 1e9
    box_size: float = 40.0
    om: float = 0.3
    ol: float = 0.7
    h0: float = 0.7
    w0: float = -1.0
    wa: float = 0.0
    fof_linking_length: float = 0.28
    fof_fraction: float = 0.7
    force_res: float = 0.003
    force_res_phys_max: float = 0.0
    scale_now: float = 1.0
    initial_metric_scaling: float = 1.0
    include_host_potential_ratio: float = 0.3
    unbound_threshold: float = 0.5
    min_halo_particles: int = 10
    min_halo_output_size: int = 20
    bound_props: int = 1
    shape_iterations: int = 10
    weighted_shapes: int = 1
    exact_ll_calc: int = 0
    total_particles: int = 0


class RsgConfig(C.Structure):
    _fields_ = ([(f.name, C.c_double if f.type is float else C.c_int64) for f in fields(Config)]
                + [("avg_particle_spacing", C.c_double),
                   ("particle_thresh_dens", C.c_double * 5),
                   ("particle_rvir_dens", C.c_double), ("particle_rvir_dens_z0", C.c_double),
                   ("dynamical_time", C.c_double), ("min_dens_index", C.c_int64)])


def config_struct(cfg):
    return RsgConfig(**{f.name: getattr(cfg, f.name) for f in fields(Config)})
