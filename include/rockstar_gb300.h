/* C ABI of the GB300 halo-finding hot path.
 *
 * Every entry point is extern "C" and takes plain pointers and sizes.  The
 * record layouts below are byte-for-byte those of the reference build
 * (gcc, -DOUTPUT_RVMAX -DOUTPUT_NFW_CHI2 -DOUTPUT_INERTIA_TENSOR), so arrays
 * can be passed between this library and code compiled against the
 * reference headers without conversion:
 *   rsg_particle        == struct particle        (src/particle.h:5-8)
 *   rsg_fof             == struct fof             (src/fof.h:7-10)
 *   rsg_halo            == struct halo            (src/halo.h:8-35)
 *   rsg_extra_halo_info == struct extra_halo_info (src/halo.h:37-41)
 *   rsg_potential       == struct potential       (src/potential.h:7-21)
 * The names carry a prefix so this header can be included next to the
 * reference's own headers.
 *
 * Errors: functions return 0 on success and a negative RSG_ERR_* code on
 * failure; rsg_last_error() describes the last failure of the calling
 * thread.  Nothing here calls exit(); a drop-in shim maps a non-zero return
 * to the reference's rockstar_abort() (src/error.h:17-20).
 */
#ifndef ROCKSTAR_GB300_H
#define ROCKSTAR_GB300_H
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define RSG_OK 0
#define RSG_ERR_ARGS (-1)       /* bad arguments or capacity too small */
#define RSG_ERR_CUDA (-2)       /* a CUDA call failed */
#define RSG_ERR_NO_DEVICE (-3)  /* no usable GPU */
#define RSG_ERR_LIMIT (-4)      /* a bounded device loop hit its limit */
#define RSG_ERR_INPUT (-5)      /* non-finite particle data, or an input file the reader refuses */
#define RSG_ERR_BUSY (-6)       /* a call that shares fixed scratch is in progress */
#define RSG_ERR_IO (-7)         /* a file could not be opened, read or written */

struct rsg_particle { int64_t id; float pos[6]; };
struct rsg_fof { int64_t num_p; struct rsg_particle *particles; };
struct rsg_halo {
    int64_t id;
    float pos[6], corevel[3], bulkvel[3];
    float m, r, child_r, vmax_r, mgrav, vmax, rvmax, rs, klypin_rs, vrms, J[3],
        energy, spin, alt_m[4], Xoff, Voff, b_to_a, c_to_a, A[3], b_to_a2,
        c_to_a2, A2[3], bullock_spin, kin_to_pot, m_pe_b, m_pe_d,
        halfmass_radius;
    int64_t num_p, num_child_particles, p_start, desc, flags, n_core;
    float min_pos_err, min_vel_err, min_bulkvel_err;
    float inertia_tensor[6];
    float inertia_tensor2[6];
    float chi2;
};
struct rsg_extra_halo_info {
    int64_t child, next_cochild, prev_cochild;
    int64_t sub_of, ph;
    float max_metric;
};
struct rsg_potential {
    float pos[6], r2;
    double pe;
    float ke;
    int32_t flags;
};

/* Hot-path parameters, named after src/config.template.h.  Fields marked
 * (derived) are filled by rsg_config_setup(). */
struct rsg_config {
    double particle_mass;                /* PARTICLE_MASS (0: from box, Om, N) */
    double box_size;                     /* BOX_SIZE */
    double om, ol, h0, w0, wa;           /* Om, Ol, h0, W0, WA */
    double fof_linking_length;           /* FOF_LINKING_LENGTH */
    double fof_fraction;                 /* FOF_FRACTION */
    double force_res, force_res_phys_max;/* FORCE_RES, FORCE_RES_PHYS_MAX */
    double scale_now;                    /* SCALE_NOW */
    double initial_metric_scaling;       /* INITIAL_METRIC_SCALING */
    double include_host_potential_ratio; /* INCLUDE_HOST_POTENTIAL_RATIO */
    double unbound_threshold;            /* UNBOUND_THRESHOLD */
    int64_t min_halo_particles;          /* MIN_HALO_PARTICLES */
    int64_t min_halo_output_size;        /* MIN_HALO_OUTPUT_SIZE */
    int64_t bound_props;                 /* BOUND_PROPS */
    int64_t shape_iterations;            /* SHAPE_ITERATIONS */
    int64_t weighted_shapes;             /* WEIGHTED_SHAPES */
    int64_t exact_ll_calc;               /* EXACT_LL_CALC */
    int64_t total_particles;             /* TOTAL_PARTICLES */
    /* (derived) */
    double avg_particle_spacing;         /* AVG_PARTICLE_SPACING, src/config.c:24-25 */
    double particle_thresh_dens[5];      /* src/groupies.c:127-142 */
    double particle_rvir_dens, particle_rvir_dens_z0, dynamical_time;
    int64_t min_dens_index;
};

/* Library version and per-thread error text. */
int rsg_version(void);
const char *rsg_last_error(void);

/* Derives AVG_PARTICLE_SPACING, the effective FORCE_RES and the density
 * thresholds exactly as src/config.c:17-64, src/rockstar.c:58-61 and
 * src/groupies.c:97-142 do.  Host only. */
int rsg_config_setup(struct rsg_config *cfg);

/* 3D friends-of-friends: replaces rockstar(bounds = NULL, manual_subs = 1)
 * (src/rockstar.c:53-128).  p[0..*num_p) is permuted in place on return so
 * that every group is contiguous; duplicates (same position or id as the
 * previous particle in kd-tree order, src/rockstar.c:368-397) are removed
 * and *num_p shrinks accordingly.  Group i occupies
 * p[fof_offsets[i] .. fof_offsets[i] + fof_sizes[i]); groups of fewer than
 * MIN_HALO_PARTICLES are dropped as in src/fof.c:226-255.  The result is
 * the reference's byte for byte: the permutation of p (particles in no group
 * first, then one run per union-find label in ascending label order, groups
 * too small to keep included, as partition_sort_particles leaves them,
 * src/fof.c:184-224) and the groups in build_fullfofs order.  The union-find
 * labels are derived from the link lists in parallel and equal the ones the
 * reference's sequential linking produces. */
int rsg_rockstar_fof(struct rsg_particle *p, int64_t *num_p, const struct rsg_config *cfg,
                     int64_t *fof_offsets, int64_t *fof_sizes, int64_t max_fofs,
                     int64_t *num_fofs);

/* Substructure, particle assignment, potentials and halo properties for every
 * group: replaces the per-group calls find_subs(f, fofinfo, haloinfo)
 * (src/groupies.c:669-708) as the OpenMP loop of src/mpi_main.cpp:1363-1389
 * issues them, followed by copy_halos (src/mpi_main.cpp:1335-1361).
 * Groups i = 0..num_fofs-1 are p[fof_offsets[i] .. + fof_sizes[i]) and must
 * not overlap.  Each group's particles are permuted in place exactly as the
 * reference permutes f->particles (halos contiguous, sorted by distance at
 * the top level).  Halos of all groups are written in group order to
 * halos/extra (capacity max_halos); p_start is relative to p and the
 * child/sub_of links are indices into the output, as copy_halos leaves
 * them.  One call with num_fofs == 1 is the plain per-group drop-in. */
int rsg_find_subs(struct rsg_particle *p, int64_t num_p, const int64_t *fof_offsets,
                  const int64_t *fof_sizes, int64_t num_fofs, const struct rsg_config *cfg,
                  struct rsg_halo *halos, struct rsg_extra_halo_info *extra, int64_t max_halos,
                  int64_t *num_halos);

/* Batched form of rsg_find_subs (same arguments), replacing the same OpenMP
 * loop (src/mpi_main.cpp:1363-1389).  The 6D hierarchy is built as in the
 * plain form (the reference's union-find labels, particle order, samples and
 * quickselect); norm_sd, the Barnes-Hut node sums and the property scans of
 * halos above a few thousand records use parallel reductions, and the
 * potentials use the FP32 Kahan form (rsg_set_potential_form).  Halo
 * membership equals the reference's except where a one-ulp change of a
 * normalised coordinate or potential decides a link or a bound flag (the
 * pairs within 1e-6 of a linking length are counted, RSG_STAT_NEAR_6D);
 * properties agree to FP64 rounding except where a near-tie in one of the
 * reference's discrete choices goes the other way. */
int rsg_find_subs_batch(struct rsg_particle *p, int64_t num_p, const int64_t *fof_offsets,
                        const int64_t *fof_sizes, int64_t num_fofs, const struct rsg_config *cfg,
                        struct rsg_halo *halos, struct rsg_extra_halo_info *extra,
                        int64_t max_halos, int64_t *num_halos);

/* The whole hot path -- rockstar(NULL, 1) then find_subs over every group
 * -- on device-resident data (no host copies): d_in holds n id-sorted
 * particles, d_out receives the permuted particles (*num_p_out of them)
 * and d_halos/d_extra (capacity max_halos) the halos of all groups;
 * batched selects the rsg_find_subs_batch form for the substructure step.  Has no
 * single reference counterpart: it fuses the calls of src/mpi_main.cpp:1564
 * and :1363-1389 for callers that keep particles on the GPU. */
int rsg_path_device(const struct rsg_particle *d_in, int64_t n, const struct rsg_config *cfg,
                    struct rsg_particle *d_out, int64_t *num_p_out, int64_t *num_fofs,
                    struct rsg_halo *d_halos, struct rsg_extra_halo_info *d_extra,
                    int64_t max_halos, int64_t *num_halos, int32_t batched);

/* Barnes-Hut potentials of one particle set: replaces compute_potential(po,
 * num_po) (src/potential.h:23, src/potential.c:183-192) with PARTICLE_MASS
 * and FORCE_RES taken from cfg.  As in the reference, po is permuted in
 * place into the potential tree's order and every po[i].pe is overwritten.
 *   form 0: the reference's arithmetic (FP64 distances and sums),
 *           bit-identical potentials;
 *   form 1: the batched precision form (FP32 distances and 1/r, FP32
 *           Kahan-compensated sums; node sizes from parallel sums; the same
 *           tree and opening rule);
 *   form 2: form 1's terms summed in plain FP32 (no compensation);
 *   form 3: FP64 direct sum over all pairs, mp / max(r, FORCE_RES) (no
 *           reference counterpart: the precision reference; O(n^2)).
 * Every form permutes po the same way. */
int rsg_compute_potential(struct rsg_potential *po, int64_t num_po, const struct rsg_config *cfg,
                          int32_t form);

/* Kinetic energies of one particle set about a centre: replaces
 * compute_kinetic_energy(po, num_po, vel_cen, pos_cen, scale_now)
 * (src/potential.h:25, src/potential.c:194-211), with the cosmology (Om, Ol,
 * W0, WA) taken from cfg.  Every record with ke >= 0 gets
 * ke = a/(2G) sum_k (v_k - vel_cen_k + H(a) a (x_k - pos_cen_k))^2 with the
 * reference's float/double conversions; records with ke < 0 (potential-only)
 * are left alone.  po is not reordered. */
int rsg_compute_kinetic_energy(struct rsg_potential *po, int64_t num_po, const float *vel_cen,
                               const float *pos_cen, float scale_now,
                               const struct rsg_config *cfg);

/* Catalogue output (host; the halos, links and particles the calls above
 * return, p_start relative to p).  Options of one catalogue: */
struct rsg_catalog {
    int64_t id_offset;        /* id of the first halo written */
    int64_t snap, chunk;      /* binary header fields */
    const float *bounds;      /* 6 floats (min x y z, max x y z) or NULL: every
                                 halo is within bounds; the binary header then
                                 gets the printed halos' extent */
    int64_t num_p;            /* "#Total particles processed" (0: line omitted) */
    int64_t strict_so_masses; /* STRICT_SO_MASSES (ascii header line) */
};
/* _should_print (src/io/meta_io.c:266-286): the halo is inside bounds, and
 * carries ALWAYS_PRINT_FLAG or has at least MIN_HALO_OUTPUT_SIZE particles,
 * m * UNBOUND_THRESHOLD < mgrav and mgrav >= 1.5 PARTICLE_MASS (the last
 * when UNBOUND_THRESHOLD > 0).  Returns 1 or 0 (RSG_ERR_ARGS for NULLs);
 * rsg_count_halos_to_print is count_halos_to_print (:462-468). */
int rsg_should_print(const struct rsg_halo *h, const float *bounds, const struct rsg_config *cfg);
int64_t rsg_count_halos_to_print(const struct rsg_halo *halos, int64_t num_halos,
                                 const float *bounds, const struct rsg_config *cfg);
/* output_ascii (src/io/meta_io.c:288-371): the out_<snap>.list table of the
 * printable halos, ids from id_offset, to `path`, with the reference's
 * column header, header block and number formats (mass definitions vir,
 * 200b, 200c, 500c, 2500c, the ones the density thresholds use).  The idx,
 * i_so (sub_of), i_ph and mmetric columns come from extra. */
int rsg_write_ascii(const char *path, const struct rsg_halo *halos,
                    const struct rsg_extra_halo_info *extra, int64_t num_halos,
                    const struct rsg_catalog *opt, const struct rsg_config *cfg);
/* output_binary with output_particles = 1 (src/io/io_internal.c:118-186):
 * the 256-byte binary_output_header (src/io/io_internal.h:15-27; magic,
 * cosmology, bounds, counts, format revision 2, version "1.0.0RC", add_flag
 * 5 for the NFW chi2 and inertia-tensor layout), the printable halos with id
 * and p_start rewritten, then the int64 ids of their particles. */
int rsg_write_binary(const char *path, const struct rsg_halo *halos, int64_t num_halos,
                     const struct rsg_particle *p, int64_t num_p,
                     const struct rsg_catalog *opt, const struct rsg_config *cfg);

/* output_full_particles with print_child_particles (src/io/meta_io.c:378-461):
 * the halos_<snap>.<chunk>.particles table.  opt supplies id_offset, bounds,
 * num_p and strict_so_masses; unfiltered is UNFILTERED_HALO_OUTPUT and
 * every_n OUTPUT_EVERY_N_PARTICLES.  The printable halos get ids from
 * id_offset, the others -1 (listed only when unfiltered); every listed halo's
 * particles are followed, recursively, by its children's (extra child /
 * next_cochild).  ids_out (num_halos entries, or NULL) receives the ids the
 * reference writes back into halos[].id.  RSG_ERR_ARGS for a halo whose
 * particles lie outside p or a child link that leaves the halos or loops. */
int rsg_write_particles(const char *path, const struct rsg_halo *halos,
                        const struct rsg_extra_halo_info *extra, int64_t num_halos,
                        const struct rsg_particle *p, int64_t num_p,
                        const struct rsg_catalog *opt, int64_t unfiltered, int64_t every_n,
                        const struct rsg_config *cfg, int64_t *ids_out);

/* struct binary_output_header (src/io/io_internal.h:15-27), 256 bytes: the
 * header of the halo catalogue (halos_<snap>.<chunk>.bin) and of the
 * internal particle format. */
struct rsg_binary_header {
    uint64_t magic; /* 0xfadedacec0c0d0d0 */
    int64_t snap, chunk;
    float scale, Om, Ol, h0;
    float bounds[6];
    int64_t num_halos, num_particles;
    float box_size, particle_mass;
    int64_t particle_type; /* 0 none, 1 ids, 2 full records */
    int32_t format_revision;
    char rockstar_version[12];
    int32_t add_flag;
    char unused[256 - 12 - 4 * 12 - 4 * 2 - 8 * 6];
};
/* load_binary_halos (src/io/io_internal.c:199-225) on one catalogue file:
 * the header, the halo records and the particle ids, and cfg's scale_now,
 * om, ol, h0, box_size and particle_mass from the header
 * (read_binary_header_config).  With halos and ids NULL only the header is
 * read (its num_halos and num_particles size the arrays).  RSG_ERR_IO for an
 * unreadable, truncated or foreign file (the reference asserts or exits);
 * RSG_ERR_ARGS if max_halos or max_ids is too small.  File I/O only (parallel
 * reads), no device step. */
int rsg_read_binary(const char *path, struct rsg_binary_header *header, struct rsg_config *cfg,
                    struct rsg_halo *halos, int64_t max_halos, int64_t *ids, int64_t max_ids);

/* Particle input (host buffers; the records are assembled and sorted on the
 * device).  Options of a GADGET-2 file, named after src/config.template.h: */
struct rsg_gadget_opts {
    int64_t halo_particle_type;    /* GADGET_HALO_PARTICLE_TYPE (1) */
    int64_t skip_non_halo;         /* GADGET_SKIP_NON_HALO_PARTICLES (1) */
    double length_conversion;      /* GADGET_LENGTH_CONVERSION (1.0) */
    double mass_conversion;        /* GADGET_MASS_CONVERSION (1e10) */
    int64_t rescale_particle_mass; /* RESCALE_PARTICLE_MASS (0) */
    int64_t lightcone;             /* LIGHTCONE (0) */
    int64_t lgadget;               /* FILE_FORMAT "LGADGET" (0: "GADGET2") */
};
/* load_particles_gadget2 (src/io/io_gadget.c:200-254) for one file: the
 * particles of the halo type (or all), in file order, as the reference's
 * records -- positions times length_conversion, velocities times sqrt(a)
 * (1 for a lightcone), 4-byte ids widened as unsigned -- for any of the
 * three GADGET variants (untagged, 4- or 8-byte block tags), either byte
 * order, 4- or 8-byte ids and float or double coordinates.  cfg is updated
 * as gadget2_extract_header_info updates the reference's globals (:122-179):
 * om, ol, h0, box_size, total_particles, scale_now, particle_mass (from the
 * header's mass, unless it is 0 and cfg already has one, or from the
 * cosmology with rescale_particle_mass) and avg_particle_spacing.  With p
 * NULL only the count is returned in *num_p.  RSG_ERR_IO for an unreadable
 * or malformed file, RSG_ERR_INPUT for a curved cosmology (the reference
 * exits). */
int rsg_read_gadget2(const char *path, const struct rsg_gadget_opts *opt, struct rsg_config *cfg,
                     struct rsg_particle *p, int64_t max_p, int64_t *num_p);
/* The same with the records left in device memory: d_p (device) has room
 * for max_p records and holds the file's particles when the call returns, so
 * a snapshot goes from the file to rsg_sort_particles_by_id_device and
 * rsg_path_device without passing through host memory as records.  No
 * reference counterpart (the reference's reader fills host memory). */
int rsg_read_gadget2_device(const char *path, const struct rsg_gadget_opts *opt,
                            struct rsg_config *cfg, struct rsg_particle *d_p, int64_t max_p,
                            int64_t *num_p);
/* The reference's internal particle format (FILE_FORMAT "INTERNAL"; the
 * DUMP_PARTICLES output): load_particles_internal (src/io/io_internal.c:85-100)
 * on one file -- the 256-byte binary header (magic, PARTICLE_TYPE_FULL) and
 * the records verbatim.  cfg's scale_now, om, ol, h0, box_size and
 * particle_mass take the header's values, as read_binary_header_config does
 * (:43-50).  With p NULL only the count is returned in *num_p.  RSG_ERR_IO
 * for an unreadable, truncated or foreign file (the reference asserts).
 * The host variant reads with parallel preads and needs no device; the
 * device variant leaves the records in d_p (device memory). */
int rsg_read_internal(const char *path, struct rsg_config *cfg, struct rsg_particle *p,
                      int64_t max_p, int64_t *num_p);
int rsg_read_internal_device(const char *path, struct rsg_config *cfg, struct rsg_particle *d_p,
                             int64_t max_p, int64_t *num_p);
/* output_particles_internal(snap, chunk, 1) (src/io/io_internal.c:52-83):
 * the header of fill_binary_header with num_particles = num_p and
 * PARTICLE_TYPE_FULL, then p[0..num_p).  The random subsample of a fraction
 * in (0, 1) (the weak-lensing output) is not provided. */
int rsg_write_internal(const char *path, const struct rsg_particle *p, int64_t num_p,
                       int64_t snap, int64_t chunk, const struct rsg_config *cfg);
/* The reference sorts the particles by id before halo finding
 * (std::sort, src/mpi_main.cpp:2021-2024); this sorts p[0..n) by id on the
 * device (radix sort, stable: particles with equal ids, for which the
 * reference's order is unspecified, keep their input order). */
int rsg_sort_particles_by_id(struct rsg_particle *p, int64_t n);
/* The same on device-resident records d_p[0..n), in place. */
int rsg_sort_particles_by_id_device(struct rsg_particle *d_p, int64_t n);

/* Selects the potential form (0-3, as for rsg_compute_potential) that the
 * batched substructure form (rsg_find_subs_batch, rsg_path_device with
 * batched = 1) uses from now on, process-wide; the default is 1.  The plain
 * form always uses form 0.  Returns the previous form, or RSG_ERR_ARGS.
 * No reference counterpart: it serves the potential precision study. */
int32_t rsg_set_potential_form(int32_t form);

/* Size-class thresholds and chunk sizes of the batched form, by name
 * (process-wide; no reference counterpart):
 *   asc_bucket_min  nodes with more growing halos scan Morton-ordered
 *                   buckets in the particle assignment and parent search (64)
 *   bh_huge         Barnes-Hut nodes with more points take the chunked
 *                   node pass (65536), bh_chunk points per chunk (16384)
 *   seg_max         records per potential-set copy segment (8192)
 *   norm_chunk      records per chunk of the chunked norm_sd (4096)
 *   bp_big          halos with more particles take the chunked basic
 *                   properties (16384), bp_chunk particles per chunk (4096)
 * They change speed only (choices stay exact, sums change at most by FP64
 * rounding).  rsg_set_tuning returns RSG_ERR_ARGS for an unknown name or a
 * value outside the parameter's range; mpi-rockstar_gb300/autotune.py picks
 * them by measurement. */
int32_t rsg_set_tuning(const char *name, int64_t value);
int32_t rsg_get_tuning(const char *name, int64_t *value);

/* The per-halo potential records the reference hands to its
 * analyze_halo_generic callback (src/properties.c:554-555, declared in
 * src/io/io_generic.h:12-18): after the potentials and kinetic energies,
 * with the potential-only records dropped, sorted by r^2.  When
 * rsg_keep_halo_records(1) is set (process-wide), rsg_find_subs,
 * rsg_find_subs_batch and rsg_path_device keep them.  rsg_halo_records then
 * copies those of the calling thread's last call to out, and count[i] records of halo i
 * (its index in that call's halo output, nh halos) start at out[first[i]].
 * Call it with out = NULL for the sizes.  Returns the number of records, or
 * RSG_ERR_ARGS when cap is too small.  Records are kept per host thread;
 * rsg_keep_halo_records(0) frees the calling thread's at once and every
 * other thread's at that thread's next call, and while the switch is off
 * rsg_halo_records reports none. */
int32_t rsg_keep_halo_records(int32_t on);
int64_t rsg_halo_records(struct rsg_potential *out, int64_t cap, int64_t *first, int64_t *count,
                         int64_t nh);

/* Allocation-free 3D FOF of one chunk: rsg_rockstar_fof on device buffers,
 * with no counterpart in the reference (whose fof.c grows its buffers with
 * realloc).  It allocates no device memory: every scratch buffer is carved
 * from one fixed device array of RSG_NOALLOC_SCRATCH_BYTES per device.  The
 * first call in a process (and the first after a device reset) loads the
 * library's kernels and that array, which takes device memory once: make
 * it at setup, before any stream capture.  Later calls take none.  For
 * callers that cannot let a library allocate or free device memory while
 * their own kernels run.
 *   d_in  : num_p particles on the device (num_p <= RSG_NOALLOC_MAX_PARTICLES,
 *           else RSG_ERR_LIMIT); not modified.
 *   d_out : device, capacity num_p, must not overlap d_in; receives the
 *           permuted, deduplicated particles (*num_p_out of them).
 *   d_fof_offsets / d_fof_sizes : device, capacity max_fofs; groups as
 *           rsg_rockstar_fof returns them (same groups, same order).
 *   stream: a cudaStream_t (NULL = the legacy default stream); the call
 *           returns after the stream has drained.
 * Very dense chunks can need more scratch than the array holds (the FOF's
 * neighbour lists grow with density): the call then fails with
 * RSG_ERR_LIMIT.  Calls on one device must not overlap in time; a call made
 * while another is in progress on the same device returns RSG_ERR_BUSY. */
#define RSG_NOALLOC_MAX_PARTICLES 65536
#define RSG_NOALLOC_SCRATCH_BYTES (64u << 20)
int rsg_rockstar_fof_noalloc(const struct rsg_particle *d_in, int64_t num_p,
                             const struct rsg_config *cfg, struct rsg_particle *d_out,
                             int64_t *num_p_out, int64_t *d_fof_offsets, int64_t *d_fof_sizes,
                             int64_t max_fofs, int64_t *num_fofs, void *stream);

/* Work counters of the last rsg_path_device / rsg_find_subs* /
 * rsg_rockstar_fof call on the calling thread (vals[0..n), n <=
 * RSG_STAT_COUNT), for throughput and roofline accounting. */
#define RSG_STAT_PARTICLES 0     /* particles after dedupe */
#define RSG_STAT_GROUPS 1        /* 3D FOF groups */
#define RSG_STAT_HALOS 2         /* halos written */
#define RSG_STAT_POT_RECORDS 3   /* potential records over all halos */
#define RSG_STAT_KEPT_BIG 4      /* kept records of block-processed halos */
#define RSG_STAT_KEPT_SMALL 5    /* kept records of thread-processed halos */
#define RSG_STAT_HALOS_BIG 6
#define RSG_STAT_HALOS_SMALL 7
#define RSG_STAT_DENSE 8         /* 3D FOF particles with > 16 neighbours */
#define RSG_STAT_DENSE_PAIRS 9   /* 3D FOF pairs of dense particles k < j with j in
                                    k's r-sphere */
#define RSG_STAT_6D_ITEMS 10     /* particles summed over the 6D hierarchy levels */
#define RSG_STAT_6D_SAMPLES 11   /* linking-length samples summed over the levels */
#define RSG_STAT_NEAR_6D 12      /* 6D particle pairs whose distance is within 1e-6
                                    (relative) of their subgroup's linking length */
#define RSG_STAT_SEED_STEPS 13   /* 3D FOF seed frontiers (device-side loop steps) */
#define RSG_STAT_COUNT 14
int rsg_last_stats(int64_t *vals, int32_t n);

/* Instrumentation: kernels launched by this library so far (process-wide),
 * and CUDA-event timing of every launch of the kernels whose name contains
 * `kernel_substring` (empty string: off).  rsg_profile_read returns the
 * number of timed launches and their summed device time, then clears. */
int64_t rsg_launch_count(void);
int rsg_profile_select(const char *kernel_substring);
int rsg_profile_read(int64_t *launches, double *total_ms);
/* Per-kernel table of the timed launches ("*" selects every kernel):
 * lines "name<TAB>launches<TAB>total_ms<TAB>gap_ms", largest total first
 * (gap_ms: device time between the end of the previous timed launch and the
 * start of this kernel's launches -- untimed work and host round trips --
 * when every kernel is timed), written to
 * buf (capacity cap, NUL-terminated); returns the table's length, then
 * clears the timed launches. */
int64_t rsg_profile_table(char *buf, int64_t cap);

#ifdef __cplusplus
}
#endif
#endif /* ROCKSTAR_GB300_H */
