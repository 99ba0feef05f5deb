/* Reference-side binding of the GB300 library: the C file a maintainer adds to
 * MPI-Rockstar's src/ (as src/gpu_shim.c) to run the per-group hot path on
 * the GPU behind the reference's own calls.  It is compiled against the
 * reference's headers and include/rockstar_gb300.h with the reference's build
 * flags (-DOUTPUT_RVMAX -DOUTPUT_NFW_CHI2 -DOUTPUT_INERTIA_TENSOR) and linked
 * with mpi-rockstar_gb300/_build/librockstar_gb300.so.
 *
 * Call sites it serves (reference file:line):
 *   rockstar_gpu()               in place of rockstar(NULL, 1)
 *                                (src/rockstar.c:53-128, src/mpi_main.cpp:1564)
 *   do_halo_finding_gpu(batched) in place of the OpenMP find_subs loop with
 *                                extend_halos / copy_halos
 *                                (src/mpi_main.cpp:1331-1389)
 *   find_subs_gpu(f, fi, hi)     in place of one find_subs (src/groupies.h:36)
 *   compute_potential_gpu(...)   for compute_potential (src/potential.h:23,
 *                                called at src/properties.c:538)
 *   compute_kinetic_energy_gpu   for compute_kinetic_energy (src/potential.h:25,
 *                                called at src/properties.c:548-550)
 *   analyze_halos_gpu(base, nh)  calls the analyze_halo_generic hook
 *                                (src/io/io_generic.h:12-18) per halo
 *   output_catalogs_gpu(...)     in place of output_halos (src/io/meta_io.c:
 *                                489-509): output_ascii, output_binary,
 *                                output_full_particles and the particle dump
 *   load_particles_gadget2_gpu   in place of load_particles_gadget2
 *                                (src/io/io_gadget.h:29-30, called at
 *                                src/io/meta_io.c:170)
 *   sort_particles_by_id_gpu     in place of the std::sort by id before
 *                                find_halos (src/mpi_main.cpp:2021-2024)
 *   load_particles_internal_gpu  in place of load_particles_internal
 *                                (src/io/io_internal.h:35-36, called at
 *                                src/io/meta_io.c:175)
 *   output_particles_internal_gpu in place of output_particles_internal(snap,
 *                                chunk, 1) (src/io/meta_io.c:505)
 *   load_binary_halos_gpu        in place of load_binary_halos
 *                                (src/io/io_internal.h:41-44, the merger
 *                                tree's catalogue reader)
 * Errors: the library never exits; a non-zero return is mapped onto the
 * reference's rockstar_abort (src/error.h:17-20). */
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <strings.h>

#include "check_syscalls.h"
#include "config_vars.h"
#include "error.h"
#include "fof.h"
#include "groupies.h"
#include "io/io_generic.h"
#include "io/io_internal.h"
#include "io/meta_io.h"
#include "potential.h"
#include "rockstar.h"
#include "rockstar_gb300.h"

_Static_assert(sizeof(struct particle) == sizeof(struct rsg_particle), "particle layout");
_Static_assert(sizeof(struct halo) == sizeof(struct rsg_halo), "halo layout (build flags)");
_Static_assert(sizeof(struct extra_halo_info) == sizeof(struct rsg_extra_halo_info), "extra");
_Static_assert(sizeof(struct potential) == sizeof(struct rsg_potential), "potential layout");

/* ---- errors: rsg_* return codes -> rockstar_abort ------------------------ */
static void gpu_fail(const char *what) {
    fprintf(stderr, "[Error] %s: %s\n", what, rsg_last_error());
    rockstar_abort(1);
}

/* ---- configuration: the reference's globals (src/config_vars.h) ---------- */
static void gpu_config(struct rsg_config *c) {
    memset(c, 0, sizeof *c);
    c->particle_mass = PARTICLE_MASS;
    c->box_size = BOX_SIZE;
    c->om = Om;
    c->ol = Ol;
    c->h0 = h0;
    c->w0 = W0;
    c->wa = WA;
    c->fof_linking_length = FOF_LINKING_LENGTH;
    c->fof_fraction = FOF_FRACTION;
    c->force_res = FORCE_RES;
    c->force_res_phys_max = FORCE_RES_PHYS_MAX;
    c->scale_now = SCALE_NOW;
    c->initial_metric_scaling = INITIAL_METRIC_SCALING;
    c->include_host_potential_ratio = INCLUDE_HOST_POTENTIAL_RATIO;
    c->unbound_threshold = UNBOUND_THRESHOLD;
    c->min_halo_particles = MIN_HALO_PARTICLES;
    c->min_halo_output_size = MIN_HALO_OUTPUT_SIZE;
    c->bound_props = BOUND_PROPS;
    c->shape_iterations = SHAPE_ITERATIONS;
    c->weighted_shapes = WEIGHTED_SHAPES;
    c->exact_ll_calc = EXACT_LL_CALC;
    c->total_particles = TOTAL_PARTICLES;
    if (rsg_config_setup(c)) gpu_fail("rsg_config_setup");
}

/* ---- rockstar(NULL, 1): the single-domain 3D FOF ---------------------------
 * p is permuted in place exactly as the reference permutes it and all_fofs
 * gets the same groups in the same order (with bounds -- MPI boundary
 * tagging -- the reference's own rockstar() still runs). */
void rockstar_gpu(void) {
    struct rsg_config c;
    gpu_config(&c);
    int64_t cap = num_p / 2 + 1, n = num_p, nf = 0;
    int64_t *off = malloc(sizeof(int64_t) * cap), *sz = malloc(sizeof(int64_t) * cap);
    if (!off || !sz) gpu_fail("rockstar_gpu: out of host memory");
    if (rsg_rockstar_fof((struct rsg_particle *)p, &n, &c, off, sz, cap, &nf))
        gpu_fail("rsg_rockstar_fof");
    num_p = n;
    all_fofs = realloc(all_fofs, sizeof(struct fof) * (nf ? nf : 1));
    for (int64_t i = 0; i < nf; i++) {
        all_fofs[i].particles = p + off[i];
        all_fofs[i].num_p = sz[i];
    }
    num_all_fofs = nf;
    num_bfofs = 0;
    free(off);
    free(sz);
}

/* ---- the group loop of do_halo_finding -------------------------------------
 * One call covers every group; the output is in group order with p_start
 * relative to p, so the append only shifts the links by the halos already
 * present, as copy_halos does (src/mpi_main.cpp:1335-1361). */
void do_halo_finding_gpu(int batched) {
    struct rsg_config c;
    gpu_config(&c);
    int64_t nf = num_all_fofs - num_bfofs, cap = num_p / 2 + nf + 16, nh = 0;
    int64_t *off = malloc(sizeof(int64_t) * (nf + 1)), *sz = malloc(sizeof(int64_t) * (nf + 1));
    struct rsg_halo *h = malloc(sizeof *h * cap);
    struct rsg_extra_halo_info *e = malloc(sizeof *e * cap);
    if (!off || !sz || !h || !e) gpu_fail("do_halo_finding_gpu: out of host memory");
    for (int64_t i = 0; i < nf; i++) {
        off[i] = all_fofs[i].particles - p;
        sz[i] = all_fofs[i].num_p;
    }
    int rc = batched ? rsg_find_subs_batch((struct rsg_particle *)p, num_p, off, sz, nf, &c,
                                           h, e, cap, &nh)
                     : rsg_find_subs((struct rsg_particle *)p, num_p, off, sz, nf, &c,
                                     h, e, cap, &nh);
    if (rc) gpu_fail("rsg_find_subs");
    int64_t base = num_halos;
    realloc_halos(base + nh); /* src/mpi_main.cpp:1321-1324 */
    for (int64_t i = 0; i < nh; i++) {
        int64_t *l[4] = {&e[i].child, &e[i].next_cochild, &e[i].prev_cochild, &e[i].sub_of};
        for (int k = 0; k < 4; k++)
            if (*l[k] != -1) *l[k] += base;
    }
    memcpy(halos + base, h, sizeof *h * nh);
    memcpy(extra_info + base, e, sizeof *e * nh);
    num_halos = base + nh;
    free(off);
    free(sz);
    free(h);
    free(e);
}

/* ---- one find_subs(f, fofinfo, haloinfo) -----------------------------------
 * For callers that keep the reference's own loop; p_start is made relative
 * to the global p as src/groupies.c:705-707 does. */
void find_subs_gpu(struct fof *f, struct FOFInfo *fofinfo, struct HaloInfo *hi) {
    (void)fofinfo; /* scratch lives on the device */
    struct rsg_config c;
    gpu_config(&c);
    int64_t off = 0, sz = f->num_p, cap = f->num_p / 2 + 16, nh = 0;
    struct rsg_halo *h = malloc(sizeof *h * cap);
    struct rsg_extra_halo_info *e = malloc(sizeof *e * cap);
    if (!h || !e) gpu_fail("find_subs_gpu: out of host memory");
    if (rsg_find_subs((struct rsg_particle *)f->particles, f->num_p, &off, &sz, 1, &c, h, e, cap,
                      &nh))
        gpu_fail("rsg_find_subs");
    int64_t base = hi->num_halos, shift = f->particles - p;
    hi->halos = realloc(hi->halos, sizeof(struct halo) * (base + nh));
    hi->extra_info = realloc(hi->extra_info, sizeof(struct extra_halo_info) * (base + nh));
    for (int64_t i = 0; i < nh; i++) {
        h[i].p_start += shift;
        int64_t *l[4] = {&e[i].child, &e[i].next_cochild, &e[i].prev_cochild, &e[i].sub_of};
        for (int k = 0; k < 4; k++)
            if (*l[k] != -1) *l[k] += base;
    }
    memcpy(hi->halos + base, h, sizeof *h * nh);
    memcpy(hi->extra_info + base, e, sizeof *e * nh);
    hi->num_halos = base + nh;
    free(h);
    free(e);
}

/* ---- potentials and kinetic energies of one set ----------------------------
 * Same arguments and effect as compute_potential / compute_kinetic_energy
 * (src/potential.c:183-211): po comes back in the potential tree's order
 * with pe set (bit-identical, form 0), or with ke set.  A maintainer points
 * the calls of src/properties.c:538,548-550 at these (or renames them). */
void compute_potential_gpu(struct potential *po, int64_t num_po) {
    struct rsg_config c;
    gpu_config(&c);
    if (rsg_compute_potential((struct rsg_potential *)po, num_po, &c, 0))
        gpu_fail("rsg_compute_potential");
}

void compute_kinetic_energy_gpu(struct potential *po, int64_t num_po, float *vel_cen,
                                float *pos_cen, float scale_now) {
    struct rsg_config c;
    gpu_config(&c);
    if (rsg_compute_kinetic_energy((struct rsg_potential *)po, num_po, vel_cen, pos_cen,
                                   scale_now, &c))
        gpu_fail("rsg_compute_kinetic_energy");
}

/* ---- the analyze_halo_generic hook ------------------------------------------
 * After do_halo_finding_gpu, with rsg_keep_halo_records(1) set before it:
 * every halo's records as the reference hands them to the hook
 * (src/properties.c:554-555), in halo output order. */
void analyze_halos_gpu(int64_t base, int64_t nh) {
    if (!analyze_halo_generic || !nh) return;
    int64_t *first = malloc(sizeof(int64_t) * nh), *cnt = malloc(sizeof(int64_t) * nh);
    if (!first || !cnt) gpu_fail("analyze_halos_gpu: out of host memory");
    int64_t n = rsg_halo_records(NULL, 0, first, cnt, nh);
    struct potential *po = malloc(sizeof(struct potential) * (n > 0 ? n : 1));
    if (n < 0 || !po || rsg_halo_records((struct rsg_potential *)po, n, first, cnt, nh) < 0)
        gpu_fail("rsg_halo_records");
    for (int64_t i = 0; i < nh; i++)
        if (cnt[i]) analyze_halo_generic(halos + base + i, po + first[i], cnt[i]);
    free(po);
    free(first);
    free(cnt);
}

void output_particles_internal_gpu(int64_t snap, int64_t chunk);

/* ---- catalogue output -------------------------------------------------------
 * output_halos (src/io/meta_io.c:489-509) with the library's writers, from
 * halos, extra_info and p, under the reference's file names and conditions:
 * the out_<snap>.list and halos_<snap>.<chunk>.bin catalogues (OUTPUT_FORMAT
 * ASCII, BINARY or BOTH), the .particles table for chunk < FULL_PARTICLE_CHUNKS
 * (writing back the halo ids it assigns, as output_full_particles does) and
 * the DUMP_PARTICLES dump.  The weak-lensing subsample, drawn with the C
 * library's rand(), is left to the reference's own output_particles_internal. */
void output_catalogs_gpu(int64_t id_offset, int64_t snap, int64_t chunk, float *bounds) {
    struct rsg_config c;
    char buffer[1024];
    gpu_config(&c);
    struct rsg_catalog o = {id_offset, snap, chunk, bounds, num_p, STRICT_SO_MASSES};
    if (!strcasecmp(OUTPUT_FORMAT, "BOTH") || !strcasecmp(OUTPUT_FORMAT, "ASCII")) {
        get_output_filename(buffer, 1024, snap, chunk, "ascii");
        if (rsg_write_ascii(buffer, (struct rsg_halo *)halos,
                            (struct rsg_extra_halo_info *)extra_info, num_halos, &o, &c))
            gpu_fail("rsg_write_ascii");
    }
    if (!strcasecmp(OUTPUT_FORMAT, "BOTH") || !strcasecmp(OUTPUT_FORMAT, "BINARY") ||
        (TEMPORAL_HALO_FINDING && !LIGHTCONE)) {
        get_output_filename(buffer, 1024, snap, chunk, "bin");
        if (rsg_write_binary(buffer, (struct rsg_halo *)halos, num_halos,
                             (struct rsg_particle *)p, num_p, &o, &c))
            gpu_fail("rsg_write_binary");
    }
    if (chunk < FULL_PARTICLE_CHUNKS) {
        int64_t *ids = (int64_t *)check_realloc(NULL, (num_halos ? num_halos : 1) * sizeof(int64_t),
                                                "Allocating halo ids.");
        get_output_filename(buffer, 1024, snap, chunk, "particles");
        if (rsg_write_particles(buffer, (struct rsg_halo *)halos,
                                (struct rsg_extra_halo_info *)extra_info, num_halos,
                                (struct rsg_particle *)p, num_p, &o, UNFILTERED_HALO_OUTPUT,
                                OUTPUT_EVERY_N_PARTICLES, &c, ids))
            gpu_fail("rsg_write_particles");
        for (int64_t i = 0; i < num_halos; i++) halos[i].id = ids[i];
        free(ids);
    }
    if (DUMP_PARTICLES[0] && (chunk >= DUMP_PARTICLES[1] && chunk <= DUMP_PARTICLES[2]))
        output_particles_internal_gpu(snap, chunk);
    if (WEAK_LENSING_FRACTION > 0) output_particles_internal(snap, chunk, WEAK_LENSING_FRACTION);
}

/* ---- particle input -----------------------------------------------------------
 * One GADGET-2 (or LGADGET) file appended to *p, with the same arguments and
 * effects as load_particles_gadget2: the configuration globals its header
 * sets (Om, Ol, h0, BOX_SIZE, TOTAL_PARTICLES, SCALE_NOW, PARTICLE_MASS,
 * AVG_PARTICLE_SPACING) and *num_p advanced by the particles read.  A file the
 * reference would stop on (unreadable, truncated, curved cosmology) aborts. */
void load_particles_gadget2_gpu(char *filename, struct particle **p, int64_t *num_p) {
    struct rsg_config c;
    struct rsg_gadget_opts o = {GADGET_HALO_PARTICLE_TYPE,
                                GADGET_SKIP_NON_HALO_PARTICLES,
                                GADGET_LENGTH_CONVERSION,
                                GADGET_MASS_CONVERSION,
                                RESCALE_PARTICLE_MASS,
                                LIGHTCONE,
                                !strncasecmp(FILE_FORMAT, "LGADGET", 7)};
    int64_t n = 0;
    gpu_config(&c);
    if (rsg_read_gadget2(filename, &o, &c, NULL, 0, &n)) gpu_fail("rsg_read_gadget2");
    *p = (struct particle *)check_realloc(*p, ((*num_p) + n) * sizeof(struct particle),
                                          "Allocating particles.");
    gpu_config(&c);
    if (rsg_read_gadget2(filename, &o, &c, (struct rsg_particle *)(*p + *num_p), n, &n))
        gpu_fail("rsg_read_gadget2");
    Om = c.om;
    Ol = c.ol;
    h0 = c.h0;
    BOX_SIZE = c.box_size;
    TOTAL_PARTICLES = c.total_particles;
    SCALE_NOW = c.scale_now;
    PARTICLE_MASS = c.particle_mass;
    AVG_PARTICLE_SPACING = c.avg_particle_spacing;
    *num_p += n;
}

/* The particles sorted by id on the device (the reference's std::sort before
 * find_halos; equal ids keep their order). */
void sort_particles_by_id_gpu(struct particle *parts, int64_t n) {
    if (rsg_sort_particles_by_id((struct rsg_particle *)parts, n))
        gpu_fail("rsg_sort_particles_by_id");
}

/* The internal particle format (FILE_FORMAT "INTERNAL"): as
 * load_particles_internal, *p is replaced by the file's particles (not
 * appended to) and SCALE_NOW, Om, Ol, h0, BOX_SIZE and PARTICLE_MASS take the
 * header's values.  The records are read with the library's parallel reads. */
void load_particles_internal_gpu(char *filename, struct particle **parts, int64_t *num_parts) {
    struct rsg_config c;
    int64_t n = 0;
    gpu_config(&c);
    if (rsg_read_internal(filename, &c, NULL, 0, &n)) gpu_fail("rsg_read_internal");
    *parts = (struct particle *)check_realloc(*parts, (n ? n : 1) * sizeof(struct particle),
                                              "Allocating particles.");
    if (rsg_read_internal(filename, &c, (struct rsg_particle *)*parts, n, &n))
        gpu_fail("rsg_read_internal");
    SCALE_NOW = c.scale_now;
    Om = c.om;
    Ol = c.ol;
    h0 = c.h0;
    BOX_SIZE = c.box_size;
    PARTICLE_MASS = c.particle_mass;
    *num_parts = n;
}

/* output_particles_internal(snap, chunk, 1): p[0..num_p) with the
 * reference's header, to the reference's file name. */
void output_particles_internal_gpu(int64_t snap, int64_t chunk) {
    struct rsg_config c;
    char buffer[1024];
    gpu_config(&c);
    get_output_filename(buffer, 1024, snap, chunk, "rbin");
    if (rsg_write_internal(buffer, (struct rsg_particle *)p, num_p, snap, chunk, &c))
        gpu_fail("rsg_write_internal");
}

/* load_binary_halos: the catalogue of (snap, chunk) read back into *halos
 * and *part_ids (reallocated), its header into *bheader, and the six
 * configuration globals read_binary_header_config sets. */
void load_binary_halos_gpu(int64_t snap, int64_t chunk, struct binary_output_header *bheader,
                           struct halo **hs, int64_t **part_ids, int64_t coalesced) {
    struct rsg_config c;
    char buffer[1024];
    _Static_assert(sizeof(struct binary_output_header) == sizeof(struct rsg_binary_header),
                   "binary header layout");
    gpu_config(&c);
    get_output_filename(buffer, 1024, snap, chunk, coalesced ? "coalesced.bin" : "bin");
    struct rsg_binary_header *h = (struct rsg_binary_header *)bheader;
    if (rsg_read_binary(buffer, h, &c, NULL, 0, NULL, 0)) gpu_fail("rsg_read_binary");
    *hs = (struct halo *)check_realloc(*hs, (h->num_halos ? h->num_halos : 1) * sizeof(struct halo),
                                       "Allocating halos.");
    *part_ids = (int64_t *)check_realloc(
        *part_ids, (h->num_particles ? h->num_particles : 1) * sizeof(int64_t),
        "Allocating particle IDs.");
    if (rsg_read_binary(buffer, h, &c, (struct rsg_halo *)*hs, h->num_halos, *part_ids,
                        h->num_particles))
        gpu_fail("rsg_read_binary");
    SCALE_NOW = c.scale_now;
    Om = c.om;
    Ol = c.ol;
    h0 = c.h0;
    BOX_SIZE = c.box_size;
    PARTICLE_MASS = c.particle_mass;
}
