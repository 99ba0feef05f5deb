/* Test-only driver around the reference's own hot-path sources.
 *
 * This file is ORACLE infrastructure: it is compiled together with the
 * unmodified reference sources (read in place from the reference checkout by
 * oracle/ref/Makefile) into oracle/_ref/libref_rockstar.so, which the tests
 * use to generate golden fixtures and to pin the C restatement in
 * oracle/rockstar_oracle.c.  Nothing in the product links or calls it.
 *
 * It supplies what the single-process hot path needs from outside the
 * compiled files:
 *   - realloc_halos / copy_halos, whose contract is given by
 *     src/mpi_main.cpp:1321-1361 (grow the global halo arrays; append a
 *     HaloInfo block at an offset, shifting its parent/child links);
 *   - the boundary-group globals that src/rockstar.c:130-221 refers to
 *     (unused when rockstar() is called with bounds == NULL);
 *   - aborting stand-ins for the two temporal-halo-finding I/O helpers that
 *     src/fun_times.c references (temporal finding is switched off).
 * and a small C API that ctypes can call. */
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <stdint.h>
#include <omp.h>
#include "rockstar.h"
#include "particle.h"
#include "fof.h"
#include "halo.h"
#include "groupies.h"
#include "potential.h"
#include "config.h"
#include "config_vars.h"
#include "io/io_internal.h"

/* boundary-group globals named by src/interleaving.h:21-27 */
int64_t num_new_bp = 0;
struct bgroup *bg = NULL;
struct bgroup *final_bg = NULL;
int64_t num_bg_sets = 0;
int64_t *bg_set_sizes = NULL;
int64_t *bg_set_indices = NULL;
int64_t our_chunk = 0;

/* get_output_filename (src/io/meta_io.c) builds names from OUTBASE; here the
 * one catalogue file a ref_output_binary call writes (temporal halo
 * finding, the other caller, is switched off). */
static const char *ref_out_path = NULL;
void get_output_filename(char *buffer, int maxlen, int64_t snap, int64_t chunk,
                         char *type) {
    (void)snap; (void)chunk; (void)type;
    if (!ref_out_path) {
        fprintf(stderr, "oracle: temporal halo finding is disabled\n");
        abort();
    }
    snprintf(buffer, maxlen, "%s", ref_out_path);
}
/* _within_bounds / _should_print, restated from src/io/meta_io.c:266-286
 * (meta_io.c itself needs the tirpc library's headers and is not built):
 * output_binary (src/io/io_internal.c, compiled here) calls it. */
int _should_print(struct halo *h, float *bounds) {
    int64_t i;
    if (bounds)
        for (i = 0; i < 3; i++)
            if (h->pos[i] < bounds[i] || h->pos[i] > bounds[i + 3]) return 0;
    if (h->flags & ALWAYS_PRINT_FLAG) return 1;
    if ((h->num_p < MIN_HALO_OUTPUT_SIZE) || (h->m * UNBOUND_THRESHOLD >= h->mgrav) ||
        ((h->mgrav < 1.5 * PARTICLE_MASS) && UNBOUND_THRESHOLD > 0))
        return 0;
    return 1;
}
void output_binary(int64_t id_offset, int64_t snap, int64_t chunk, float *bounds,
                   int64_t output_particles);
/* The reference's output_binary over the given halos and particles (the
 * globals it reads are pointed at them for the call). */
void ref_output_binary(const char *path, struct halo *h, int64_t nh, struct particle *parts,
                       int64_t np, int64_t id_offset, int64_t snap, int64_t chunk,
                       float *bounds) {
    struct halo *sh = halos;
    int64_t snh = num_halos, snp = num_p;
    struct particle *sp = p;
    halos = h;
    num_halos = nh;
    p = parts;
    num_p = np;
    ref_out_path = path;
    output_binary(id_offset, snap, chunk, bounds, 1);
    ref_out_path = NULL;
    halos = sh;
    num_halos = snh;
    p = sp;
    num_p = snp;
}

void realloc_halos(int64_t new_num_halos) {
    halos = realloc(halos, sizeof(struct halo) * (new_num_halos ? new_num_halos : 1));
    extra_info = realloc(extra_info,
                         sizeof(struct extra_halo_info) * (new_num_halos ? new_num_halos : 1));
}

void copy_halos(const struct HaloInfo *haloinfo, int64_t offset) {
    struct extra_halo_info *ei = haloinfo->extra_info;
    for (int64_t i = 0; i < haloinfo->num_halos; i++) {
        if (ei[i].sub_of != -1) ei[i].sub_of += offset;
        if (ei[i].child != -1) ei[i].child += offset;
        if (ei[i].next_cochild != -1) ei[i].next_cochild += offset;
        if (ei[i].prev_cochild != -1) ei[i].prev_cochild += offset;
    }
    memcpy(halos + offset, haloinfo->halos, sizeof(struct halo) * haloinfo->num_halos);
    memcpy(extra_info + offset, haloinfo->extra_info,
           sizeof(struct extra_halo_info) * haloinfo->num_halos);
}

/* Hot-path parameters a caller may set.  Everything else keeps the
 * reference default from src/config.template.h. */
struct ref_params {
    double particle_mass, box_size, om, ol, h0, w0, wa;
    double fof_linking_length, fof_fraction, force_res, force_res_phys_max;
    double scale_now, initial_metric_scaling, include_host_potential_ratio;
    double unbound_threshold;
    int64_t min_halo_particles, min_halo_output_size, bound_props;
    int64_t shape_iterations, weighted_shapes, exact_ll_calc, total_particles;
};

int64_t ref_sizeof_halo(void) { return sizeof(struct halo); }
int64_t ref_sizeof_extra(void) { return sizeof(struct extra_halo_info); }
int64_t ref_sizeof_potential(void) { return sizeof(struct potential); }

void ref_setup(const struct ref_params *q) {
    static int configured = 0;
    if (!configured) { do_config(NULL); configured = 1; }
    PARTICLE_MASS = q->particle_mass;
    BOX_SIZE = q->box_size;
    Om = q->om; Ol = q->ol; h0 = q->h0; W0 = q->w0; WA = q->wa;
    FOF_LINKING_LENGTH = q->fof_linking_length;
    FOF_FRACTION = q->fof_fraction;
    FORCE_RES = q->force_res;
    FORCE_RES_PHYS_MAX = q->force_res_phys_max;
    SCALE_NOW = q->scale_now;
    INITIAL_METRIC_SCALING = q->initial_metric_scaling;
    INCLUDE_HOST_POTENTIAL_RATIO = q->include_host_potential_ratio;
    UNBOUND_THRESHOLD = q->unbound_threshold;
    MIN_HALO_PARTICLES = q->min_halo_particles;
    MIN_HALO_OUTPUT_SIZE = q->min_halo_output_size;
    BOUND_PROPS = q->bound_props;
    SHAPE_ITERATIONS = q->shape_iterations;
    WEIGHTED_SHAPES = q->weighted_shapes;
    EXACT_LL_CALC = q->exact_ll_calc;
    TOTAL_PARTICLES = q->total_particles;
    TEMPORAL_HALO_FINDING = 0;
    PERIODIC = 0;
    LIGHTCONE = 0;
    AVG_PARTICLE_SPACING = 0; /* must be re-derived on every setup */
    setup_config();
    calc_mass_definition();
}

double ref_avg_particle_spacing(void) { return AVG_PARTICLE_SPACING; }
double ref_particle_mass(void) { return PARTICLE_MASS; }
void ref_thresholds(double *out8) {
    for (int i = 0; i < 5; i++) out8[i] = particle_thresh_dens[i];
    out8[5] = particle_rvir_dens;
    out8[6] = particle_rvir_dens_z0;
    out8[7] = dynamical_time;
}

/* 3D FOF only: rockstar(NULL, 1) on a copy of `in` (caller sorts by id).
 * Writes the permuted/deduplicated particles to `out` (capacity n), the new
 * particle count to *num_out and each group's (offset, size) into the
 * caller's arrays (capacity max_fofs).  Returns the number of groups. */
int64_t ref_fof(const struct particle *in, int64_t n, struct particle *out,
                int64_t *num_out, int64_t *fof_off, int64_t *fof_np,
                int64_t max_fofs) {
    p = malloc(sizeof(struct particle) * (n ? n : 1));
    memcpy(p, in, sizeof(struct particle) * n);
    num_p = n;
    rockstar(NULL, 1);
    memcpy(out, p, sizeof(struct particle) * num_p);
    *num_out = num_p;
    int64_t nf = num_all_fofs;
    for (int64_t i = 0; i < nf && i < max_fofs; i++) {
        fof_off[i] = all_fofs[i].particles - p;
        fof_np[i] = all_fofs[i].num_p;
    }
    rockstar_cleanup();
    free(p); p = NULL; num_p = 0;
    return nf;
}

/* find_subs over groups that are already contiguous in `parts` (n total),
 * exactly as the OMP loop of src/mpi_main.cpp:1363-1389 runs it.  `parts` is
 * permuted in place, as the reference does.  Halos are appended to
 * halos_out / extra_out (capacity max_halos) in group order when
 * nthreads == 1.  Returns the number of halos, or -1 on overflow. */
int64_t ref_find_subs(struct particle *parts, int64_t n, const int64_t *fof_off,
                      const int64_t *fof_np, int64_t nfofs,
                      struct halo *halos_out, struct extra_halo_info *extra_out,
                      int64_t max_halos, int nthreads) {
    p = parts;
    num_p = n;
    all_fofs = malloc(sizeof(struct fof) * (nfofs ? nfofs : 1));
    for (int64_t i = 0; i < nfofs; i++) {
        all_fofs[i].particles = parts + fof_off[i];
        all_fofs[i].num_p = fof_np[i];
    }
    num_all_fofs = nfofs;
    num_bfofs = 0;
    num_halos = 0;
    int64_t *offs = calloc(nthreads + 1, sizeof(int64_t));
#pragma omp parallel num_threads(nthreads) copyin(particle_thresh_dens, particle_rvir_dens, particle_rvir_dens_z0, min_dens_index, dynamical_time, scale_dx)
    {
        struct FOFInfo fofinfo;
        init_fofinfo(&fofinfo);
        struct HaloInfo haloinfo;
        init_haloinfo(&haloinfo);
#pragma omp for schedule(dynamic)
        for (int64_t i = 0; i < nfofs; i++)
            find_subs(&all_fofs[i], &fofinfo, &haloinfo);
        int tid = omp_get_thread_num();
        offs[tid + 1] = haloinfo.num_halos;
#pragma omp barrier
#pragma omp single
        {
            for (int t = 0; t < nthreads; t++) offs[t + 1] += offs[t];
            realloc_halos(offs[nthreads]);
            num_halos = offs[nthreads];
        }
        copy_halos(&haloinfo, offs[tid]);
        free_fofinfo(&fofinfo);
        free_haloinfo(&haloinfo);
    }
    free(offs);
    int64_t nh = num_halos;
    if (nh <= max_halos) {
        memcpy(halos_out, halos, sizeof(struct halo) * nh);
        memcpy(extra_out, extra_info, sizeof(struct extra_halo_info) * nh);
    }
    free(all_fofs); all_fofs = NULL; num_all_fofs = 0;
    free(halos); halos = NULL;
    free(extra_info); extra_info = NULL;
    num_halos = 0;
    p = NULL; num_p = 0;
    return nh <= max_halos ? nh : -1;
}

/* Plain compute_potential (src/potential.c:183) on a caller array. */
void ref_compute_potential(struct potential *po, int64_t n) {
    compute_potential(po, n);
}

void ref_compute_kinetic_energy(struct potential *po, int64_t n, float *vel_cen,
                                float *pos_cen, float scale_now) {
    compute_kinetic_energy(po, n, vel_cen, pos_cen, scale_now);
}

/* Timing helper: wall time of the whole path, FOF and find_subs separately. */
int64_t ref_time_path(const struct particle *in, int64_t n, int nthreads,
                      double *t_fof, double *t_subs) {
    p = malloc(sizeof(struct particle) * (n ? n : 1));
    memcpy(p, in, sizeof(struct particle) * n);
    num_p = n;
    double t0 = omp_get_wtime();
    rockstar(NULL, 1);
    double t1 = omp_get_wtime();
    int64_t nf = num_all_fofs;
    int64_t *off = malloc(sizeof(int64_t) * (nf ? nf : 1));
    int64_t *np_ = malloc(sizeof(int64_t) * (nf ? nf : 1));
    for (int64_t i = 0; i < nf; i++) {
        off[i] = all_fofs[i].particles - p;
        np_[i] = all_fofs[i].num_p;
    }
    struct particle *parts = p;
    int64_t np0 = num_p;
    rockstar_cleanup();
    p = NULL;
    double t2 = omp_get_wtime();
    int64_t cap = nf * 64 + 1000;
    struct halo *h = malloc(sizeof(struct halo) * cap);
    struct extra_halo_info *e = malloc(sizeof(struct extra_halo_info) * cap);
    int64_t nh = ref_find_subs(parts, np0, off, np_, nf, h, e, cap, nthreads);
    double t3 = omp_get_wtime();
    *t_fof = t1 - t0;
    *t_subs = t3 - t2;
    free(h); free(e); free(off); free(np_); free(parts);
    return nh;
}

/* The reference's internal particle format (src/io/io_internal.c, compiled
 * here): output_particles_internal(snap, chunk, 1) over the given particles
 * with the configuration cfg_in = {SCALE_NOW, Om, Ol, h0, BOX_SIZE,
 * PARTICLE_MASS}, and load_particles_internal on one file, returning the
 * particles and the same six values after the read. */
void output_particles_internal(int64_t snap, int64_t chunk, double fraction);
void load_particles_internal(char *filename, struct particle **part, int64_t *num_part);
static void ref_cfg_get(double *c) {
    c[0] = SCALE_NOW;
    c[1] = Om;
    c[2] = Ol;
    c[3] = h0;
    c[4] = BOX_SIZE;
    c[5] = PARTICLE_MASS;
}
static void ref_cfg_set(const double *c) {
    SCALE_NOW = c[0];
    Om = c[1];
    Ol = c[2];
    h0 = c[3];
    BOX_SIZE = c[4];
    PARTICLE_MASS = c[5];
}
void ref_output_particles_internal(const char *path, struct particle *parts, int64_t np,
                                   int64_t snap, int64_t chunk, const double *cfg_in) {
    double saved[6];
    ref_cfg_get(saved);
    struct particle *sp = p;
    int64_t snp = num_p;
    ref_cfg_set(cfg_in);
    p = parts;
    num_p = np;
    ref_out_path = path;
    output_particles_internal(snap, chunk, 1);
    ref_out_path = NULL;
    p = sp;
    num_p = snp;
    ref_cfg_set(saved);
}
int64_t ref_load_internal(const char *path, struct particle *out, int64_t max_p,
                          double *cfg_out) {
    struct particle *pp = NULL;
    int64_t n = 0;
    load_particles_internal((char *)path, &pp, &n);
    if (n <= max_p) memcpy(out, pp, sizeof(struct particle) * n);
    free(pp);
    ref_cfg_get(cfg_out);
    return n;
}

/* The reference's load_binary_halos (src/io/io_internal.c:199-225) on one
 * catalogue file: header, halos and particle ids, and the six configuration
 * values read_binary_header_config sets.  Returns the number of halos. */
void load_binary_halos(int64_t snap, int64_t chunk, struct binary_output_header *bheader,
                       struct halo **halos, int64_t **part_ids, int64_t coalesced);
int64_t ref_load_binary(const char *path, void *header_out, struct halo *h_out, int64_t max_h,
                        int64_t *ids_out, int64_t max_ids, double *cfg_out) {
    struct binary_output_header bh;
    struct halo *hh = NULL;
    int64_t *ids = NULL;
    ref_out_path = path;
    load_binary_halos(0, 0, &bh, &hh, &ids, 0);
    ref_out_path = NULL;
    memcpy(header_out, &bh, sizeof bh);
    if (bh.num_halos <= max_h) memcpy(h_out, hh, sizeof(struct halo) * bh.num_halos);
    if (bh.num_particles <= max_ids) memcpy(ids_out, ids, sizeof(int64_t) * bh.num_particles);
    free(hh);
    free(ids);
    ref_cfg_get(cfg_out);
    return bh.num_halos;
}

/* The merger tree's descendant rule (src/merger.c, compiled here): halos1 /
 * part1 of one snapshot against halos2 / part2 of the next, through
 * init_descendants, connect_particle_ids_to_halo_ids and
 * calculate_descendants; desc_out receives halos1[i].desc. */
#include "merger.h"
void ref_descendants(const struct halo *h1, int64_t nh1, const int64_t *p1, int64_t np1,
                     const struct halo *h2, int64_t nh2, const int64_t *p2, int64_t np2,
                     int64_t *desc_out) {
    clear_merger_tree();
    halos1 = malloc(sizeof(struct halo) * (nh1 ? nh1 : 1));
    halos2 = malloc(sizeof(struct halo) * (nh2 ? nh2 : 1));
    part1 = malloc(sizeof(int64_t) * (np1 ? np1 : 1));
    part2 = malloc(sizeof(int64_t) * (np2 ? np2 : 1));
    memcpy(halos1, h1, sizeof(struct halo) * nh1);
    memcpy(halos2, h2, sizeof(struct halo) * nh2);
    memcpy(part1, p1, sizeof(int64_t) * np1);
    memcpy(part2, p2, sizeof(int64_t) * np2);
    head1.num_halos = nh1;
    head1.num_particles = np1;
    head2.num_halos = nh2;
    head2.num_particles = np2;
    init_descendants();
    connect_particle_ids_to_halo_ids();
    calculate_descendants();
    for (int64_t i = 0; i < nh1; i++) desc_out[i] = halos1[i].desc;
    clear_merger_tree();
}

/* The reference's GADGET-2 reader (src/io/io_gadget.c, compiled here) on one
 * file with the given reader settings: the particles in file order and the
 * configuration values it sets (Om, Ol, h0, BOX_SIZE, TOTAL_PARTICLES,
 * SCALE_NOW, PARTICLE_MASS, AVG_PARTICLE_SPACING). */
void load_particles_gadget2(char *filename, struct particle **p, int64_t *num_p);
int64_t ref_load_gadget2(const char *path, int64_t type, int64_t skip_non_halo, double lconv,
                         double mconv, int64_t rescale, int64_t lightcone, int64_t lgadget,
                         double particle_mass, struct particle *out, int64_t max_p,
                         double *cfg_out) {
    static char gadget2[] = "GADGET2", lgad[] = "LGADGET";
    GADGET_HALO_PARTICLE_TYPE = type;
    GADGET_SKIP_NON_HALO_PARTICLES = skip_non_halo;
    GADGET_LENGTH_CONVERSION = lconv;
    GADGET_MASS_CONVERSION = mconv;
    RESCALE_PARTICLE_MASS = rescale;
    LIGHTCONE = lightcone;
    FILE_FORMAT = lgadget ? lgad : gadget2;
    PARTICLE_MASS = particle_mass;
    struct particle *pp = NULL;
    int64_t n = 0;
    load_particles_gadget2((char *)path, &pp, &n);
    if (n <= max_p) memcpy(out, pp, sizeof(struct particle) * n);
    free(pp);
    cfg_out[0] = Om;
    cfg_out[1] = Ol;
    cfg_out[2] = h0;
    cfg_out[3] = BOX_SIZE;
    cfg_out[4] = (double)TOTAL_PARTICLES;
    cfg_out[5] = SCALE_NOW;
    cfg_out[6] = PARTICLE_MASS;
    cfg_out[7] = AVG_PARTICLE_SPACING;
    return n;
}
