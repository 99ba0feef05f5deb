// Catalogue output: the reference's halo filter and its two halo catalogue
// writers, applied to the halos, links and particles this library returns.
//   rsg_should_print   _within_bounds + _should_print (src/io/meta_io.c:266-286)
//   rsg_write_ascii    output_ascii with print_ascii_header_info
//                      (src/io/meta_io.c:288-371): the out_<snap>.list table
//   rsg_write_binary   output_binary with fill_binary_header
//                      (src/io/io_internal.c:16-41,118-186; header layout
//                      src/io/io_internal.h:6-27): halos_<snap>.<chunk>.bin
//   rsg_read_binary    load_binary_halos (src/io/io_internal.c:199-225): the
//                      same file read back
// Host code: formatting and file writes.  The file name is the caller's (the
// reference builds it from OUTBASE, snap and chunk in get_output_filename).
#include <fcntl.h>
#include <inttypes.h>
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <sys/stat.h>
#include <unistd.h>

#include <vector>

#include "binheader.cuh"
#include "common.cuh"
#include "hoststage.cuh"

namespace rsg {
namespace {

const int64_t kAlwaysPrint = 16;  // ALWAYS_PRINT_FLAG, src/groupies.h:12
// the mass definitions the density thresholds are derived with
// (src/config.template.h:9-13)
const char *const kMassDef[5] = {"vir", "200b", "200c", "500c", "2500c"};

bool within_bounds(const rsg_halo &h, const float *b) {
    if (!b) return true;
    for (int i = 0; i < 3; i++)
        if (h.pos[i] < b[i] || h.pos[i] > b[i + 3]) return false;
    return true;
}

bool should_print(const rsg_halo &h, const float *b, const rsg_config &c) {
    if (!within_bounds(h, b)) return false;
    if (h.flags & kAlwaysPrint) return true;
    // UNBOUND_THRESHOLD and PARTICLE_MASS are doubles in the reference: the
    // products and the comparison are in double
    if (h.num_p < c.min_halo_output_size || (double)h.m * c.unbound_threshold >= (double)h.mgrav ||
        ((double)h.mgrav < 1.5 * c.particle_mass && c.unbound_threshold > 0))
        return false;
    return true;
}

struct File {
    FILE *f = nullptr;
    ~File() {
        if (f) fclose(f);
    }
};

void header_info(FILE *o, const float *bounds, int64_t np, int64_t strict_so,
                 const rsg_config &c) {
    fprintf(o, "#a = %f\n", c.scale_now);
    if (bounds)
        fprintf(o, "#Bounds: (%f, %f, %f) - (%f, %f, %f)\n", bounds[0], bounds[1], bounds[2],
                bounds[3], bounds[4], bounds[5]);
    fprintf(o, "#Om = %f; Ol = %f; h = %f\n", c.om, c.ol, c.h0);
    fprintf(o, "#FOF linking length: %f\n", c.fof_linking_length);
    fprintf(o, "#Unbound Threshold: %f; FOF Refinement Threshold: %f\n", c.unbound_threshold,
            c.fof_fraction);
    fprintf(o, "#Particle mass: %.5e Msun/h\n", c.particle_mass);
    fprintf(o, "#Box size: %f Mpc/h\n", c.box_size);
    if (np) fprintf(o, "#Total particles processed: %" PRId64 "\n", np);
    fprintf(o, "#Force resolution assumed: %g Mpc/h\n", c.force_res);
    if (strict_so && !np) fprintf(o, "#Using Strict Spherical Overdensity Masses\n");
    fputs("#Units: Masses in Msun / h\n"
          "#Units: Positions in Mpc / h (comoving)\n"
          "#Units: Velocities in km / s (physical, peculiar)\n"
          "#Units: Halo Distances, Lengths, and Radii in kpc / h (comoving)\n"
          "#Units: Angular Momenta in (Msun/h) * (Mpc/h) * km/s (physical)\n"
          "#Units: Spins are dimensionless\n",
          o);
    if (np)
        fputs("#Units: Total energy in (Msun/h)*(km/s)^2 (physical)\n"
              "#Note: idx, i_so, and i_ph are internal debugging quantities\n",
              o);
    fputs("#Np is an internal debugging quantity.\n", o);
    fprintf(o, "#MPI-Rockstar Version: %s\n", kVersion);
}

}  // namespace
}  // namespace rsg

using namespace rsg;

extern "C" int rsg_should_print(const struct rsg_halo *h, const float *bounds,
                                const struct rsg_config *cfg) {
    if (!h || !cfg) return RSG_ERR_ARGS;
    return should_print(*h, bounds, *cfg) ? 1 : 0;
}

extern "C" int64_t rsg_count_halos_to_print(const struct rsg_halo *h, int64_t nh,
                                            const float *bounds, const struct rsg_config *cfg) {
    if ((!h && nh) || !cfg || nh < 0) return RSG_ERR_ARGS;
    int64_t k = 0;
    for (int64_t i = 0; i < nh; i++) k += should_print(h[i], bounds, *cfg);
    return k;
}

extern "C" int rsg_write_ascii(const char *path, const struct rsg_halo *h,
                               const struct rsg_extra_halo_info *e, int64_t nh,
                               const struct rsg_catalog *opt, const struct rsg_config *cfg) {
    if (!path || (!h && nh) || (!e && nh) || !opt || !cfg || nh < 0) {
        set_error(RSG_ERR_ARGS, "rsg_write_ascii: bad arguments");
        return RSG_ERR_ARGS;
    }
    const rsg_config &c = *cfg;
    File F;
    F.f = fopen(path, "w");
    if (!F.f) {
        set_error(RSG_ERR_IO, "rsg_write_ascii: cannot open %s", path);
        return RSG_ERR_IO;
    }
    FILE *o = F.f;
    const char *const *M = kMassDef;
    fprintf(o,
            "#id num_p m%s mbound_%s r%s vmax rvmax vrms x y z vx vy vz Jx Jy "
            "Jz E Spin PosUncertainty VelUncertainty bulk_vx bulk_vy bulk_vz "
            "BulkVelUnc n_core m%s m%s m%s m%s Xoff Voff spin_bullock b_to_a "
            "c_to_a A[x] A[y] A[z] b_to_a(%s) c_to_a(%s) A[x](%s) A[y](%s) "
            "A[z](%s) Rs Rs_Klypin T/|U| M_pe_Behroozi M_pe_Diemer "
            "Halfmass_Radius idx i_so i_ph num_cp mmetric\n",
            M[0], M[0], M[0], M[1], M[2], M[3], M[4], M[3], M[3], M[3], M[3], M[3]);
    header_info(o, opt->bounds, opt->num_p, opt->strict_so_masses, c);
    int64_t id = 0;
    for (int64_t i = 0; i < nh; i++) {
        if (!should_print(h[i], opt->bounds, c)) continue;
        const rsg_halo &t = h[i];
        fprintf(o,
                "%" PRId64 " %" PRId64 " %.3e %.3e"
                " %f %f %f %f %f %f %f %f %f %f %g %g %g %g %g %f %f %f %f %f "
                "%f %" PRId64 " %e %e %e %e %f %f %f %f %f %f %f %f %f %f %f "
                "%f %f %f %f %f %e %e %f %" PRId64 " %" PRId64 " %" PRId64 " %" PRId64 " %f\n",
                id + opt->id_offset, t.num_p, t.m, t.mgrav, t.r, t.vmax, t.rvmax, t.vrms,
                t.pos[0], t.pos[1], t.pos[2], t.pos[3], t.pos[4], t.pos[5], t.J[0], t.J[1],
                t.J[2], t.energy, t.spin, sqrt((double)t.min_pos_err),
                sqrt((double)t.min_vel_err), t.bulkvel[0], t.bulkvel[1], t.bulkvel[2],
                sqrt((double)t.min_bulkvel_err), t.n_core, t.alt_m[0], t.alt_m[1], t.alt_m[2],
                t.alt_m[3], t.Xoff, t.Voff, t.bullock_spin, t.b_to_a, t.c_to_a, t.A[0], t.A[1],
                t.A[2], t.b_to_a2, t.c_to_a2, t.A2[0], t.A2[1], t.A2[2], t.rs, t.klypin_rs,
                t.kin_to_pot, t.m_pe_b, t.m_pe_d, t.halfmass_radius, i, e[i].sub_of, e[i].ph,
                t.num_child_particles, e[i].max_metric);
        id++;
    }
    if (ferror(o)) {
        set_error(RSG_ERR_IO, "rsg_write_ascii: write to %s failed", path);
        return RSG_ERR_IO;
    }
    return 0;
}

extern "C" int rsg_write_particles(const char *path, const struct rsg_halo *h,
                                   const struct rsg_extra_halo_info *e, int64_t nh,
                                   const struct rsg_particle *p, int64_t num_p,
                                   const struct rsg_catalog *opt, int64_t unfiltered,
                                   int64_t every_n, const struct rsg_config *cfg,
                                   int64_t *ids_out) {
    if (!path || (nh && (!h || !e)) || !opt || !cfg || nh < 0 || num_p < 0 || (!p && num_p)) {
        set_error(RSG_ERR_ARGS, "rsg_write_particles: bad arguments");
        return RSG_ERR_ARGS;
    }
    const rsg_config &c = *cfg;
    // the ids output_full_particles assigns (and writes back into the halos)
    std::vector<int64_t> ids((size_t)nh);
    int64_t next = 0;
    for (int64_t i = 0; i < nh; i++)
        ids[i] = should_print(h[i], opt->bounds, c) ? opt->id_offset + next++ : -1;
    // the halos whose particles are listed, and everything their child links
    // reach, must stay inside p and the halo array, without cycles
    auto listed = [&](int64_t i) { return unfiltered || ids[i] > -1; };
    std::vector<int64_t> seen((size_t)nh, -1), stack;
    for (int64_t top = 0; top < nh; top++) {
        if (!listed(top)) continue;
        stack.assign(1, top);
        while (!stack.empty()) {
            const int64_t i = stack.back();
            stack.pop_back();
            if (i < 0 || i >= nh || seen[i] == top || h[i].p_start < 0 || h[i].num_p < 0 ||
                h[i].p_start + h[i].num_p > num_p) {
                set_error(RSG_ERR_ARGS, "rsg_write_particles: bad halo or child link below halo %" PRId64,
                          top);
                return RSG_ERR_ARGS;
            }
            seen[i] = top;
            for (int64_t ch = e[i].child; ch > -1; ch = (ch < nh ? e[ch].next_cochild : -1)) {
                if (ch >= nh || (int64_t)stack.size() > nh) {
                    set_error(RSG_ERR_ARGS, "rsg_write_particles: bad child link below halo %" PRId64,
                              top);
                    return RSG_ERR_ARGS;
                }
                stack.push_back(ch);
            }
        }
    }
    File F;
    F.f = fopen(path, "w");
    if (!F.f) {
        set_error(RSG_ERR_IO, "rsg_write_particles: cannot open %s", path);
        return RSG_ERR_IO;
    }
    FILE *o = F.f;
    const char *M0 = kMassDef[0];
    fputs("#Halo table:\n", o);
    fprintf(o,
            "#id internal_id num_p m%s mbound_%s r%s vmax rvmax vrms x y z vx vy vz Jx Jy Jz "
            "energy spin\n",
            M0, M0, M0);
    fputs("#Particle table:\n"
          "#x y z vx vy vz particle_id assigned_internal_haloid internal_haloid "
          "external_haloid\n",
          o);
    if (every_n > 1)
        fprintf(o, "#Notes: Only particles with IDs divisible by %" PRId64 " are printed.\n",
                every_n);
    fputs("#Notes: As not all halos are printed, some halos may not have external halo ids.  "
          "(Hence the need to print internal halo ids).  Each particle is assigned to a unique "
          "halo; however, some properties (such as halo bound mass) are calculated including "
          "all substructure.  As such, particles belonging to subhalos are included in "
          "outputs; to exclude substructure, verify that the internal halo id is the same as "
          "the assigned internal halo id.\n",
          o);
    header_info(o, opt->bounds, opt->num_p, opt->strict_so_masses, c);
    fputs("#Halo table begins here:\n", o);
    for (int64_t i = 0; i < nh; i++) {
        if (!listed(i)) continue;
        const rsg_halo &t = h[i];
        fprintf(o,
                "#%" PRId64 " %" PRId64 " %" PRId64 " %.3e %.3e %f %f %f %f %f %f %f %f %f %f "
                "%g %g %g %g %g\n",
                ids[i], i, t.num_p, t.m, t.mgrav, t.r, t.vmax, t.rvmax, t.vrms, t.pos[0], t.pos[1],
                t.pos[2], t.pos[3], t.pos[4], t.pos[5], t.J[0], t.J[1], t.J[2], t.energy, t.spin);
    }
    fputs("#Particle table begins here:\n", o);
    // each listed halo's particles, then its children's in child /
    // next_cochild order, depth first (print_child_particles)
    auto emit = [&](int64_t i, int64_t top) {
        for (int64_t j = 0; j < h[i].num_p; j++) {
            const rsg_particle &q = p[h[i].p_start + j];
            if (every_n <= 1 || !(q.id % every_n))
                fprintf(o, "%f %f %f %f %f %f %" PRId64 " %" PRId64 " %" PRId64 " %" PRId64 "\n",
                        q.pos[0], q.pos[1], q.pos[2], q.pos[3], q.pos[4], q.pos[5], q.id, i, top,
                        ids[top]);
        }
    };
    for (int64_t top = 0; top < nh; top++) {
        if (!listed(top)) continue;
        emit(top, top);
        stack.assign(1, e[top].child);  // the next child to visit at each depth
        while (!stack.empty()) {
            const int64_t ch = stack.back();
            if (ch < 0) {
                stack.pop_back();
                continue;
            }
            stack.back() = e[ch].next_cochild;
            emit(ch, top);
            stack.push_back(e[ch].child);
        }
    }
    if (ids_out) memcpy(ids_out, ids.data(), sizeof(int64_t) * (size_t)nh);
    if (ferror(o)) {
        set_error(RSG_ERR_IO, "rsg_write_particles: write to %s failed", path);
        return RSG_ERR_IO;
    }
    return 0;
}

extern "C" int rsg_write_binary(const char *path, const struct rsg_halo *h, int64_t nh,
                                const struct rsg_particle *p, int64_t num_p,
                                const struct rsg_catalog *opt, const struct rsg_config *cfg) {
    if (!path || (!h && nh) || !opt || !cfg || nh < 0 || num_p < 0 || (!p && num_p)) {
        set_error(RSG_ERR_ARGS, "rsg_write_binary: bad arguments");
        return RSG_ERR_ARGS;
    }
    const rsg_config &c = *cfg;
    const float *bounds = opt->bounds;
    BinHeader H;
    memset(&H, 0, sizeof H);
    // the halo records (id and p_start rewritten) and the bounds of the
    // printed halos; the running min/max start from the first halo,
    // printed or not (src/io/io_internal.c:137-157)
    float mn[3] = {0, 0, 0}, mx[3] = {0, 0, 0};
    if (nh) {
        memcpy(mn, h[0].pos, sizeof mn);
        memcpy(mx, h[0].pos, sizeof mx);
    }
    std::vector<char> keep((size_t)nh);
    for (int64_t i = 0; i < nh; i++) {
        keep[i] = should_print(h[i], bounds, c);
        if (!keep[i]) continue;
        if (h[i].p_start < 0 || h[i].num_p < 0 || h[i].p_start + h[i].num_p > num_p) {
            set_error(RSG_ERR_ARGS, "rsg_write_binary: halo %" PRId64 " lies outside p", i);
            return RSG_ERR_ARGS;
        }
        for (int j = 0; j < 3; j++) {
            if (mn[j] > h[i].pos[j]) mn[j] = h[i].pos[j];
            if (mx[j] < h[i].pos[j]) mx[j] = h[i].pos[j];
        }
    }
    File F;
    F.f = fopen(path, "wb");
    if (!F.f) {
        set_error(RSG_ERR_IO, "rsg_write_binary: cannot open %s", path);
        return RSG_ERR_IO;
    }
    FILE *o = F.f;
    fwrite(&H, sizeof H, 1, o);  // rewritten once the counts are known
    int64_t id = 0;
    for (int64_t i = 0; i < nh; i++) {
        if (!keep[i]) continue;
        rsg_halo t = h[i];
        t.id = id + opt->id_offset;
        t.p_start = H.num_particles;
        fwrite(&t, sizeof t, 1, o);
        H.num_halos++;
        H.num_particles += t.num_p;
        id++;
    }
    std::vector<int64_t> ids;
    for (int64_t i = 0; i < nh; i++) {
        if (!keep[i]) continue;
        ids.resize((size_t)h[i].num_p);
        for (int64_t j = 0; j < h[i].num_p; j++) ids[j] = p[h[i].p_start + j].id;
        if (!ids.empty()) fwrite(ids.data(), sizeof(int64_t), ids.size(), o);
    }
    const int64_t nhalos = H.num_halos, nparts = H.num_particles;
    fill_header(H, opt->snap, opt->chunk, c);
    H.num_halos = nhalos;
    H.num_particles = nparts;
    H.particle_type = kParticleTypeIds;
    if (bounds) {
        memcpy(H.bounds, bounds, sizeof(float) * 6);
    } else {
        memcpy(H.bounds, mn, sizeof(float) * 3);
        memcpy(H.bounds + 3, mx, sizeof(float) * 3);
    }
    rewind(o);
    fwrite(&H, sizeof H, 1, o);
    if (ferror(o)) {
        set_error(RSG_ERR_IO, "rsg_write_binary: write to %s failed", path);
        return RSG_ERR_IO;
    }
    return 0;
}

extern "C" int rsg_read_binary(const char *path, struct rsg_binary_header *header,
                               struct rsg_config *cfg, struct rsg_halo *halos, int64_t max_halos,
                               int64_t *ids, int64_t max_ids) {
    if (!path || !header || !cfg || max_halos < 0 || max_ids < 0 || (max_halos && !halos) ||
        (max_ids && !ids)) {
        set_error(RSG_ERR_ARGS, "rsg_read_binary: bad arguments");
        return RSG_ERR_ARGS;
    }
    int fd = open(path, O_RDONLY);
    struct stat sb;
    if (fd < 0 || fstat(fd, &sb) != 0) {
        if (fd >= 0) close(fd);
        set_error(RSG_ERR_IO, "rsg_read_binary: cannot open %s", path);
        return RSG_ERR_IO;
    }
    struct Closer {
        int fd;
        ~Closer() { close(fd); }
    } closer{fd};
    BinHeader H;
    if (pread(fd, &H, sizeof H, 0) != (ssize_t)sizeof H) {
        set_error(RSG_ERR_IO, "rsg_read_binary: file is truncated in %s", path);
        return RSG_ERR_IO;
    }
    // the reference asserts the magic and the counts and exits on a short
    // read (src/io/io_internal.c:212-222)
    const int64_t hb = (int64_t)sizeof(rsg_halo), need_h = H.num_halos, need_i = H.num_particles;
    const char *bad =
        H.magic != kMagic                ? "not a Rockstar binary file"
        : need_h < 0 || need_i < 0       ? "negative counts"
        : need_h > ((int64_t)1 << 40) / hb || need_i > ((int64_t)1 << 40) / 8 ? "implausible counts"
        : (int64_t)sb.st_size < (int64_t)sizeof H + need_h * hb + need_i * 8 ? "file is truncated"
                                                                             : nullptr;
    if (bad) {
        set_error(RSG_ERR_IO, "rsg_read_binary: %s in %s", bad, path);
        return RSG_ERR_IO;
    }
    *header = H;
    if (!halos && !ids) return 0;  // the header alone
    if (need_h > max_halos || need_i > max_ids) {
        set_error(RSG_ERR_ARGS, "rsg_read_binary: %lld halos / %lld ids for %lld / %lld places",
                  (long long)need_h, (long long)need_i, (long long)max_halos, (long long)max_ids);
        return RSG_ERR_ARGS;
    }
    try {
        read_file_parallel(fd, sizeof H, halos, (size_t)(need_h * hb), path);
        read_file_parallel(fd, (int64_t)sizeof H + need_h * hb, ids, (size_t)(need_i * 8), path);
    } catch (Failure &) {
        return error_code();
    }
    // read_binary_header_config
    cfg->scale_now = H.scale;
    cfg->om = H.Om;
    cfg->ol = H.Ol;
    cfg->h0 = H.h0;
    cfg->box_size = H.box_size;
    cfg->particle_mass = H.particle_mass;
    return 0;
}
