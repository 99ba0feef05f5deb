// C-ABI entry points (declared in include/rockstar_gb300.h).
#include <math.h>
#include <stdlib.h>
#include <string.h>

#include <atomic>
#include <vector>

#include "hoststage.cuh"
#include "kdtree_impl.cuh"
#include "subs.cuh"

namespace rsg {

extern std::vector<int32_t> g_dbg_level, g_dbg_start, g_dbg_n;
extern std::vector<float> g_dbg_target;

struct FofOut {
    int64_t num_p;
    int64_t nfofs;
};
FofOut fof3d_device(Arena &ar, const rsg_particle *d_in, int64_t n, const rsg_config &cfg,
                    rsg_particle *d_out, int64_t *d_off, int64_t *d_sz, cudaStream_t st);

__global__ void k_zero_pe(PotRec *PO, int64_t n) {
    int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i < n) PO[i].pe = 0;
}

void bh_potential(Arena &ar, PotRec *PO, int64_t npo, const int32_t *rs, const int32_t *rn,
                  int32_t ntrees, double mp, double force_res, int *err, cudaStream_t st,
                  int form);
int set_batched_potential_form(int f);
void kinetic_energy_device(PotRec *d, int64_t n, const float *vc, const float *pc, float scale,
                           double hub, cudaStream_t st);
double hubble100(const rsg_config &c, float scale);
extern std::atomic<bool> g_keep_po;
extern thread_local std::vector<PotRec> g_dbg_po;

// One device context per host thread: a stream and a scratch arena that is
// reused across calls (the role the reference's threadprivate scratch
// buffers play, src/groupies.c:52-57).
struct Ctx {
    cudaStream_t st = nullptr;
    Arena ar;
    int dev = -1;
};
static thread_local Ctx *g_ctx = nullptr;

Ctx &ctx() {
    if (!g_ctx) {
        int n = 0;
        if (cudaGetDeviceCount(&n) != cudaSuccess || n == 0) {
            set_error(RSG_ERR_NO_DEVICE, "no CUDA device available");
            throw Failure();
        }
        g_ctx = new Ctx();
        RSG_CUDA(cudaGetDevice(&g_ctx->dev));
        RSG_CUDA(cudaStreamCreateWithFlags(&g_ctx->st, cudaStreamNonBlocking));
    }
    return *g_ctx;
}

// The calling thread's arena, reserved for `bytes` and reset, and its stream
// (for the entry points of other translation units).
Arena &call_arena(size_t bytes, cudaStream_t *st) {
    Ctx &C = ctx();
    C.ar.reserve(bytes);
    C.ar.reset();
    *st = C.st;
    return C.ar;
}

// ---- configuration (host) ----------------------------------------------
static const double RHO_C = 2.77519737e11;  // src/universal_constants.h:5
static const double GRAV = 4.30117902e-9;   // src/universal_constants.h:4

struct Cosmo {
    const rsg_config *c;
    // src/hubble.c:8-19
    double weff(double a) const { return (a != 1.0) ? c->w0 + c->wa - c->wa * (a - 1.0) / log(a) : c->w0; }
    double hubble(double z) const {
        double z1 = 1.0 + z, a = 1.0 / z1;
        return sqrt(c->om * (z1 * z1 * z1) + c->ol * pow(a, -3.0 * (1.0 + weff(a))));
    }
    // src/groupies.c:97-100
    double vir(double a) const {
        double x = (c->om / pow(a, 3)) / pow(hubble(1.0 / a - 1.0), 2.0) - 1.0;
        return ((18 * M_PI * M_PI + 82.0 * x - 39 * x * x) / (1.0 + x));
    }
    // src/groupies.c:102-125; `kind` 'b' / 'c' with multiplier, or 'v' (virial)
    float thresh(char kind, double mult, double *z0) const {
        float scale = (float)c->scale_now;
        float mf = (float)((c->om / pow(scale, 3)) / pow(hubble(1.0 / scale - 1.0), 2.0));
        float cons = (float)(c->om * RHO_C / c->particle_mass);
        float t;
        if (kind == 'b') t = (float)(mult * cons);
        else if (kind == 'c') t = (float)(mult * cons / mf);
        else t = (float)(vir(scale) * cons);
        *z0 = vir(1.0) * cons;
        return t;
    }
};

}  // namespace rsg

using namespace rsg;

extern "C" {

int rsg_config_setup(struct rsg_config *c) {
    if (!c) return RSG_ERR_ARGS;
    if (!c->particle_mass) {
        if (!c->total_particles) {
            set_error(RSG_ERR_ARGS, "particle_mass = 0 needs total_particles");
            return RSG_ERR_ARGS;
        }
        c->particle_mass = RHO_C * c->box_size * c->box_size * c->box_size * c->om / c->total_particles;
    }
    c->avg_particle_spacing = cbrt(c->particle_mass / (c->om * RHO_C));
    if (!c->force_res_phys_max) c->force_res_phys_max = c->force_res;
    if (c->force_res * c->scale_now > c->force_res_phys_max)
        c->force_res = c->force_res_phys_max / c->scale_now;
    Cosmo k{c};
    double z0;
    c->particle_thresh_dens[0] = k.thresh('v', 0, &z0);
    c->particle_thresh_dens[1] = k.thresh('b', 200, &z0);
    c->particle_thresh_dens[2] = k.thresh('c', 200, &z0);
    c->particle_thresh_dens[3] = k.thresh('c', 500, &z0);
    c->particle_thresh_dens[4] = k.thresh('c', 2500, &z0);
    c->particle_rvir_dens = k.thresh('v', 0, &z0);
    c->particle_rvir_dens_z0 = z0;
    c->dynamical_time =
        1.0 / sqrt((4.0 * M_PI * GRAV / 3.0) * c->particle_rvir_dens * c->particle_mass);
    c->min_dens_index = 0;
    for (int i = 1; i < 5; i++)
        if (c->particle_thresh_dens[i] < c->particle_thresh_dens[c->min_dens_index])
            c->min_dens_index = i;
    return RSG_OK;
}

int rsg_rockstar_fof(struct rsg_particle *p, int64_t *num_p, const struct rsg_config *cfg,
                     int64_t *fof_offsets, int64_t *fof_sizes, int64_t max_fofs,
                     int64_t *num_fofs) {
    if (!p || !num_p || !cfg || !num_fofs || *num_p < 0) {
        set_error(RSG_ERR_ARGS, "rsg_rockstar_fof: null argument");
        return RSG_ERR_ARGS;
    }
    try {
        Ctx &C = ctx();
        int64_t n = *num_p;
        if (n == 0) {
            *num_fofs = 0;
            return RSG_OK;
        }
        C.ar.reserve((size_t)n * 600 + (256u << 20));
        C.ar.reset();
        rsg_particle *d_in = C.ar.get<rsg_particle>(n), *d_out = C.ar.get<rsg_particle>(n);
        int64_t *d_off = C.ar.get<int64_t>(n / 2 + 1), *d_sz = C.ar.get<int64_t>(n / 2 + 1);
        host_to_device(d_in, p, sizeof(rsg_particle) * n, C.st);
        FofOut o = fof3d_device(C.ar, d_in, n, *cfg, d_out, d_off, d_sz, C.st);
        if (o.nfofs > max_fofs) {
            set_error(RSG_ERR_ARGS, "rsg_rockstar_fof: %lld groups exceed max_fofs %lld",
                      (long long)o.nfofs, (long long)max_fofs);
            return RSG_ERR_ARGS;
        }
        device_to_host(p, d_out, sizeof(rsg_particle) * o.num_p, C.st);
        if (o.nfofs) {
            RSG_CUDA(cudaMemcpyAsync(fof_offsets, d_off, sizeof(int64_t) * o.nfofs, cudaMemcpyDeviceToHost, C.st));
            RSG_CUDA(cudaMemcpyAsync(fof_sizes, d_sz, sizeof(int64_t) * o.nfofs, cudaMemcpyDeviceToHost, C.st));
        }
        RSG_CUDA(cudaStreamSynchronize(C.st));
        *num_p = o.num_p;
        *num_fofs = o.nfofs;
        return RSG_OK;
    } catch (Failure &) {
        return error_code();
    }
}

static int find_subs_host(struct rsg_particle *p, int64_t num_p, const int64_t *fof_offsets,
                          const int64_t *fof_sizes, int64_t num_fofs,
                          const struct rsg_config *cfg, struct rsg_halo *halos,
                          struct rsg_extra_halo_info *extra, int64_t max_halos,
                          int64_t *num_halos, int exact) {
    if (!p || !cfg || !num_halos || num_p < 0 || num_fofs < 0 ||
        (num_fofs && (!fof_offsets || !fof_sizes))) {
        set_error(RSG_ERR_ARGS, "rsg_find_subs: bad arguments");
        return RSG_ERR_ARGS;
    }
    try {
        Ctx &C = ctx();
        int64_t M = 0;
        for (int64_t g = 0; g < num_fofs; g++) M += fof_sizes[g] > 0 ? fof_sizes[g] : 0;
        *num_halos = 0;
        if (M == 0) return RSG_OK;
        int64_t hcap = M / 2 + num_fofs + 16;
        C.ar.reserve((size_t)M * 900 + (size_t)num_p * 64 + (size_t)hcap * 360 + (256u << 20));
        C.ar.reset();
        rsg_particle *d_p = C.ar.get<rsg_particle>(num_p);
        rsg_halo *d_h = C.ar.get<rsg_halo>(hcap);
        rsg_extra_halo_info *d_e = C.ar.get<rsg_extra_halo_info>(hcap);
        host_to_device(d_p, p, sizeof(rsg_particle) * num_p, C.st);
        SubsOut o = find_subs_device(C.ar, d_p, num_p, fof_offsets, fof_sizes, num_fofs, *cfg,
                                     d_h, d_e, hcap, C.st, exact);
        if (o.nhalos > max_halos) {
            set_error(RSG_ERR_ARGS, "rsg_find_subs: %lld halos exceed max_halos %lld",
                      (long long)o.nhalos, (long long)max_halos);
            return RSG_ERR_ARGS;
        }
        device_to_host(p, d_p, sizeof(rsg_particle) * num_p, C.st);
        if (o.nhalos) {
            device_to_host(halos, d_h, sizeof(rsg_halo) * o.nhalos, C.st);
            device_to_host(extra, d_e, sizeof(rsg_extra_halo_info) * o.nhalos, C.st);
        }
        RSG_CUDA(cudaStreamSynchronize(C.st));
        *num_halos = o.nhalos;
        last_stats()[RSG_STAT_HALOS] = o.nhalos;
        return RSG_OK;
    } catch (Failure &) {
        return error_code();
    }
}

int rsg_find_subs(struct rsg_particle *p, int64_t num_p, const int64_t *fof_offsets,
                  const int64_t *fof_sizes, int64_t num_fofs, const struct rsg_config *cfg,
                  struct rsg_halo *halos, struct rsg_extra_halo_info *extra, int64_t max_halos,
                  int64_t *num_halos) {
    return find_subs_host(p, num_p, fof_offsets, fof_sizes, num_fofs, cfg, halos, extra,
                          max_halos, num_halos, 1);
}

int rsg_find_subs_batch(struct rsg_particle *p, int64_t num_p, const int64_t *fof_offsets,
                        const int64_t *fof_sizes, int64_t num_fofs, const struct rsg_config *cfg,
                        struct rsg_halo *halos, struct rsg_extra_halo_info *extra,
                        int64_t max_halos, int64_t *num_halos) {
    return find_subs_host(p, num_p, fof_offsets, fof_sizes, num_fofs, cfg, halos, extra,
                          max_halos, num_halos, 0);
}

int rsg_path_device(const struct rsg_particle *d_in, int64_t n, const struct rsg_config *cfg,
                    struct rsg_particle *d_out, int64_t *num_p_out, int64_t *num_fofs,
                    struct rsg_halo *d_halos, struct rsg_extra_halo_info *d_extra,
                    int64_t max_halos, int64_t *num_halos, int32_t batched) {
    if (!d_in || !d_out || !cfg || n < 0 || !num_halos || !num_fofs || !num_p_out) {
        set_error(RSG_ERR_ARGS, "rsg_path_device: bad arguments");
        return RSG_ERR_ARGS;
    }
    try {
        Ctx &C = ctx();
        *num_halos = 0;
        *num_fofs = 0;
        *num_p_out = n;
        if (n == 0) return RSG_OK;
        C.ar.reserve((size_t)n * 1000 + (512u << 20));
        C.ar.reset();
        int64_t *d_off = C.ar.get<int64_t>(n / 2 + 1), *d_sz = C.ar.get<int64_t>(n / 2 + 1);
        size_t mark = C.ar.used;
        FofOut o = fof3d_device(C.ar, d_in, n, *cfg, d_out, d_off, d_sz, C.st);
        C.ar.used = mark;
        std::vector<int64_t> off(o.nfofs), sz(o.nfofs);
        if (o.nfofs) {
            RSG_CUDA(cudaMemcpyAsync(off.data(), d_off, 8 * o.nfofs, cudaMemcpyDeviceToHost, C.st));
            RSG_CUDA(cudaMemcpyAsync(sz.data(), d_sz, 8 * o.nfofs, cudaMemcpyDeviceToHost, C.st));
            RSG_CUDA(cudaStreamSynchronize(C.st));
        }
        SubsOut s2 = find_subs_device(C.ar, d_out, o.num_p, off.data(), sz.data(), o.nfofs, *cfg,
                                      d_halos, d_extra, max_halos, C.st, batched ? 0 : 1);
        RSG_CUDA(cudaStreamSynchronize(C.st));
        phase_report();
        *num_p_out = o.num_p;
        *num_fofs = o.nfofs;
        *num_halos = s2.nhalos;
        last_stats()[RSG_STAT_HALOS] = s2.nhalos;
        return RSG_OK;
    } catch (Failure &) {
        return error_code();
    }
}

int rsg_compute_potential(struct rsg_potential *po, int64_t num_po, const struct rsg_config *cfg,
                          int32_t form) {
    if (!cfg || num_po < 0 || (num_po > 0 && !po) || form < 0 || form > 3) {
        set_error(RSG_ERR_ARGS, "rsg_compute_potential: bad arguments");
        return RSG_ERR_ARGS;
    }
    if (num_po >= (1ll << 31) - 2) {
        set_error(RSG_ERR_ARGS, "rsg_compute_potential: at most 2^31-2 records");
        return RSG_ERR_ARGS;
    }
    try {
        Ctx &C = ctx();
        if (num_po == 0) return RSG_OK;
        C.ar.reserve((size_t)num_po * 400 + (64u << 20));
        C.ar.reset();
        static_assert(sizeof(PotRec) == sizeof(rsg_potential), "potential record layout");
        PotRec *d = C.ar.get<PotRec>(num_po);
        int32_t *seg = C.ar.get<int32_t>(2);
        int *err = C.ar.get<int>(2);
        int32_t hseg[2] = {0, (int32_t)num_po};
        host_to_device(d, po, sizeof(PotRec) * num_po, C.st);
        RSG_CUDA(cudaMemcpyAsync(seg, hseg, sizeof(hseg), cudaMemcpyHostToDevice, C.st));
        RSG_CUDA(cudaMemsetAsync(err, 0, 2 * sizeof(int), C.st));
        launch(k_zero_pe, nblk(num_po, 256), 256, 0, C.st, d, num_po);
        bh_potential(C.ar, d, num_po, seg, seg + 1, 1, cfg->particle_mass, cfg->force_res, err,
                     C.st, form);
        int herr[2];
        device_to_host(po, d, sizeof(PotRec) * num_po, C.st);
        RSG_CUDA(cudaMemcpyAsync(herr, err, sizeof(herr), cudaMemcpyDeviceToHost, C.st));
        RSG_CUDA(cudaStreamSynchronize(C.st));
        if (herr[0]) {
            set_error(RSG_ERR_LIMIT, "potential tree traversal exceeded its stack");
            return RSG_ERR_LIMIT;
        }
        last_stats()[RSG_STAT_POT_RECORDS] = num_po;
        return RSG_OK;
    } catch (Failure &) {
        return error_code();
    }
}

int rsg_compute_kinetic_energy(struct rsg_potential *po, int64_t num_po, const float *vel_cen,
                               const float *pos_cen, float scale_now,
                               const struct rsg_config *cfg) {
    if (!cfg || !vel_cen || !pos_cen || num_po < 0 || (num_po > 0 && !po) || !(scale_now > 0)) {
        set_error(RSG_ERR_ARGS, "rsg_compute_kinetic_energy: bad arguments");
        return RSG_ERR_ARGS;
    }
    try {
        Ctx &C = ctx();
        if (num_po == 0) return RSG_OK;
        C.ar.reserve((size_t)num_po * sizeof(PotRec) + (16u << 20));
        C.ar.reset();
        PotRec *d = C.ar.get<PotRec>(num_po);
        host_to_device(d, po, sizeof(PotRec) * num_po, C.st);
        kinetic_energy_device(d, num_po, vel_cen, pos_cen, scale_now, hubble100(*cfg, scale_now),
                              C.st);
        device_to_host(po, d, sizeof(PotRec) * num_po, C.st);
        RSG_CUDA(cudaStreamSynchronize(C.st));
        return RSG_OK;
    } catch (Failure &) {
        return error_code();
    }
}

// name, field, smallest and largest accepted value
struct TuneField {
    const char *name;
    int32_t rsg::Tuning::*f;
    int64_t lo, hi;
};
static const TuneField kTune[] = {
    {"asc_bucket_min", &rsg::Tuning::asc_bucket_min, 32, 1 << 20},
    {"bh_huge", &rsg::Tuning::bh_huge, 4096, 1 << 30},
    {"bh_chunk", &rsg::Tuning::bh_chunk, 1024, 1 << 24},
    {"seg_max", &rsg::Tuning::seg_max, 256, 1 << 24},
    {"norm_chunk", &rsg::Tuning::norm_chunk, 256, 1 << 20},
    {"bp_big", &rsg::Tuning::bp_big, 1024, 1 << 30},
    {"bp_chunk", &rsg::Tuning::bp_chunk, 256, 1 << 20},
};

int32_t rsg_set_tuning(const char *name, int64_t value) {
    for (const TuneField &t : kTune)
        if (name && !strcmp(name, t.name)) {
            if (value < t.lo || value > t.hi) {
                set_error(RSG_ERR_ARGS, "rsg_set_tuning: %s must lie in [%lld, %lld]", t.name,
                          (long long)t.lo, (long long)t.hi);
                return RSG_ERR_ARGS;
            }
            rsg::tuning().*(t.f) = (int32_t)value;
            return RSG_OK;
        }
    set_error(RSG_ERR_ARGS, "rsg_set_tuning: unknown parameter %s", name ? name : "(null)");
    return RSG_ERR_ARGS;
}

int32_t rsg_get_tuning(const char *name, int64_t *value) {
    for (const TuneField &t : kTune)
        if (name && value && !strcmp(name, t.name)) {
            *value = rsg::tuning().*(t.f);
            return RSG_OK;
        }
    set_error(RSG_ERR_ARGS, "rsg_get_tuning: unknown parameter %s", name ? name : "(null)");
    return RSG_ERR_ARGS;
}

int32_t rsg_set_potential_form(int32_t form) {
    if (form < 0 || form > 3) {
        set_error(RSG_ERR_ARGS, "rsg_set_potential_form: form must be 0-3");
        return RSG_ERR_ARGS;
    }
    return rsg::set_batched_potential_form(form);
}

void rsg_debug_keep_potentials(int32_t on) {
    rsg::g_keep_po.store(on != 0);
    if (!on) std::vector<rsg::PotRec>().swap(rsg::g_dbg_po);
}

int64_t rsg_debug_potentials(struct rsg_potential *out, int64_t cap) {
    int64_t k = (int64_t)rsg::g_dbg_po.size();
    if (out && cap > 0) memcpy(out, rsg::g_dbg_po.data(), sizeof(rsg_potential) * (size_t)(k < cap ? k : cap));
    return k;
}

int32_t rsg_keep_halo_records(int32_t on) {
    rsg_debug_keep_potentials(on);
    return RSG_OK;
}

int64_t rsg_halo_records(struct rsg_potential *out, int64_t cap, int64_t *first, int64_t *count,
                         int64_t nh) {
    static const std::vector<rsg::PotRec> none;
    // with the switch off, no thread's records are handed out any more
    const std::vector<rsg::PotRec> &R = rsg::g_keep_po.load() ? rsg::g_dbg_po : none;
    if (nh < 0 || (nh > 0 && (!first || !count))) {
        set_error(RSG_ERR_ARGS, "rsg_halo_records: bad arguments");
        return RSG_ERR_ARGS;
    }
    // a record's halo is its index in the call's halo output (kept in the
    // record's padding); potential-only records carry ke < 0
    auto halo_of = [](const rsg::PotRec &r) {
        int32_t h;
        memcpy(&h, &r.pad, sizeof h);
        return (int64_t)h;
    };
    std::vector<int64_t> c((size_t)(nh > 0 ? nh : 0), 0);
    int64_t total = 0;
    for (const rsg::PotRec &r : R) {
        int64_t h = halo_of(r);
        if (r.ke < 0 || h < 0 || h >= nh) continue;
        c[(size_t)h]++;
        total++;
    }
    if (nh > 0) {
        int64_t at = 0;
        for (int64_t h = 0; h < nh; h++) {
            first[h] = at;
            count[h] = c[(size_t)h];
            at += c[(size_t)h];
        }
    }
    if (out) {
        if (cap < total) {
            set_error(RSG_ERR_ARGS, "rsg_halo_records: %lld records, capacity %lld",
                      (long long)total, (long long)cap);
            return RSG_ERR_ARGS;
        }
        std::vector<int64_t> at(first, first + nh);
        for (const rsg::PotRec &r : R) {
            int64_t h = halo_of(r);
            if (r.ke < 0 || h < 0 || h >= nh) continue;
            memcpy(out + at[(size_t)h]++, &r, sizeof(rsg_potential));
        }
    }
    return total;
}

// Test hook: the subgroup hierarchy of the last rsg_find_subs call on this
// thread: per node its level, size and 6D linking length (normalised units).
int64_t rsg_debug_hierarchy(int32_t *level, int32_t *n, float *target_r, int64_t cap) {
    int64_t k = (int64_t)rsg::g_dbg_level.size();
    for (int64_t i = 0; i < k && i < cap; i++) {
        level[i] = rsg::g_dbg_level[i];
        n[i] = rsg::g_dbg_n[i];
        target_r[i] = rsg::g_dbg_target[i];
    }
    return k;
}

// Test hook: kd-tree permutation of the particle records alone (dim 3 or 6,
// leaf size as given), returned as the permuted array.
int rsg_debug_tree_order(struct rsg_particle *p, int64_t n, int dim, int leaf) {
    try {
        Ctx &C = ctx();
        C.ar.reserve((size_t)n * 200 + (64u << 20));
        C.ar.reset();
        rsg_particle *d_in = C.ar.get<rsg_particle>(n);
        Rec *recs = C.ar.get<Rec>(n);
        RSG_CUDA(cudaMemcpyAsync(d_in, p, sizeof(rsg_particle) * n, cudaMemcpyHostToDevice, C.st));
        std::vector<Rec> h(n);
        std::vector<rsg_particle> hp(p, p + n);
        for (int64_t i = 0; i < n; i++) {
            memcpy(h[i].pos, p[i].pos, sizeof(float) * 6);
            h[i].ridx = (int32_t)i;
            h[i].aux = 0;
        }
        RSG_CUDA(cudaMemcpyAsync(recs, h.data(), sizeof(Rec) * n, cudaMemcpyHostToDevice, C.st));
        int32_t *seg = C.ar.get<int32_t>(2);
        int32_t hs[2] = {0, (int32_t)n};
        RSG_CUDA(cudaMemcpyAsync(seg, hs, sizeof(hs), cudaMemcpyHostToDevice, C.st));
        if (dim == 3) build_forest<3, Rec>(C.ar, recs, n, seg, seg + 1, 1, n, leaf, C.st);
        else build_forest<6, Rec>(C.ar, recs, n, seg, seg + 1, 1, n, leaf, C.st);
        RSG_CUDA(cudaMemcpyAsync(h.data(), recs, sizeof(Rec) * n, cudaMemcpyDeviceToHost, C.st));
        RSG_CUDA(cudaStreamSynchronize(C.st));
        for (int64_t i = 0; i < n; i++) p[i] = hp[h[i].ridx];
        return RSG_OK;
    } catch (Failure &) {
        return error_code();
    }
}

}  // extern "C"
