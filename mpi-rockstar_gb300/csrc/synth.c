/* Seeded synthetic N-body snapshots for the halo-finding workloads.
 *
 * Particles use the reference's own record layout (src/particle.h:5-8):
 * int64 id followed by float pos[6] (x, y, z in Mpc/h; vx, vy, vz in km/s).
 * Every random draw comes from a counter-based generator (SplitMix64 of a
 * (seed, stream, counter) triple), so the output is identical for any thread
 * count and on any host.  Output arrays are id-sorted: particles are
 * shuffled first and then numbered 0..N-1 in array order, so ids carry no
 * information about structure.
 *
 * Workloads (the `cfg` argument); `scale` multiplies the particle count and
 * the number of structures, and the box length by scale^(1/3), so density
 * and linking length stay the same:
 *   1  64^3 particles, 40 Mpc/h box, m_p = 1e9 Msun/h; NFW halos (c = 8,
 *      counts log-uniform in [50, 20000]) are drawn until they hold 70% of
 *      the particles; the rest is a uniform background with 100 km/s
 *      velocities.  Halo bulk velocities are N(0, 300 km/s) per component.
 *   2  128^3 particles, 80 Mpc/h box; hosts with counts from dN/dN ~ N^-1.9
 *      on [20, 2e5], c = 6, drawn until 65% of particles are in hosts; hosts
 *      above 5000 particles carry 0-20 NFW subhalos (1-10% of the host each,
 *      c = 12) at radii drawn from the host profile, moving with a bulk
 *      velocity drawn from the host dispersion; 35% background.
 *   3  isolated groups for the potential/unbinding precision study:
 *      200000 groups with counts from dN/dN ~ N^-1.9 on [20, hi], where
 *      hi = 2e6 at scale 1 and 2e6 * scale (at least 2000) below it, so a
 *      reduced-scale run keeps the expected number of groups near the top
 *      of the range; m_p = 1e9 Msun/h.  Half NFW, half Hernquist (a = r200/c),
 *      c log-uniform in [4, 15], both truncated at r200, one group per cell
 *      of a cubic lattice (cell = 2 r200 of the largest group + 1 Mpc/h), so
 *      no group links to another.  Velocities: bulk N(0, 300 km/s) per
 *      component plus N(0, V200^2/3) per component, except for the first 10%
 *      of each group's particles, which move isotropically at 1.2-3 times the
 *      escape speed of the truncated profile at their radius.  No background.
 *   4  512^3 particles, 500 Mpc/h box; hosts on [20, 5e6] with
 *      c = 10 (N/1e4)^-0.1, subhalos as in 2, 45% background.
 *   5  one NFW host of 2e7 particles (c = 5) with 2000 subhalos (power law on
 *      [20, 2e5], c = 12); the 20 largest carry 5-30 sub-subhalos each; plus
 *      5e6 background particles in a 20 Mpc/h box.
 * Particle masses for 2, 4 and 5 follow the box: m_p = Om rho_c L^3 / N.
 * With scale < 1 the structure counts shrink with it as described above.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

struct particle {
    int64_t id;
    float pos[6];
};

#define RHO_CRIT 2.77519737e11 /* (Msun/h) / (Mpc/h)^3 */
#define GRAV 4.30117902e-9     /* (km/s)^2 Mpc / Msun */
#define OMEGA_M 0.3

static inline uint64_t mix64(uint64_t z) {
    z += 0x9e3779b97f4a7c15ULL;
    z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ULL;
    z = (z ^ (z >> 27)) * 0x94d049bb133111ebULL;
    return z ^ (z >> 31);
}
/* uniform double in (0, 1) for draw `ctr` of stream `stream` */
static inline double u01(uint64_t seed, uint64_t stream, uint64_t ctr) {
    uint64_t z = mix64(seed ^ mix64(stream * 0x632be59bd9b4e019ULL + ctr));
    return ((double)(z >> 11) + 0.5) * (1.0 / 9007199254740992.0);
}
static inline double gauss(uint64_t seed, uint64_t stream, uint64_t ctr) {
    double a = u01(seed, stream, 2 * ctr), b = u01(seed, stream, 2 * ctr + 1);
    return sqrt(-2.0 * log(a)) * cos(2.0 * M_PI * b);
}

/* mass fraction inside x = r/rs for NFW, unnormalised */
static double nfw_m(double x) { return log1p(x) - x / (1.0 + x); }
/* radius (units of rs) enclosing fraction f of the mass inside x = c */
static double nfw_inverse(double f, double c) {
    double y = f * nfw_m(c), lo = 0.0, hi = c, x = 0.5 * c;
    for (int it = 0; it < 60; it++) {
        double g = nfw_m(x) - y;
        if (g > 0) hi = x; else lo = x;
        double d = x / ((1.0 + x) * (1.0 + x));
        double nx = (d > 0) ? x - g / d : 0.5 * (lo + hi);
        if (!(nx > lo && nx < hi)) nx = 0.5 * (lo + hi);
        if (fabs(nx - x) < 1e-13 * (1.0 + x)) { x = nx; break; }
        x = nx;
    }
    return x;
}

struct halo_spec {
    int64_t n;         /* particles */
    int64_t start;     /* first particle slot */
    double cen[3], vel[3];
    double rs, c, sigma; /* scale radius (Mpc/h), concentration, 1D dispersion */
    double r200;
    int prof;          /* 0 NFW, 1 Hernquist (a = r200 / c) */
    int64_t n_fast;    /* leading particles launched above the escape speed */
};

struct synth_plan {
    struct halo_spec *h;
    int64_t nh, cap;
    int64_t n_total, n_struct;
    double box, mp;
    double bg_sigma;
};

static void plan_push(struct synth_plan *pl, struct halo_spec s) {
    if (pl->nh == pl->cap) {
        pl->cap = pl->cap ? 2 * pl->cap : 1024;
        pl->h = (struct halo_spec *)realloc(pl->h, sizeof(*pl->h) * pl->cap);
    }
    pl->h[pl->nh++] = s;
}

static void set_profile(struct halo_spec *s, double mp, double c) {
    double m = (double)s->n * mp;
    s->r200 = cbrt(3.0 * m / (4.0 * M_PI * 200.0 * RHO_CRIT));
    s->c = c;
    s->rs = s->r200 / c;
    s->sigma = sqrt(GRAV * m / s->r200) / sqrt(3.0);
}

static double powerlaw(double u, double a, double b, double alpha) {
    double e = 1.0 - alpha;
    return pow(pow(a, e) + u * (pow(b, e) - pow(a, e)), 1.0 / e);
}

/* position drawn from an NFW profile around `par` (used to place subhalos) */
static void nfw_point(const struct halo_spec *par, uint64_t seed, uint64_t st,
                      uint64_t k, double *out) {
    double x = nfw_inverse(u01(seed, st, 4 * k), par->c) * par->rs;
    double mu = 2.0 * u01(seed, st, 4 * k + 1) - 1.0;
    double ph = 2.0 * M_PI * u01(seed, st, 4 * k + 2);
    double sn = sqrt(fmax(0.0, 1.0 - mu * mu));
    out[0] = par->cen[0] + x * sn * cos(ph);
    out[1] = par->cen[1] + x * sn * sin(ph);
    out[2] = par->cen[2] + x * mu;
}

/* Carve subhalos out of host `hi`: each takes 1-10% of the host's count. */
static void add_subhalos(struct synth_plan *pl, int64_t hi, int nsub_max,
                         double csub, uint64_t seed, uint64_t stream) {
    struct halo_spec host = pl->h[hi];
    int nsub = (int)floor(u01(seed, stream, 0) * (nsub_max + 1));
    int64_t taken = 0;
    for (int k = 0; k < nsub; k++) {
        double frac = 0.01 + 0.09 * u01(seed, stream, 1 + 8 * k);
        int64_t ns = (int64_t)(frac * host.n);
        if (ns < 20 || taken + ns > host.n / 2) continue;
        struct halo_spec s;
        memset(&s, 0, sizeof(s));
        s.n = ns;
        nfw_point(&host, seed, stream * 131 + 7, k, s.cen);
        for (int d = 0; d < 3; d++)
            s.vel[d] = host.vel[d] + host.sigma * gauss(seed, stream * 131 + 9, 8 * k + d);
        set_profile(&s, pl->mp, csub);
        plan_push(pl, s);
        taken += ns;
    }
    pl->h[hi].n -= taken;
}

static void plan_hosts(struct synth_plan *pl, int cfg, double scale, uint64_t seed) {
    double fill, lo, hi, alpha = 1.9;
    int subs = 1;
    if (cfg == 1) { fill = 0.70; lo = 50; hi = 20000; subs = 0; }
    else if (cfg == 2) { fill = 0.65; lo = 20; hi = 2e5; }
    else { fill = 0.55; lo = 20; hi = 5e6; }
    if (hi > pl->n_total * fill * 0.5) hi = pl->n_total * fill * 0.5;
    if (hi < 2 * lo) hi = 2 * lo;
    int64_t target = (int64_t)(fill * pl->n_total), have = 0;
    for (uint64_t k = 0; have < target; k++) {
        double u = u01(seed, 11, k);
        double n = (cfg == 1) ? exp(log(lo) + u * (log(hi) - log(lo)))
                              : powerlaw(u, lo, hi, alpha);
        struct halo_spec s;
        memset(&s, 0, sizeof(s));
        s.n = (int64_t)n;
        if (have + s.n > target) s.n = target - have;
        if (s.n < 1) break;
        for (int d = 0; d < 3; d++) {
            s.cen[d] = pl->box * u01(seed, 12, 3 * k + d);
            s.vel[d] = 300.0 * gauss(seed, 13, 3 * k + d);
        }
        double c = (cfg == 1) ? 8.0 : (cfg == 2) ? 6.0 : 10.0 * pow(s.n / 1e4, -0.1);
        set_profile(&s, pl->mp, c);
        plan_push(pl, s);
        if (subs && s.n > 5000) add_subhalos(pl, pl->nh - 1, 20, 12.0, seed, 1000 + k);
        have += s.n;
    }
    (void)scale;
}

/* Hernquist radius (Mpc/h) enclosing fraction f of the mass inside R = c a */
static double hernquist_inverse(double f, double a, double c) {
    double sr = sqrt(f) * c / (c + 1.0);
    return a * sr / (1.0 - sr);
}

/* escape speed (km/s) at radius r of a profile truncated at r200 */
static double escape_speed(const struct halo_spec *s, double mp, double r) {
    double m = (double)s->n * mp, phi;
    if (r < 1e-6 * s->rs) r = 1e-6 * s->rs;
    if (s->prof == 1) {
        double a = s->rs, R = s->r200, mn = m * (R + a) * (R + a) / (R * R);
        phi = GRAV * mn * (1.0 / (r + a) - a / ((R + a) * (R + a)));
    } else {
        double x = r / s->rs;
        phi = GRAV * m / (s->rs * nfw_m(s->c)) * (log1p(x) / x - 1.0 / (1.0 + s->c));
    }
    return sqrt(2.0 * fmax(phi, 0.0));
}

static void plan_isolated(struct synth_plan *pl, double scale, uint64_t seed) {
    int64_t ng = (int64_t)(200000 * scale + 0.5);
    if (ng < 1) ng = 1;
    double hi = scale >= 1.0 ? 2e6 : fmax(2000.0, 2e6 * scale);
    double rmax = 0;
    for (int64_t k = 0; k < ng; k++) {
        struct halo_spec s;
        memset(&s, 0, sizeof(s));
        s.n = (int64_t)powerlaw(u01(seed, 51, k), 20, hi, 1.9);
        double c = exp(log(4.0) + u01(seed, 52, k) * (log(15.0) - log(4.0)));
        s.prof = u01(seed, 53, k) < 0.5 ? 1 : 0;
        set_profile(&s, pl->mp, c);
        s.n_fast = s.n / 10;
        for (int d = 0; d < 3; d++) s.vel[d] = 300.0 * gauss(seed, 54, 3 * k + d);
        if (s.r200 > rmax) rmax = s.r200;
        plan_push(pl, s);
    }
    double cell = 2.0 * rmax + 1.0;
    int64_t side = 1;
    while (side * side * side < ng) side++;
    pl->box = cell * (double)side;
    for (int64_t k = 0; k < ng; k++) {
        int64_t c[3] = {k % side, (k / side) % side, k / (side * side)};
        for (int d = 0; d < 3; d++) pl->h[k].cen[d] = ((double)c[d] + 0.5) * cell;
    }
}

static void plan_cluster(struct synth_plan *pl, double scale, uint64_t seed) {
    int64_t nhost = (int64_t)(2e7 * scale);
    struct halo_spec host;
    memset(&host, 0, sizeof(host));
    host.n = nhost;
    for (int d = 0; d < 3; d++) host.cen[d] = 0.5 * pl->box;
    set_profile(&host, pl->mp, 5.0);
    plan_push(pl, host);
    int64_t nsubs = (int64_t)(2000 * scale + 0.5);
    if (nsubs < 1) nsubs = 1;
    double shi = 2e5 * scale > 200 ? 2e5 * scale : 200;
    int64_t taken = 0;
    int64_t first_sub = pl->nh;
    for (int64_t k = 0; k < nsubs; k++) {
        struct halo_spec s;
        memset(&s, 0, sizeof(s));
        s.n = (int64_t)powerlaw(u01(seed, 21, k), 20, shi, 1.9);
        if (taken + s.n > nhost / 2) continue;
        nfw_point(&pl->h[0], seed, 22, k, s.cen);
        for (int d = 0; d < 3; d++)
            s.vel[d] = pl->h[0].sigma * gauss(seed, 23, 3 * k + d);
        set_profile(&s, pl->mp, 12.0);
        plan_push(pl, s);
        taken += s.n;
    }
    pl->h[0].n -= taken;
    /* the 20 largest subhalos get 5-30 sub-subhalos each */
    int64_t nsub_real = pl->nh - first_sub;
    int64_t *order = (int64_t *)malloc(sizeof(int64_t) * (nsub_real ? nsub_real : 1));
    for (int64_t i = 0; i < nsub_real; i++) order[i] = first_sub + i;
    for (int64_t i = 0; i < nsub_real && i < 20; i++) {
        int64_t b = i;
        for (int64_t j = i + 1; j < nsub_real; j++)
            if (pl->h[order[j]].n > pl->h[order[b]].n) b = j;
        int64_t t = order[i]; order[i] = order[b]; order[b] = t;
    }
    for (int64_t i = 0; i < nsub_real && i < 20; i++) {
        int64_t si = order[i];
        struct halo_spec par = pl->h[si];
        int nss = 5 + (int)floor(u01(seed, 24, i) * 26);
        int64_t t2 = 0;
        for (int k = 0; k < nss; k++) {
            struct halo_spec s;
            memset(&s, 0, sizeof(s));
            s.n = (int64_t)(par.n * (0.005 + 0.03 * u01(seed, 25 + i, k)));
            if (s.n < 20 || t2 + s.n > par.n / 2) continue;
            nfw_point(&par, seed, 26 + i, k, s.cen);
            for (int d = 0; d < 3; d++)
                s.vel[d] = par.vel[d] + par.sigma * gauss(seed, 60 + i, 3 * k + d);
            set_profile(&s, pl->mp, 15.0);
            plan_push(pl, s);
            t2 += s.n;
        }
        pl->h[si].n -= t2;
    }
    free(order);
}

static int make_plan(struct synth_plan *pl, int cfg, double scale, uint64_t seed) {
    memset(pl, 0, sizeof(*pl));
    if (!(scale > 0)) return -1;
    switch (cfg) {
    case 1: pl->n_total = (int64_t)(262144 * scale); pl->box = 40.0 * cbrt(scale); pl->mp = 1e9; break;
    case 2: pl->n_total = (int64_t)(2097152 * scale); pl->box = 80.0 * cbrt(scale); break;
    case 3: pl->mp = 1e9; plan_isolated(pl, scale, seed); break;
    case 4: pl->n_total = (int64_t)(134217728 * scale); pl->box = 500.0 * cbrt(scale); break;
    case 5: pl->n_total = (int64_t)(2.5e7 * scale); pl->box = 20.0 * cbrt(scale); break;
    default: return -1;
    }
    if (cfg == 3) {
        int64_t s = 0;
        for (int64_t i = 0; i < pl->nh; i++) { pl->h[i].start = s; s += pl->h[i].n; }
        pl->n_struct = pl->n_total = s;
        return 0;
    }
    if (pl->n_total < 1) return -1;
    if (!pl->mp) pl->mp = OMEGA_M * RHO_CRIT * pl->box * pl->box * pl->box / (double)pl->n_total;
    pl->bg_sigma = 100.0;
    if (cfg == 5) plan_cluster(pl, scale, seed);
    else plan_hosts(pl, cfg, scale, seed);
    int64_t s = 0;
    for (int64_t i = 0; i < pl->nh; i++) { pl->h[i].start = s; s += pl->h[i].n; }
    pl->n_struct = s;
    if (s > pl->n_total) return -1;
    return 0;
}

static inline float wrap(double x, double box) {
    double y = fmod(x, box);
    if (y < 0) y += box;
    float f = (float)y;
    if (f >= (float)box) f = 0.0f;
    return f;
}

/* Number of particles that synth_generate writes for (cfg, scale). */
int64_t synth_count(int cfg, double scale, uint64_t seed) {
    struct synth_plan pl;
    if (make_plan(&pl, cfg, scale, seed)) return -1;
    free(pl.h);
    return pl.n_total;
}

/* Fills out[0..n) (n from synth_count) and returns 0.  box_size and
 * particle_mass receive the workload's box length and particle mass;
 * n_halos the number of planted structures (hosts plus subhalos). */
int synth_generate(int cfg, double scale, uint64_t seed, struct particle *out,
                   int64_t n, double *box_size, double *particle_mass,
                   int64_t *n_halos) {
    struct synth_plan pl;
    if (make_plan(&pl, cfg, scale, seed)) return -1;
    if (n != pl.n_total) { free(pl.h); return -2; }
    double box = pl.box;
    /* structured particles */
#pragma omp parallel for schedule(dynamic, 16)
    for (int64_t hi = 0; hi < pl.nh; hi++) {
        const struct halo_spec *s = pl.h + hi;
        uint64_t st = 1000000 + (uint64_t)hi;
        for (int64_t k = 0; k < s->n; k++) {
            double x = s->prof == 1 ? hernquist_inverse(u01(seed, st, 8 * k), s->rs, s->c)
                                    : nfw_inverse(u01(seed, st, 8 * k), s->c) * s->rs;
            double mu = 2.0 * u01(seed, st, 8 * k + 1) - 1.0;
            double ph = 2.0 * M_PI * u01(seed, st, 8 * k + 2);
            double sn = sqrt(fmax(0.0, 1.0 - mu * mu));
            struct particle *q = out + s->start + k;
            q->pos[0] = wrap(s->cen[0] + x * sn * cos(ph), box);
            q->pos[1] = wrap(s->cen[1] + x * sn * sin(ph), box);
            q->pos[2] = wrap(s->cen[2] + x * mu, box);
            if (k < s->n_fast) {
                /* isotropic, 1.2-3x the escape speed at this radius */
                uint64_t sf = 5000000 + (uint64_t)hi;
                double v = (1.2 + 1.8 * u01(seed, sf, 3 * k)) * escape_speed(s, pl.mp, x);
                double vm = 2.0 * u01(seed, sf, 3 * k + 1) - 1.0;
                double vp = 2.0 * M_PI * u01(seed, sf, 3 * k + 2);
                double vs = sqrt(fmax(0.0, 1.0 - vm * vm));
                q->pos[3] = (float)(s->vel[0] + v * vs * cos(vp));
                q->pos[4] = (float)(s->vel[1] + v * vs * sin(vp));
                q->pos[5] = (float)(s->vel[2] + v * vm);
                continue;
            }
            for (int d = 0; d < 3; d++)
                q->pos[3 + d] = (float)(s->vel[d] + s->sigma * gauss(seed, st, 4 * k + 2 + d + 4 * (int64_t)s->n));
        }
    }
    /* uniform background */
#pragma omp parallel for schedule(static)
    for (int64_t k = pl.n_struct; k < n; k++) {
        struct particle *q = out + k;
        for (int d = 0; d < 3; d++) q->pos[d] = wrap(box * u01(seed, 31, 3 * (uint64_t)k + d), box);
        for (int d = 0; d < 3; d++) q->pos[3 + d] = (float)(pl.bg_sigma * gauss(seed, 32, 3 * (uint64_t)k + d));
    }
    /* shuffle (Fisher-Yates on counter draws), then number in array order */
    for (int64_t i = n - 1; i > 0; i--) {
        int64_t j = (int64_t)(u01(seed, 41, (uint64_t)i) * (double)(i + 1));
        if (j > i) j = i;
        struct particle t = out[i]; out[i] = out[j]; out[j] = t;
    }
    for (int64_t i = 0; i < n; i++) out[i].id = i;
    if (box_size) *box_size = box;
    if (particle_mass) *particle_mass = pl.mp;
    if (n_halos) *n_halos = pl.nh;
    free(pl.h);
    return 0;
}
