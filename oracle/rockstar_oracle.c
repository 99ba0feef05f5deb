/* C restatement of MPI-Rockstar's per-group halo-finding hot path.
 *
 * TEST INFRASTRUCTURE ONLY (the oracle): tests/, the smoke check and the CPU
 * baseline of bench.py call this through oracle/restatement.py; the product
 * never links it.  It is sequential C that follows the reference algorithm
 * step by step (citations are file:line in the reference project), so on the
 * same platform it reproduces the reference's output bit for bit, including
 * tree permutations, union-find labels and the glibc rand_r/qsort streams.
 * That equality is pinned by tests/test_oracle_pin.py against the reference
 * sources compiled as-is (oracle/ref).
 *
 * Float/double conversions follow C's usual arithmetic conversions exactly as
 * the reference expressions produce them; the file must be compiled without
 * FMA contraction (-ffp-contract=off).
 */
#include <math.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

/* ---------------------------------------------------------------- records */
struct particle { int64_t id; float pos[6]; };            /* src/particle.h:5-8 */
struct fofrec { int64_t num_p; struct particle *particles; }; /* src/fof.h:7-10 */
struct halo {                                             /* src/halo.h:8-35 */
    int64_t id;
    float pos[6], corevel[3], bulkvel[3];
    float m, r, child_r, vmax_r, mgrav, vmax, rvmax, rs, klypin_rs, vrms, J[3],
        energy, spin, alt_m[4], Xoff, Voff, b_to_a, c_to_a, A[3], b_to_a2,
        c_to_a2, A2[3], bullock_spin, kin_to_pot, m_pe_b, m_pe_d,
        halfmass_radius;
    int64_t num_p, num_child_particles, p_start, desc, flags, n_core;
    float min_pos_err, min_vel_err, min_bulkvel_err;
    float inertia_tensor[6], inertia_tensor2[6];
    float chi2;
};
struct extra { int64_t child, next_cochild, prev_cochild, sub_of, ph; float max_metric; };
struct potential { float pos[6], r2; double pe; float ke; int32_t flags; }; /* src/potential.h:7-21 */
struct metric_pt { float pos[4]; int64_t target; };       /* src/subhalo_metric.h */

#define GROWING 1
#define SKIP_THRESH 16          /* src/rockstar.h:16 */
#define SAMPLE_MAX 10000        /* src/groupies.c:286 */
#define VMAX_BINS 50            /* src/properties.c:1 */
#define GC 4.30117902e-9        /* src/universal_constants.h:4-8 */
#define RHO_C 2.77519737e11
#define VMAX_CONST 6.55833746e-5
#define RMAX_TO_RS 2.1626
#define RS_CONSTANT 0.216216595

/* ----------------------------------------------------------------- config */
struct ocfg {
    double particle_mass, box_size, om, ol, h0, w0, wa;
    double fof_linking_length, fof_fraction, force_res, force_res_phys_max;
    double scale_now, initial_metric_scaling, include_host_potential_ratio;
    double unbound_threshold;
    int64_t min_halo_particles, min_halo_output_size, bound_props;
    int64_t shape_iterations, weighted_shapes, exact_ll_calc, total_particles;
};
static struct ocfg C;
static double avg_spacing;
static double thresh_dens[5], rvir_dens, rvir_dens_z0, dyn_time;
static int64_t min_dens_idx;

/* src/hubble.c:8-19 */
static double weff(double a) { return (a != 1.0) ? C.w0 + C.wa - C.wa * (a - 1.0) / log(a) : C.w0; }
static double hubble_scaling(double z) {
    double z1 = 1.0 + z, a = 1.0 / z1;
    return sqrt(C.om * (z1 * z1 * z1) + C.ol * pow(a, -3.0 * (1.0 + weff(a))));
}
/* src/groupies.c:97-100 */
static double vir_density(double a) {
    double x = (C.om / pow(a, 3)) / pow(hubble_scaling(1.0 / a - 1.0), 2.0) - 1.0;
    return ((18 * M_PI * M_PI + 82.0 * x - 39 * x * x) / (1.0 + x));
}
/* src/groupies.c:102-125 for "<n>b", "<n>c" and "vir" definitions */
static float mass_def(const char *md) {
    float scale = C.scale_now;
    size_t len = strlen(md);
    char last = len ? md[len - 1] : 0;
    float matter_fraction = (C.om / pow(scale, 3)) / pow(hubble_scaling(1.0 / scale - 1.0), 2.0);
    float cons = C.om * RHO_C / C.particle_mass;
    const char *m = md;
    float t;
    if (m[0] == 'm' || m[0] == 'M') m++;
    if (last == 'b' || last == 'B') t = atof(m) * cons;
    else if (last == 'c' || last == 'C') t = atof(m) * cons / matter_fraction;
    else t = vir_density(scale) * cons;
    rvir_dens_z0 = vir_density(1.0) * cons;
    return t;
}

/* Applies the hot-path parameters: src/config.c:17-64 (spacing),
 * src/rockstar.c:58-61 and src/groupies.c:127-142 (density thresholds). */
void oracle_setup(const struct ocfg *q) {
    C = *q;
    if (!C.particle_mass)
        C.particle_mass = RHO_C * C.box_size * C.box_size * C.box_size * C.om / C.total_particles;
    avg_spacing = cbrt(C.particle_mass / (C.om * RHO_C));
    if (!C.force_res_phys_max) C.force_res_phys_max = C.force_res;
    if (C.force_res * C.scale_now > C.force_res_phys_max)
        C.force_res = C.force_res_phys_max / C.scale_now;
    thresh_dens[0] = mass_def("vir");
    thresh_dens[1] = mass_def("200b");
    thresh_dens[2] = mass_def("200c");
    thresh_dens[3] = mass_def("500c");
    thresh_dens[4] = mass_def("2500c");
    rvir_dens = mass_def("vir");
    dyn_time = 1.0 / sqrt((4.0 * M_PI * GC / 3.0) * rvir_dens * C.particle_mass);
    min_dens_idx = 0;
    for (int i = 1; i < 5; i++)
        if (thresh_dens[i] < thresh_dens[min_dens_idx]) min_dens_idx = i;
}
double oracle_avg_spacing(void) { return avg_spacing; }
void oracle_thresholds(double *o) {
    for (int i = 0; i < 5; i++) o[i] = thresh_dens[i];
    o[5] = rvir_dens; o[6] = rvir_dens_z0; o[7] = dyn_time;
}

/* ------------------------------------------------------------ kd-tree ----
 * Median-of-extent BSP tree built in place, as src/fast3tree.c:736-908:
 * each node splits at the float midpoint of its widest dimension with a
 * two-pointer swap partition, children are built left then right, leaves
 * hold at most `leaf` points.  Records are moved as raw bytes, so one
 * implementation serves particles (6D / 3D), potentials and halo metrics. */
struct knode {
    float min[6], max[6];
    int64_t start, n;
    int div;
    int64_t left, right, parent;
    float mc[3], m, dmin;         /* potential tree extras (src/potential.c:60-63) */
};
struct ktree {
    char *base; size_t stride, off; int dim, leaf;
    int64_t n;
    struct knode *nd; int64_t nn, cap;
};
static inline float *kpos(const struct ktree *t, int64_t i) { return (float *)(t->base + (size_t)i * t->stride + t->off); }
static void kswap(struct ktree *t, int64_t a, int64_t b) {
    char tmp[64];
    char *pa = t->base + (size_t)a * t->stride, *pb = t->base + (size_t)b * t->stride;
    memcpy(tmp, pa, t->stride); memcpy(pa, pb, t->stride); memcpy(pb, tmp, t->stride);
}
/* src/fast3tree.c:778-794 */
static void kminmax(struct ktree *t, struct knode *nd) {
    float *p0 = kpos(t, nd->start);
    for (int j = 0; j < t->dim; j++) nd->min[j] = nd->max[j] = p0[j];
    for (int64_t i = 1; i < nd->n; i++) {
        float *q = kpos(t, nd->start + i);
        for (int j = 0; j < t->dim; j++) {
            float x = q[j];
            if (x < nd->min[j]) nd->min[j] = x;
            else if (x > nd->max[j]) nd->max[j] = x;
        }
    }
}
static int64_t knew(struct ktree *t) {
    if (t->nn == t->cap) { t->cap = t->cap * 2 + 64; t->nd = realloc(t->nd, sizeof(struct knode) * t->cap); }
    memset(t->nd + t->nn, 0, sizeof(struct knode));
    return t->nn++;
}
/* split: src/fast3tree.c:736-774 (widest dim, ties to the lowest index after
 * the last dim is taken as the starting candidate) and :798-846 */
static void ksplit(struct ktree *t, int64_t ni) {
    struct knode *nd = t->nd + ni;
    int dim = t->dim - 1;
    float d = nd->max[t->dim - 1] - nd->min[t->dim - 1];
    for (int i = 0; i < t->dim - 1; i++) {
        float d2 = nd->max[i] - nd->min[i];
        if (d2 > d) { d = d2; dim = i; }
    }
    nd->div = dim;
    int64_t nl;
    if (nd->max[dim] == nd->min[dim]) nl = nd->n;
    else {
        float lim = 0.5 * (nd->max[dim] + nd->min[dim]);
        int64_t i, j = nd->n - 1, s = nd->start;
        for (i = 0; i < j; i++) {
            if (kpos(t, s + i)[dim] > lim) { kswap(t, s + i, s + j); i--; j--; }
        }
        if (i == j && kpos(t, s + i)[dim] <= lim) i++;
        nl = i;
    }
    if (nl == nd->n || nl == 0) { nd->div = -1; return; }
    int64_t l = knew(t), r = knew(t);
    nd = t->nd + ni;
    nd->left = l; nd->right = r;
    struct knode *L = t->nd + l, *R = t->nd + r;
    L->parent = R->parent = ni;
    L->div = R->div = -1;
    L->start = nd->start; L->n = nl;
    R->start = nd->start + nl; R->n = nd->n - nl;
    kminmax(t, L); kminmax(t, R);
    if (t->nd[l].n > t->leaf) ksplit(t, l);
    if (t->nd[r].n > t->leaf) ksplit(t, r);
}
/* src/fast3tree.c:865-908 (inputs are finite here, so the NaN sweep of
 * :876-887 never moves anything) */
static void kbuild(struct ktree *t, void *base, size_t stride, size_t off, int dim, int leaf, int64_t n) {
    t->base = base; t->stride = stride; t->off = off; t->dim = dim; t->leaf = leaf; t->n = n;
    t->nn = 0;
    int64_t r = knew(t);
    t->nd[r].start = 0; t->nd[r].n = n; t->nd[r].div = -1; t->nd[r].parent = -1;
    if (n) kminmax(t, t->nd + r);
    if (n > leaf) ksplit(t, r);
}
static void kfree(struct ktree *t) { free(t->nd); memset(t, 0, sizeof(*t)); }

/* result list of record indices */
struct ilist { int64_t *v; int64_t n, cap; };
static inline void ipush(struct ilist *l, int64_t x) {
    if (l->n == l->cap) { l->cap = l->cap * 2 + 256; l->v = realloc(l->v, sizeof(int64_t) * l->cap); }
    l->v[l->n++] = x;
}

/* src/fast3tree.c:293-311 */
static int box_outside(const struct knode *nd, const float *c, float r, int dim) {
    float d = 0, e; const float r2 = r * r;
    for (int i = 0; i < dim; i++) {
        if ((e = c[i] - nd->min[i]) < 0) { d += e * e; if (d >= r2) return 1; }
        else if ((e = c[i] - nd->max[i]) > 0) { d += e * e; if (d >= r2) return 1; }
    }
    return 0;
}
/* src/fast3tree.c:317-335 */
static int box_inside(const struct knode *nd, const float *c, float r, int dim) {
    float dx, dx2, dist = 0, r2 = r * r;
    if (fabs(c[0] - nd->min[0]) > r) return 0;
    for (int i = 0; i < dim; i++) {
        dx = nd->min[i] - c[i]; dx *= dx;
        dx2 = c[i] - nd->max[i]; dx2 *= dx2;
        if (dx2 > dx) dx = dx2;
        dist += dx;
        if (dist > r2) return 0;
    }
    return 1;
}
static inline float dist2f(const float *c, const float *p, int dim) {
    float d = 0, dx;
    for (int j = 0; j < dim; j++) { dx = c[j] - p[j]; d += dx * dx; }
    return d;
}
/* sphere search, src/fast3tree.c:377-414; `from` > -1 gives the skip variant
 * of :419-465 (only records at index >= from, with `from` itself first) */
static void ksphere(const struct ktree *t, int64_t ni, const float *c, float r,
                    int64_t from, struct ilist *res) {
    const struct knode *nd = t->nd + ni;
    if (from >= 0 && nd->start + nd->n <= from) return;
    if (box_outside(nd, c, r, t->dim)) return;
    if (t->dim < 6 && box_inside(nd, c, r, t->dim)) {
        for (int64_t i = 0; i < nd->n; i++) ipush(res, nd->start + i);
        return;
    }
    if (nd->div < 0) {
        float r2 = r * r;
        int64_t i = 0;
        if (from >= 0 && nd->start < from) { ipush(res, from); i = from - nd->start + 1; }
        for (; i < nd->n; i++)
            if (dist2f(c, kpos(t, nd->start + i), t->dim) < r2) ipush(res, nd->start + i);
        return;
    }
    ksphere(t, nd->left, c, r, from, res);
    ksphere(t, nd->right, c, r, from, res);
}
/* src/fast3tree.c:956-987 */
static float knext_rec(const struct ktree *t, int64_t ni, const float *c, float r, int64_t skip) {
    const struct knode *nd = t->nd + ni;
    if (box_outside(nd, c, r, t->dim) || skip == ni) return r;
    if (nd->div < 0) {
        float r2 = r * r;
        for (int64_t i = 0; i < nd->n; i++) {
            float d = dist2f(c, kpos(t, nd->start + i), t->dim);
            if (d < r2) r2 = d;
        }
        return sqrt(r2);
    }
    int64_t a = nd->left, b = nd->right;
    if (c[nd->div] > 0.5 * (nd->min[nd->div] + nd->max[nd->div])) { a = nd->right; b = nd->left; }
    r = knext_rec(t, a, c, r, skip);
    return knext_rec(t, b, c, r, skip);
}
/* src/fast3tree.c:992-1030 */
static float knext(const struct ktree *t, const float *c) {
    int64_t ni = 0;
    while (t->nd[ni].div >= 0)
        ni = (c[t->nd[ni].div] <= t->nd[t->nd[ni].left].max[t->nd[ni].div]) ? t->nd[ni].left : t->nd[ni].right;
    while (ni != 0 && t->nd[ni].min[t->nd[t->nd[ni].parent].div] == t->nd[ni].max[t->nd[t->nd[ni].parent].div])
        ni = t->nd[ni].parent;
    const struct knode *nd = t->nd + ni;
    float md = 0, dx;
    for (int j = 0; j < t->dim; j++) { dx = nd->max[j] - nd->min[j]; md += dx * dx; }
    for (int64_t i = 0; i < nd->n; i++) {
        float d = dist2f(c, kpos(t, nd->start + i), t->dim);
        if (d && d < md) md = d;
    }
    return knext_rec(t, 0, c, sqrt(md), ni);
}

/* ------------------------------------------------------------ union-find --
 * Labels follow src/fof.c:46-170: a new set takes the next integer; when a
 * link's set meets the current set, the link's root survives. */
struct uf { int64_t *root; int64_t n, cap; };
static int64_t uf_new(struct uf *u) {
    if (u->n == u->cap) { u->cap = u->cap * 2 + 1024; u->root = realloc(u->root, sizeof(int64_t) * u->cap); }
    u->root[u->n] = u->n;
    return u->n++;
}
static inline int64_t uf_find(struct uf *u, int64_t a) {
    int64_t r = a;
    while (u->root[r] != r) r = u->root[r];
    while (u->root[a] != r) { int64_t nx = u->root[a]; u->root[a] = r; a = nx; }
    return r;
}
/* merge(link set, current set): root of the link's set survives */
static inline void uf_merge(struct uf *u, int64_t link, int64_t cur) {
    int64_t rl = uf_find(u, link), rc = uf_find(u, cur);
    if (rl != rc) u->root[rc] = rl;
}
/* src/fof.c:112-140 */
static void link_particle(int64_t *lab, struct uf *u, int64_t self, const struct ilist *l) {
    if (l->n < 2) return;
    int64_t f = lab[self];
    if (f < 0) {
        for (int64_t i = 0; i < l->n; i++) if (lab[l->v[i]] != -1) { f = lab[l->v[i]]; break; }
        if (f < 0) f = uf_new(u);
    }
    for (int64_t i = 0; i < l->n; i++) {
        int64_t j = l->v[i];
        if (lab[j] == -1) lab[j] = f;
        else uf_merge(u, lab[j], f);
    }
}
/* src/fof.c:142-158 */
static void link_groups(int64_t *lab, struct uf *u, int64_t self, const struct ilist *l) {
    int64_t f = lab[self];
    if (l->n < 2 || f < 0) return;
    for (int64_t i = 0; i < l->n; i++) {
        int64_t j = l->v[i];
        if (lab[j] == -1 || lab[j] == f) continue;
        uf_merge(u, lab[j], f);
    }
}

/* src/fof.c:184-224: recursive two-pointer partition on label midpoints */
static void partition_sort(int64_t lo, int64_t hi, struct particle *pa, int64_t *lab) {
    while (hi - lo >= 2) {
        int64_t mn = lab[lo], mx = lab[lo];
        for (int64_t i = lo + 1; i < hi; i++) { if (lab[i] > mx) mx = lab[i]; if (lab[i] < mn) mn = lab[i]; }
        if (mn == mx) return;
        int64_t piv = mn + (mx - mn) / 2, si = hi - 1, i;
        for (i = lo; i < si; i++)
            if (lab[i] > piv) {
                struct particle tp = pa[i]; pa[i] = pa[si]; pa[si] = tp;
                int64_t tl = lab[i]; lab[i] = lab[si]; lab[si] = tl;
                si--; i--;
            }
        if (i == si && lab[si] <= piv) si++;
        partition_sort(lo, si, pa, lab);
        lo = si;
    }
}

/* src/fof.c:226-255 (no boundary groups: rockstar() is run with bounds ==
 * NULL).  Emits (offset, size) of every kept group into offs and sizes. */
static int64_t full_groups(int64_t n, struct particle *pa, int64_t *lab, struct uf *u,
                           int64_t **offs, int64_t **sizes) {
    for (int64_t i = 0; i < n; i++) if (lab[i] >= 0) lab[i] = uf_find(u, lab[i]);
    partition_sort(0, n, pa, lab);
    int64_t nf = 0, cap = 0, f = -1, last = -1, i;
    int64_t *o = NULL, *s = NULL;
    for (i = 0; i < n; i++) {
        if (lab[i] < 0) continue;
        int64_t sf = lab[i];
        if (sf != last) {
            if (f > -1) s[f] = i - o[f];
            if (f < 0 || s[f] >= C.min_halo_particles) {
                if (nf == cap) { cap = cap * 2 + 64; o = realloc(o, sizeof(int64_t) * cap); s = realloc(s, sizeof(int64_t) * cap); }
                f = nf++;
            }
            o[f] = i;
            last = sf;
        }
    }
    if (f > -1) {
        s[f] = i - o[f];
        if (s[f] < C.min_halo_particles) nf--;
    }
    *offs = o; *sizes = s;
    return nf;
}

/* ------------------------------------------------------------ 3D FOF ----
 * rockstar(NULL, 1), src/rockstar.c:53-128 with build_particle_tree
 * (:368-397).  `pa` is permuted in place; returns the new particle count
 * through np and the groups through offs and sizes. */
int64_t oracle_fof(struct particle *pa, int64_t *np, int64_t **offs, int64_t **sizes) {
    int64_t n = *np;
    float r = avg_spacing * C.fof_linking_length;
    struct ktree t = {0};
    kbuild(&t, pa, sizeof(struct particle), 8, 3, 20, n);
    if (n >= 2) { /* duplicate removal against the last kept particle, backwards */
        int64_t last = n - 1, dups = 0;
        for (int64_t i = n - 2; i >= 0; i--) {
            if (!memcmp(pa[i].pos, pa[last].pos, sizeof(float) * 6) || pa[last].id == pa[i].id) {
                n--; pa[i] = pa[n]; dups++; continue;
            }
            last = i;
        }
        if (dups) { kfree(&t); kbuild(&t, pa, sizeof(struct particle), 8, 3, 20, n); }
    }
    int64_t *lab = malloc(sizeof(int64_t) * (n ? n : 1));
    char *skip = calloc(n ? n : 1, 1);
    for (int64_t i = 0; i < n; i++) lab[i] = -1;
    struct uf u = {0};
    struct ilist res = {0};
    for (int64_t i = 0; i < n; i++) {
        if (skip[i]) continue;
        res.n = 0;
        ksphere(&t, 0, pa[i].pos, r, -1, &res);
        link_particle(lab, &u, i, &res);
        if (res.n > SKIP_THRESH) {
            for (int64_t j = 0; j < res.n; j++) skip[res.v[j]] = 1;
            res.n = 0;
            ksphere(&t, 0, pa[i].pos, 2.0 * r, -1, &res);
            link_groups(lab, &u, i, &res);
        }
    }
    kfree(&t);
    int64_t nf = full_groups(n, pa, lab, &u, offs, sizes);
    free(lab); free(skip); free(u.root); free(res.v);
    *np = n;
    return nf;
}
void oracle_free(void *p) { free(p); }

/* ======================================================= find_subs state */
struct hinfo { struct halo *h; struct extra *e; int64_t n, cap; };
static struct particle *P;          /* the caller's particle array (global p) */
static struct particle *cp;         /* copies, src/groupies.c:30 */
static int64_t *phalo;              /* particle_halos */
static float *prad;                 /* particle_r */
static struct potential *po;
static int64_t ncopies;
static struct fofrec *subf; static int64_t nsubf, capsubf;
static int64_t *gh; static int64_t ngh, capgh;           /* growing halos */
static struct metric_pt *mpts; static int64_t capm;
static struct ktree mtree;                                 /* 4D halo metric tree */
static int64_t *hids; static int64_t caphids;

/* src/groupies.c:164-187 */
static void add_halo(struct hinfo *hi) {
    if (hi->n == hi->cap) {
        hi->cap = hi->cap * 2 + 1000;
        hi->h = realloc(hi->h, sizeof(struct halo) * hi->cap);
        hi->e = realloc(hi->e, sizeof(struct extra) * hi->cap);
    }
    memset(hi->h + hi->n, 0, sizeof(struct halo));
    hi->h[hi->n].flags = GROWING;
    struct extra *e = hi->e + hi->n;
    e->child = e->next_cochild = e->ph = e->prev_cochild = e->sub_of = -1;
    e->max_metric = 0;
    hi->n++;
}

/* src/jacobi.c:9-138 (cyclic Jacobi with the 1e-6 change rule; the rotation
 * scalars use long double as the source does) */
static void jacobi(double a[][3], double *eig, double v[][3]) {
    int i, j, k, l, maxc[3], chg[3], n = 3, state = 0, mr;
    double mx, c, s, t, u, w;
    for (i = 0; i < n; i++) {
        mx = 0; maxc[i] = i + 1;
        for (j = i + 1; j < n; j++) if (fabs(a[i][j]) > mx) { maxc[i] = j; mx = fabs(a[i][j]); }
    }
    for (i = 0; i < n; i++) for (j = 0; j < n; j++) v[i][j] = (i == j) ? 1 : 0;
    for (i = 0; i < n; i++) {
        eig[i] = a[i][i]; chg[i] = 1;
        for (j = 0; j < n; j++) if (j != i && a[i][j]) break;
        if (j == n) { state--; chg[i] = 0; }
    }
    state += n;
    while (state) {
        mx = fabs(a[0][maxc[0]]); mr = 0;
        for (i = 1; i < n - 1; i++) if (fabs(a[i][maxc[i]]) > mx) { mx = fabs(a[i][maxc[i]]); mr = i; }
        k = mr; l = maxc[k]; mx = a[k][l];
        if (mx == 0) break;
        w = (eig[l] - eig[k]) * 0.5;
        t = fabsl(w) + sqrtl(mx * mx + w * w);
        s = sqrtl(mx * mx + t * t);
        c = t / s; s = mx / s; t = mx * mx / t;
        if (w < 0) { s = -s; t = -t; }
#define UPD(x, y) do { double yy = (y); eig[x] += yy; \
        if (chg[x] && (fabs(yy) < 1e-6 * fabs(eig[x]))) { chg[x] = 0; state--; } \
        else if (!chg[x] && (fabs(yy) > 1e-6 * fabs(eig[x]))) { chg[x] = 1; state++; } } while (0)
        UPD(k, -t);
        UPD(l, t);
#undef UPD
        a[k][l] = 0;
#define ROT(m, p1, q1, p2, q2, upd) do { t = m[p1][q1]; u = m[p2][q2]; \
        m[p1][q1] = t * c - s * u; m[p2][q2] = s * t + c * u; \
        if (upd) { if (fabs(m[p1][q1]) > fabs(m[p1][maxc[p1]])) maxc[p1] = q1; \
                   if (p2 < 3 && fabs(m[p2][q2]) > fabs(m[p2][maxc[p2]])) maxc[p2] = q2; } } while (0)
        for (i = 0; i < k; i++) ROT(a, i, k, i, l, 1);
        for (i = k + 1; i < l; i++) ROT(a, k, i, i, l, 1);
        for (i = l + 1; i < n; i++) ROT(a, k, i, l, i, 1);
        for (i = 0; i < n; i++) ROT(v, k, i, l, i, 0);
#undef ROT
    }
    for (k = 0; k < n - 1; k++) for (l = k + 1; l < n; l++) a[k][l] = a[l][k];
}
/* src/jacobi.c:140-172 */
static void min_eig_sqrt(double in[][3], double *res) {
    double v[3][3], e[3];
    jacobi(in, e, v);
    *res = e[0];
    if (e[1] < *res) *res = e[1];
    if (e[2] < *res) *res = e[2];
    if (*res <= 0) *res = sqrt(in[0][0] + in[1][1] + in[2][2]);
    else *res = sqrt(*res);
}

/* norm_sd, src/groupies.c:788-830 */
static void norm_sd(struct particle *pa, int64_t n) {
    double mean[6] = {0}, corr[6][6], sx, sv;
    if (!n) return;
    for (int64_t i = 0; i < n; i++) for (int j = 0; j < 6; j++) mean[j] += pa[i].pos[j];
    for (int j = 0; j < 6; j++) mean[j] /= (double)n;
    memset(corr, 0, sizeof(corr));
    for (int64_t i = 0; i < n; i++) {
        for (int j = 0; j < 6; j++) pa[i].pos[j] -= mean[j];
        for (int j = 0; j < 6; j++) for (int k = j; k < 6; k++) corr[j][k] += pa[i].pos[j] * pa[i].pos[k];
    }
    for (int j = 0; j < 6; j++) for (int k = j; k < 6; k++) corr[j][k] /= (double)n;
    for (int i = 0; i < 6; i++) for (int j = 0; j < i; j++) corr[i][j] = corr[j][i];
    double in[3][3];
    for (int i = 0; i < 3; i++) for (int j = 0; j < 3; j++) in[i][j] = corr[i][j];
    min_eig_sqrt(in, &sx);
    for (int i = 0; i < 3; i++) for (int j = 0; j < 3; j++) in[i][j] = corr[i + 3][j + 3];
    min_eig_sqrt(in, &sv);
    if (n == ncopies) sx *= C.initial_metric_scaling;
    if (!sx || !sv) return;
    for (int64_t i = 0; i < n; i++) for (int j = 0; j < 6; j++) pa[i].pos[j] /= ((j < 3) ? sx : sv);
}

/* src/groupies.c:735-786 */
static float unit_r(unsigned *seed) { return ((float)(rand_r(seed) % (RAND_MAX)) / (float)(RAND_MAX)); }
static int64_t rpart(float *a, int64_t left, int64_t right, int64_t pi) {
    float piv = a[pi], t;
    int64_t si, i;
    t = a[pi]; a[pi] = a[right - 1]; a[right - 1] = t;
    si = right - 2;
    for (i = left; i < si; i++)
        if (a[i] > piv) { t = a[i]; a[i] = a[si]; a[si] = t; si--; i--; }
    if (a[si] <= piv) si++;
    t = a[right - 1]; a[right - 1] = a[si]; a[si] = t;
    return si;
}
static float kth_radius(float *a, int64_t n, float frac, unsigned *seed) {
    int64_t k = n * frac, left = 0, right = n, pi;
    if (n < 2) return a[0];
    while (1) {
        pi = rpart(a, left, right, left + unit_r(seed) * (right - left));
        if (k == pi || (a[left] == a[right - 1])) return a[k];
        if (k < pi) right = pi; else left = pi + 1;
    }
}

static struct ktree ptree6;
/* test hook: (level, n, target_r) of every 6D FOF call, in call order */
static int64_t *rec_level, *rec_n; static float *rec_tr; static int64_t rec_cnt, rec_cap, cur_level;
static void rec_push(int64_t n, float tr) {
    if (rec_cnt == rec_cap) { rec_cap = rec_cap * 2 + 1024;
        rec_level = realloc(rec_level, 8 * rec_cap); rec_n = realloc(rec_n, 8 * rec_cap);
        rec_tr = realloc(rec_tr, 4 * rec_cap); }
    rec_level[rec_cnt] = cur_level; rec_n[rec_cnt] = n; rec_tr[rec_cnt] = tr; rec_cnt++;
}
int64_t oracle_hierarchy(int64_t *level, int64_t *n, float *tr, int64_t cap) {
    for (int64_t i = 0; i < rec_cnt && i < cap; i++) { level[i] = rec_level[i]; n[i] = rec_n[i]; tr[i] = rec_tr[i]; }
    return rec_cnt;
}
static struct ilist qres;
static struct uf fuf;

/* _find_subfofs_better2 + _find_subfofs_at_r, src/groupies.c:274-314.
 * Appends the kept subgroups to subf[]. */
static void find_subgroups(struct fofrec *f, float thresh, float *target_out) {
    int64_t n = f->num_p, nt = SAMPLE_MAX, j;
    struct particle *pa = f->particles;
    if (C.exact_ll_calc) nt = n;
    norm_sd(pa, n);
    kfree(&ptree6);
    kbuild(&ptree6, pa, sizeof(struct particle), 8, 6, 40, n);
    if (nt > n) nt = n;
    unsigned seed = (unsigned)n;
    for (int64_t i = 0; i < nt; i++) {
        if (nt == n) j = i;
        else {
            j = rand_r(&seed); j <<= 31; j += rand_r(&seed); j %= n;
        }
        prad[i] = knext(&ptree6, pa[j].pos);
    }
    float tr = kth_radius(prad, nt, thresh, &seed);
    if (target_out) *target_out = tr;
    rec_push(n, tr);
    /* 6D FOF at tr: every particle links to itself and later neighbours */
    int64_t *lab = malloc(sizeof(int64_t) * (n ? n : 1));
    for (int64_t i = 0; i < n; i++) lab[i] = -1;
    fuf.n = 0;
    for (int64_t i = 0; i < n; i++) {
        qres.n = 0;
        ksphere(&ptree6, 0, pa[i].pos, tr, i, &qres);
        link_particle(lab, &fuf, i, &qres);
    }
    int64_t *o, *s;
    int64_t nf = full_groups(n, pa, lab, &fuf, &o, &s);
    for (int64_t k = 0; k < nf; k++) {
        if (nsubf == capsubf) { capsubf = capsubf * 2 + 1000; subf = realloc(subf, sizeof(struct fofrec) * capsubf); }
        subf[nsubf].num_p = s[k];
        subf[nsubf].particles = pa + o[k];
        nsubf++;
    }
    free(o); free(s); free(lab);
}

/* calc_particle_dist, src/subhalo_metric.c:51-65 */
static float pdist(const struct halo *h, const float *pos) {
    float dx, r2 = 0, v2 = 0;
    int i;
    if (h->vrms <= 0 || h->r <= 0) return 1e20;
    for (i = 0; i < 3; i++) { dx = h->pos[i] - pos[i]; r2 += dx * dx; }
    for (; i < 6; i++) { dx = h->bulkvel[i - 3] - pos[i]; v2 += dx * dx; }
    return sqrt((r2 / (h->r * h->r)) + v2 / (h->vrms * h->vrms));
}
/* src/subhalo_metric.c:67-77 */
static float hdist_raw(const struct halo *h1, const struct halo *h2) { return pdist(h1, h2->pos); }
static float hdist(const struct halo *h1, const struct halo *h2) {
    if (h2->r > h1->r * 0.99999) return 1e20;
    return hdist_raw(h1, h2);
}

/* build_subtree, src/subhalo_metric.c:24-43 */
static void build_metric_tree(struct hinfo *hi, int64_t *list, int64_t n) {
    if (n > capm) { capm = n; mpts = realloc(mpts, sizeof(struct metric_pt) * capm); }
    for (int64_t i = 0; i < n; i++) {
        struct halo *h = hi->h + list[i];
        memcpy(mpts[i].pos, h->pos, sizeof(float) * 3);
        mpts[i].pos[3] = h->r * (1.0 / -0.2);
        mpts[i].target = list[i];
    }
    kfree(&mtree);
    kbuild(&mtree, mpts, sizeof(struct metric_pt), 0, 4, 10, n);
}
/* src/subhalo_metric.c:79-109,144-149 */
static int64_t best_halo_rec(struct hinfo *hi, int64_t ni, const float *pos, float *best, int64_t bh) {
    const struct knode *nd = mtree.nd + ni;
    if (nd->div < 0) {
        for (int64_t i = 0; i < nd->n; i++) {
            const struct metric_pt *m = mpts + nd->start + i;
            float met = pdist(hi->h + m->target, pos);
            if (met < *best) { *best = met; bh = m->target; }
        }
        return bh;
    }
    for (int side = 0; side < 2; side++) {
        const struct knode *ch = mtree.nd + (side ? nd->right : nd->left);
        float max_r = ch->min[3] * *best * -0.2;
        int ok = 1;
        for (int i = 0; i < 3; i++)
            if ((pos[i] + max_r < ch->min[i]) || (pos[i] - max_r > ch->max[i])) { ok = 0; break; }
        if (ok) bh = best_halo_rec(hi, side ? nd->right : nd->left, pos, best, bh);
    }
    return bh;
}
static int64_t best_halo(struct hinfo *hi, const float *pos, int64_t start) {
    float best = pdist(hi->h + start, pos);
    return best_halo_rec(hi, 0, pos, &best, start);
}
/* src/subhalo_metric.c:151-191 */
static int64_t best_parent_rec(struct hinfo *hi, int64_t ni, const struct halo *h, float *best, int64_t bh) {
    const struct knode *nd = mtree.nd + ni;
    if (nd->div < 0) {
        for (int64_t i = 0; i < nd->n; i++) {
            const struct metric_pt *m = mpts + nd->start + i;
            float met = hdist(hi->h + m->target, h);
            if (met < *best) { *best = met; bh = m->target; }
        }
        return bh;
    }
    for (int side = 0; side < 2; side++) {
        const struct knode *ch = mtree.nd + (side ? nd->right : nd->left);
        float rr = ch->min[3] * -0.2;
        float max_r = rr * *best;
        int ok = 1;
        if (rr < h->r * 1.00001) ok = 0;
        for (int i = 0; ok && i < 3; i++)
            if ((h->pos[i] + max_r < ch->min[i]) || (h->pos[i] - max_r > ch->max[i])) ok = 0;
        if (ok) bh = best_parent_rec(hi, side ? nd->right : nd->left, h, best, bh);
    }
    return bh;
}
static int64_t best_parent(struct hinfo *hi, int64_t h, int64_t biggest) {
    if (h == biggest) return h;
    float best = hdist(hi->h + biggest, hi->h + h);
    return best_parent_rec(hi, 0, hi->h + h, &best, biggest);
}

/* estimate_vmax (children = 0), src/properties.c:12-69 */
static void estimate_vmax(struct halo *h) {
    int64_t bins[VMAX_BINS] = {0};
    h->vmax = h->vmax_r = 0;
    if (!(h->child_r > 0)) return;
    float rsc = ((double)VMAX_BINS) / h->child_r;
    for (int64_t i = 0; i < h->num_p; i++) {
        float ds = 0, dx;
        for (int j = 0; j < 3; j++) { dx = h->pos[j] - cp[h->p_start + i].pos[j]; ds += dx * dx; }
        int64_t b = sqrt(ds) * rsc;
        if (b >= VMAX_BINS) continue;
        bins[b]++;
    }
    float vm = 0, vc, r;
    int64_t tp = 0;
    for (int i = 0; i < VMAX_BINS; i++) {
        r = (i + 1.0) / rsc;
        if (r < C.force_res) r = C.force_res;
        tp += bins[i];
        vc = tp / r;
        if (vc > vm) vm = vc;
    }
    float sn = C.scale_now;
    float v = sqrt(GC * vm * C.particle_mass / sn);
    h->vmax = v;
    h->vmax_r = sqrt(sn) * v * dyn_time;
}
/* calc_basic_halo_props, src/properties.c:71-125 */
static void basic_props(struct halo *h) {
    double pos[6] = {0}, pos2[6] = {0}, x, pe, ve;
    h->r = h->vrms = 0;
    for (int64_t j = 0; j < h->num_p; j++) for (int k = 0; k < 6; k++) pos[k] += cp[h->p_start + j].pos[k];
    for (int k = 0; k < 6; k++) pos[k] /= (double)h->num_p;
    for (int64_t j = 0; j < h->num_p; j++)
        for (int k = 0; k < 6; k++) { x = cp[h->p_start + j].pos[k] - pos[k]; pos2[k] += x * x; }
    for (int k = 0; k < 6; k++) {
        if (k < 3) h->r += pos2[k] / (double)h->num_p;
        else h->vrms += pos2[k] / (double)h->num_p;
    }
    pe = h->r / (double)h->num_p;
    ve = h->vrms / (double)h->num_p;
    if ((!h->min_pos_err) || (h->min_pos_err > pe)) {
        h->min_pos_err = pe; h->n_core = h->num_p;
        for (int k = 0; k < 3; k++) h->pos[k] = pos[k];
    }
    if ((!h->min_vel_err) || (h->min_vel_err > ve)) {
        h->min_vel_err = ve;
        for (int k = 3; k < 6; k++) h->pos[k] = pos[k];
    }
    for (int k = 3; k < 6; k++) h->bulkvel[k - 3] = pos[k];
    h->m = h->num_p;
    if (!h->num_child_particles) h->num_child_particles = h->num_p;
    h->r = cbrt(h->num_p / ((4.0 * M_PI / 3.0) * rvir_dens));
    h->child_r = cbrt(h->num_child_particles / ((4.0 * M_PI / 3.0) * rvir_dens));
    estimate_vmax(h);
    if (h->vmax_r) h->r = h->vmax_r;
    h->vrms = sqrt(h->vrms);
}
/* src/properties.c:139-163 */
static void nchild_rec(struct hinfo *hi, int64_t h) {
    if (hi->h[h].num_child_particles) return;
    hi->h[h].num_child_particles = hi->h[h].num_p;
    for (int64_t c = hi->e[h].child; c > -1; c = hi->e[c].next_cochild) {
        nchild_rec(hi, c);
        hi->h[h].num_child_particles += hi->h[c].num_child_particles;
    }
}
static void calc_nchild(struct hinfo *hi, int64_t h0) {
    for (int64_t i = h0; i < hi->n; i++) hi->h[i].num_child_particles = 0;
    for (int64_t i = h0; i < hi->n; i++) if (!hi->h[i].num_child_particles) nchild_rec(hi, i);
}
/* could_be_poisson_or_force_res, src/groupies.c:333-360 */
static int poisson_or_force(const struct halo *h1, const struct halo *h2, int *force) {
    float dx, r = 0, v = 0, mpe, mve;
    *force = 0;
    if (!h1->min_pos_err || !h1->min_vel_err) return 1;
    for (int k = 0; k < 3; k++) {
        dx = h1->pos[k] - h2->pos[k]; r += dx * dx;
        dx = h1->pos[k + 3] - h2->pos[k + 3]; v += dx * dx;
    }
    mpe = h1->min_pos_err; mve = h1->min_vel_err;
    dx = (r / mpe + v / mve) / 2.0;
    if (!(dx > 100)) return 1;
    r = sqrt(r); v = sqrt(v);
    if ((h1->r + h2->r > r) && (1.5 * (h1->vrms + h2->vrms)) > v && (r < 1.5 * C.force_res)) {
        *force = 1; return 1;
    }
    return 0;
}
/* _find_biggest_parent without temporal information, src/groupies.c:362-380 */
static int64_t biggest(struct hinfo *hi, int64_t h0, int growing_only) {
    int64_t mi = h0;
    if (growing_only) mi = gh[0];
    for (int64_t i = h0; i < hi->n; i++) {
        if (growing_only && !(hi->h[i].flags & GROWING)) continue;
        if (hi->h[i].vmax > hi->h[mi].vmax) mi = i;
        if (hi->h[i].vmax == hi->h[mi].vmax && hi->h[i].num_p > hi->h[mi].num_p) mi = i;
    }
    return mi;
}
/* _fix_parents without temporal information, src/groupies.c:425-485 */
static void fix_parents(struct hinfo *hi, int64_t h0) {
    for (int64_t i = h0; i < hi->n; i++) {
        hi->e[i].next_cochild = hi->e[i].prev_cochild = hi->e[i].child = -1;
        if (hi->e[i].sub_of == i) hi->e[i].sub_of = -1;
    }
    for (int64_t i = h0; i < hi->n; i++) {
        hi->e[i].max_metric = 1e10;
        int64_t so = hi->e[i].sub_of;
        if (so < 0) continue;
        hi->e[i].max_metric = hdist_raw(hi->h + i, hi->h + so);
        int64_t nx = hi->e[so].child;
        hi->e[i].next_cochild = nx;
        hi->e[i].prev_cochild = -1;
        hi->e[so].child = i;
        if (nx > -1) hi->e[nx].prev_cochild = i;
    }
}
/* reassign_halo_particles, src/groupies.c:316-331 */
static void reassign(struct hinfo *hi, int64_t a, int64_t b) {
    partition_sort(a, b, cp, phalo);
    int64_t last = phalo[a], j;
    hi->h[last].p_start = a;
    for (j = a + 1; j < b; j++) {
        if (phalo[j] == last) continue;
        hi->h[last].num_p = j - hi->h[last].p_start;
        last = phalo[j];
        hi->h[last].p_start = j;
    }
    hi->h[last].num_p = j - hi->h[last].p_start;
}
static void gh_push(int64_t h) {
    if (ngh == capgh) { capgh = capgh * 2 + 1000; gh = realloc(gh, sizeof(int64_t) * capgh); }
    gh[ngh++] = h;
}
static int cmp_core(const void *a, const void *b) {
    const struct particle *c = a, *d = b;
    if (c->pos[0] < d->pos[0]) return -1;
    if (c->pos[0] > d->pos[0]) return 1;
    return 0;
}
/* convert_and_sort_core_particles(h, hp, 0, NULL), src/fun_times.c:204-227 */
static void sort_core(struct halo *h, struct particle *hp) {
    for (int64_t i = 0; i < h->num_p; i++) {
        float dx = 0, ds;
        for (int j = 0; j < 3; j++) { ds = h->pos[j] - hp[i].pos[j]; dx += ds * ds; }
        hp[i].pos[0] = dx;
    }
    qsort(hp, h->num_p, sizeof(struct particle), cmp_core);
    for (int64_t i = 0; i < h->num_p; i++) hp[i].pos[0] = P[hp[i].id].pos[0];
}


/* _find_subs, src/groupies.c:520-667 (temporal and level-output branches
 * are off).  `fi` indexes subf[] (or -1 for the level-0 group `f0`). */
static void find_subs_rec(struct fofrec *f0, int64_t fi, int64_t level, struct hinfo *hi) {
    struct fofrec f = (fi < 0) ? *f0 : subf[fi];
    int64_t p0 = f.particles - cp, fnp = f.num_p, i, j, mi;
    int force;
    int64_t fs = nsubf;
    cur_level = level;
    find_subgroups(&f, (float)C.fof_fraction, NULL);
    int64_t fe = nsubf;
    int64_t h0 = hi->n;
    for (i = fs; i < fe; i++)
        if (subf[i].num_p > C.min_halo_particles && subf[i].num_p < fnp)
            find_subs_rec(NULL, i, level + 1, hi);
    for (j = 0; j < f.num_p; j++) phalo[p0 + j] = -1;
    for (i = h0; i < hi->n; i++)
        for (j = 0; j < hi->h[i].num_p; j++) phalo[hi->h[i].p_start + j] = i;
    for (j = 0; j < f.num_p; j++) {
        struct particle *c = f.particles + j;
        memcpy(c->pos, P[c->id].pos, sizeof(float) * 6);
    }
    if (h0 == hi->n) add_halo(hi);
    mi = biggest(hi, h0, 0);
    ngh = 0;
    hi->h[mi].flags |= GROWING;
    hi->e[mi].sub_of = -1;
    gh_push(mi);
    for (i = h0; i < hi->n; i++) {
        if (i == mi || !(hi->h[i].flags & GROWING)) continue;
        if (poisson_or_force(hi->h + i, hi->h + mi, &force)) {
            hi->h[i].flags -= (hi->h[i].flags & GROWING);
            hi->e[i].sub_of = mi;
            if (!force) {
                for (j = 0; j < hi->h[i].num_p; j++) phalo[hi->h[i].p_start + j] = mi;
                hi->h[i].num_p = 0;
            }
            continue;
        }
        gh_push(i);
    }
    if (ngh == 1) {
        for (j = 0; j < f.num_p; j++) if (phalo[p0 + j] < 0) phalo[p0 + j] = mi;
    } else {
        build_metric_tree(hi, gh, ngh);
        for (j = 0; j < f.num_p; j++) {
            if (phalo[p0 + j] >= 0) continue;
            const float *pos = cp[p0 + j].pos;
            int64_t h = best_halo(hi, pos, mi);
            phalo[p0 + j] = h;
            while (hi->e[h].sub_of > -1) {
                float mm = hi->e[h].max_metric;
                if (pdist(hi->h + h, pos) > mm) { phalo[p0 + j] = hi->e[h].sub_of; h = hi->e[h].sub_of; }
                else break;
            }
        }
    }
    reassign(hi, p0, p0 + f.num_p);
    for (i = 0; i < ngh; i++) basic_props(hi->h + gh[i]);
    mi = biggest(hi, h0, 1);
    build_metric_tree(hi, gh, ngh);
    for (i = 0; i < ngh; i++) hi->e[gh[i]].sub_of = best_parent(hi, gh[i], mi);
    fix_parents(hi, h0);
    calc_nchild(hi, h0);
    for (i = 0; i < ngh; i++) basic_props(hi->h + gh[i]);
    nsubf = fs;
    if (!level) {
        ngh = 0;
        for (i = h0; i < hi->n; i++) gh_push(i);
        for (i = 0; i < ngh; i++) {
            basic_props(hi->h + gh[i]);
            sort_core(hi->h + gh[i], cp + hi->h[gh[i]].p_start);
        }
        build_metric_tree(hi, gh, ngh);
        mi = biggest(hi, h0, 0);
        for (i = 0; i < ngh; i++) hi->e[gh[i]].sub_of = best_parent(hi, gh[i], mi);
        fix_parents(hi, h0);
        calc_nchild(hi, h0);
    }
}

/* ------------------------------------------------------ potential (BH) --
 * src/potential.c:22-192 */
static double d2d(const float *a, const float *b) {
    double dx, r2 = 0;
    for (int k = 0; k < 3; k++) { dx = a[k] - b[k]; r2 += dx * dx; }
    return r2;
}
static double inv_dist(const float *a, const float *b) {
    double r = sqrt(d2d(a, b));
    if (r < C.force_res) r = C.force_res;
    return 1.0 / r;
}
static struct ktree btree;
static inline struct potential *bpt(int64_t i) { return (struct potential *)(btree.base) + i; }
static void direct_pot(struct potential *q, int64_t n) {
    for (int64_t i = 0; i < n; i++)
        for (int64_t j = i + 1; j < n; j++) {
            double d = C.particle_mass * inv_dist(q[i].pos, q[j].pos);
            q[i].pe += d; q[j].pe += d;
        }
}
static void indirect_pot(struct potential *q, int64_t n, struct potential *q2, int64_t n2) {
    for (int64_t i = 0; i < n; i++)
        for (int64_t j = 0; j < n2; j++) q[i].pe += C.particle_mass * inv_dist(q[i].pos, q2[j].pos);
}
static void comp_dmin(struct knode *nd) {
    double sx = 0, bm = 0, dx;
    for (int64_t i = 0; i < nd->n; i++) {
        dx = d2d(nd->mc, bpt(nd->start + i)->pos);
        if (bm < dx) bm = dx;
        sx += dx;
    }
    bm = sqrt(bm) / 2.0;
    nd->dmin = bm + sqrt(bm * bm + sx / (nd->n * 1.0));
}
static void mass_centers(int64_t ni) {
    struct knode *nd = btree.nd + ni;
    if (nd->div < 0) {
        double pos[3] = {0};
        nd->m = C.particle_mass * nd->n;
        for (int64_t i = 0; i < nd->n; i++) for (int j = 0; j < 3; j++) pos[j] += bpt(nd->start + i)->pos[j];
        for (int j = 0; j < 3; j++) nd->mc[j] = pos[j] ? pos[j] / (double)nd->n : 0;
        comp_dmin(nd);
        return;
    }
    mass_centers(nd->left);
    mass_centers(nd->right);
    nd = btree.nd + ni;
    struct knode *L = btree.nd + nd->left, *R = btree.nd + nd->right;
    nd->m = L->m + R->m;
    for (int j = 0; j < 3; j++) nd->mc[j] = nd->m ? ((R->mc[j] * R->m + L->mc[j] * L->m) / nd->m) : 0;
    comp_dmin(nd);
}
static void monopole(int64_t ni, int64_t n2i) {
    struct knode *n = btree.nd + ni, *n2 = btree.nd + n2i;
    int i;
    if (ni == n2i) {
        if (n->n > 2 * 10) return;
        direct_pot(bpt(n->start), n->n);
        return;
    }
    for (i = 0; i < 3; i++) if (n->min[i] < n2->min[i] || n->max[i] > n2->max[i]) break;
    float r2 = d2d(n->mc, n2->mc);
    int acceptable = (r2 > n2->dmin * n2->dmin);
    if (i == 3 || !acceptable) {
        if (n2->div < 0) indirect_pot(bpt(n->start), n->n, bpt(n2->start), n2->n);
        else { monopole(ni, n2->left); monopole(ni, n2->right); }
    } else {
        for (int64_t k = 0; k < n->n; k++) {
            float r = sqrt(d2d(bpt(n->start + k)->pos, n2->mc));
            bpt(n->start + k)->pe += n2->m / r;
        }
    }
}
/* compute_potential, src/potential.c:170-192 */
void oracle_compute_potential(struct potential *q, int64_t n) {
    for (int64_t i = 0; i < n; i++) q[i].pe = 0;
    kfree(&btree);
    kbuild(&btree, q, sizeof(struct potential), 0, 3, 10, n);
    mass_centers(0);
    for (int64_t i = 0; i < btree.nn; i++)
        if (btree.nd[i].div < 0) monopole(i, 0);
}
/* src/potential.c:194-211 */
void oracle_kinetic_energy(struct potential *q, int64_t n, const float *vc, const float *pc, float scale) {
    double dv, conv = 0.5 * scale / GC, z1 = 1.0 / scale;
    double hub = 100.0 * hubble_scaling(z1 - 1.0);
    for (int64_t i = 0; i < n; i++) {
        if (q[i].ke < 0) continue;
        q[i].ke = dv = 0;
        for (int j = 0; j < 3; j++) {
            dv = q[i].pos[j + 3] - vc[j] + hub * scale * (q[i].pos[j] - pc[j]);
            q[i].ke += dv * dv;
        }
        q[i].ke *= conv;
    }
}

/* --------------------------------------------------- halo properties ---- */
/* _reset_potentials / calc_particle_radii, src/groupies.c:212-270 */
static void reset_pot(struct halo *base, struct halo *h, const float *cen, int64_t ps, int pot_only) {
    memset(po + ps, 0, sizeof(struct potential) * h->num_p);
    for (int64_t j = 0; j < h->num_p; j++) {
        float r2 = 0, dx;
        for (int k = 0; k < 3; k++) { dx = cp[h->p_start + j].pos[k] - cen[k]; r2 += dx * dx; }
        po[ps + j].r2 = r2;
        memcpy(po[ps + j].pos, cp[h->p_start + j].pos, sizeof(float) * 6);
        if (pot_only) po[ps + j].ke = -1;
        if (h == base) po[ps + j].flags = 1;
        if (!pot_only && (h->num_p < base->num_p * 0.03)) po[ps + j].flags = 2;
    }
}
static int64_t particle_radii(struct hinfo *hi, struct halo *base, struct halo *h, const float *cen,
                              int64_t ps, int64_t level, int pot_only) {
    int64_t tot = ps;
    if (level >= caphids) { caphids += 1000; hids = realloc(hids, sizeof(int64_t) * caphids); }
    hids[level] = h - hi->h;
    for (int64_t j = 0; j < level; j++) if (hids[j] == hids[level]) return ps;
    reset_pot(base, h, cen, ps, pot_only);
    tot += h->num_p;
    for (int64_t c = hi->e[h - hi->h].child; c > -1; c = hi->e[c].next_cochild)
        tot = particle_radii(hi, base, hi->h + c, cen, tot, level + 1, pot_only);
    int64_t par = hi->e[h - hi->h].sub_of;
    if (h == base && par > -1 &&
        (hi->h[par].num_child_particles * C.include_host_potential_ratio < h->num_child_particles))
        tot = particle_radii(hi, base, hi->h + par, cen, tot, level + 1, 1);
    return tot;
}
static int cmp_r2(const void *a, const void *b) {
    float c = ((const struct potential *)a)->r2, d = ((const struct potential *)b)->r2;
    if (c > d) return 1;
    if (c < d) return -1;
    return 0;
}
/* calculate_corevel, src/properties.c:165-214 */
static void corevel(struct halo *h, struct potential *q, int64_t tot) {
    double vel[3] = {0}, var[3] = {0}, tv, bv = 0;
    double rt = rvir_dens * (4.0 * M_PI / 3.0);
    int64_t j, cmax, rmax;
    for (j = tot - 1; j >= 0; j--)
        if (j * j > (q[j].r2 * q[j].r2 * q[j].r2) * (rt * rt)) break;
    rmax = j;
    if (rmax < 1) return;
    for (j = tot - 1; j >= 0; j--) if (q[j].r2 * 100.0 < q[rmax].r2) break;
    cmax = j;
    if (cmax < 100) cmax = 100;
    for (int64_t i = 0; i < rmax; i++) {
        for (int k = 0; k < 3; k++) {
            double dl = q[i].pos[k + 3] - vel[k];
            vel[k] += dl / ((double)(i + 1));
            var[k] += dl * (q[i].pos[k + 3] - vel[k]);
        }
        tv = (var[0] + var[1] + var[2]);
        if ((i < 10) || (tv < bv * (i - 3) * i)) {
            if (i > 3) bv = tv / (double)((i - 3) * i);
            else bv = 0;
            if (i < cmax) {
                h->n_core = i;
                h->min_vel_err = bv;
                for (int k = 0; k < 3; k++) h->corevel[k] = vel[k];
            }
            for (int k = 0; k < 3; k++) h->bulkvel[k] = vel[k];
            h->min_bulkvel_err = bv;
        }
    }
    for (int k = 0; k < 3; k++) h->pos[k + 3] = h->corevel[k];
}
/* calc_shape, src/properties.c:216-326 */
static void shape(struct halo *h, int64_t tot, int bound) {
    int64_t it = C.shape_iterations, an = 0, a, b, c;
    float ba, ca, minr = C.force_res * C.force_res;
    double mt[3][3], orth[3][3], eig[3] = {0}, r = 0, dr, dr2, w = 0;
    h->b_to_a = h->c_to_a = 0;
    memset(h->A, 0, sizeof(float) * 3);
    if (!(h->r > 0)) return;
    minr *= 1e6 / (h->r * h->r);
    for (int64_t j = 0; j < tot; j++) { if (bound && (po[j].pe < po[j].ke)) continue; an++; }
    if (an < 3 || !(h->r > 0)) return;
    if (an < it) it = an;
    for (int i = 0; i < 3; i++) {
        memset(orth[i], 0, sizeof(double) * 3);
        orth[i][i] = 1;
        eig[i] = (h->r * h->r) * 1e-6;
    }
    for (int64_t i = 0; i < it; i++) {
        memset(mt, 0, sizeof(mt));
        w = 0;
        for (int64_t j = 0; j < tot; j++) {
            if (bound && (po[j].pe < po[j].ke)) continue;
            r = 0;
            for (int k = 0; k < 3; k++) {
                dr = 0;
                for (int l = 0; l < 3; l++) dr += orth[k][l] * (po[j].pos[l] - h->pos[l]);
                r += dr * dr / eig[k];
            }
            if (r < minr) r = minr;
            if (!(r > 0 && r <= 1)) continue;
            double tw = (C.weighted_shapes) ? 1.0 / r : 1.0;
            w += tw;
            for (int k = 0; k < 3; k++) {
                dr = po[j].pos[k] - h->pos[k];
                mt[k][k] += dr * dr * tw;
                for (int l = 0; l < k; l++) {
                    dr2 = po[j].pos[l] - h->pos[l];
                    mt[k][l] += dr2 * dr * tw;
                    mt[l][k] = mt[k][l];
                }
            }
        }
        if (!w) return;
        for (int k = 0; k < 3; k++) for (int l = 0; l < 3; l++) mt[k][l] /= (double)w;
        double mt2[3][3];
        memcpy(mt2, mt, sizeof(mt));
        jacobi(mt, eig, orth);
        a = 0; b = 1; c = 2;
        if (eig[1] > eig[0]) { b = 0; a = 1; }
        if (eig[2] > eig[b]) { c = b; b = 2; }
        if (eig[b] > eig[a]) { int64_t t = a; a = b; b = t; }
        if (!eig[a] || !eig[b] || !eig[c]) return;
        ba = sqrt(eig[b] / eig[a]);
        ca = sqrt(eig[c] / eig[a]);
        if ((fabs(ba - h->b_to_a) < 0.01 * h->b_to_a) && (fabs(ca - h->c_to_a) < 0.01 * h->c_to_a)) return;
        h->b_to_a = (ba > 0) ? ba : 0;
        h->c_to_a = (ca > 0) ? ca : 0;
        r = sqrt(eig[a]);
        for (int k = 0; k < 3; k++) {
            h->A[k] = 1e3 * r * orth[a][k];
            eig[k] *= (h->r * h->r * 1e-6) / (r * r);
        }
        h->inertia_tensor[0] = mt2[0][0]; h->inertia_tensor[1] = mt2[1][1];
        h->inertia_tensor[2] = mt2[2][2]; h->inertia_tensor[3] = mt2[0][1];
        h->inertia_tensor[4] = mt2[1][2]; h->inertia_tensor[5] = mt2[2][0];
    }
}
/* src/properties.c:328-349 */
static float total_energy(int64_t tot, float *ratio) {
    double phi = 0, tphi = 0, ke = 0, r;
    for (int64_t i = tot - 1; i >= 0; i--) {
        if (po[i].pe > po[i].ke) {
            ke += po[i].ke;
            r = sqrt(po[i].r2);
            if (r < C.force_res) r = C.force_res;
            tphi += C.particle_mass * i / r + phi;
            phi += C.particle_mass / r;
        }
    }
    tphi /= 2.0;
    *ratio = 0;
    if (tphi) *ratio = (ke / tphi);
    float sn = C.scale_now;
    return ((ke - tphi) * C.particle_mass * GC / sn);
}
/* src/properties.c:351-382 */
static void pseudo_masses(struct halo *h, int64_t tot, int bound) {
    int64_t np_ = 0, npd = 0;
    double r, r32, mx = 0, rpd = h->rs * 4.0;
    if (rpd < h->r / 5.0) rpd = h->r / 5.0;
    rpd *= 1e-3;
    for (int64_t j = 0; j < tot; j++) {
        if (bound && (po[j].pe < po[j].ke)) continue;
        np_++;
        r = sqrt(po[j].r2);
        r32 = sqrt(r); r32 = r32 * r32 * r32;
        if ((double)(np_ * np_) / r32 > mx) mx = (double)(np_ * np_) / r32;
        if (r < rpd) npd = np_;
    }
    h->m_pe_d = npd * C.particle_mass;
    h->m_pe_b = C.particle_mass * pow(mx, 2.0 / 3.0) / cbrt(4.0 * M_PI * rvir_dens_z0 / 3.0);
}
/* ---- NFW fit, src/nfw.c:14-173 */
static double c_to_f(double c) { double cp1 = 1.0 + c; return (c * cp1 / (log1p(c) * cp1 - c)); }
static double f_to_c(double f) {
    double c = f, tc = c_to_f(c), nc;
    while (fabs((f - tc) / f) > 1e-7) {
        double tc2 = c_to_f(c + 0.1), slope = (tc2 - tc) / 0.1;
        nc = c + (f - tc) / slope;
        if (nc < 0) c /= 2; else c = nc;
        tc = c_to_f(c);
    }
    return c;
}
static float klypin_rs(float mvir, float rvir, float vmax, float rvmax, float scale) {
    float f, c, vm2;
    if (!mvir || !rvir || !vmax) return (rvmax / RMAX_TO_RS);
    vm2 = vmax / VMAX_CONST;
    vm2 = vm2 * vm2 * scale;
    f = (rvir / 1.0e3) * vm2 / (mvir * RS_CONSTANT);
    if (f < 4.625) return (rvmax / RMAX_TO_RS);
    c = f_to_c(f);
    if (c <= 0) return (rvmax / RMAX_TO_RS);
    return (rvir / c);
}
static inline float nfw_menc(float r, float rs) { return (log((rs + r) / rs) - r / (rs + r)); }
static float chi2_scale(float rs, float *br, float *w, int64_t nb) {
    float bm = nfw_menc(br[nb], rs) / ((double)nb), last = 0, chi2 = 0, dx;
    for (int64_t i = 0; i < nb; i++) {
        float menc = nfw_menc(br[i + 1], rs);
        dx = w[i] * ((menc - last) - bm) / bm;
        chi2 += dx * dx;
        last = menc;
    }
    return chi2;
}
static float fit_bins(float rs, float *br, float *w, int64_t nb, float *chi2o) {
    if (!(rs > br[0]) || !(rs < br[nb])) rs = br[(nb + 1) / 2];
    float irs = rs, chi2 = chi2_scale(rs, br, w, nb), drs = rs / 10.0, lc = 1e30;
    int64_t it = 0;
    if (!(rs > 0)) return irs;
    while (fabs(chi2 - lc) > 0.005 * chi2 && it < 15) {
        lc = chi2;
        if (rs + drs > br[nb]) drs = 0.1 * (br[nb] - rs);
        if (rs - drs < br[0]) drs = 0.1 * (rs - br[0]);
        float cr = chi2_scale(rs + drs, br, w, nb), cl = chi2_scale(rs - drs, br, w, nb);
        float dx = 0.5 * (cr - cl) / drs;
        float dx2 = (cr + cl - 2.0 * chi2) / (drs * drs);
        float mv = 0;
        if (dx2 != 0) mv = -dx / dx2;
        if (!mv) return rs;
        if (rs + mv > 4 * rs) mv = 3.0 * rs;
        if (rs + mv < 0.25 * rs) mv = -0.75 * rs;
        float nrs = rs + mv;
        if (nrs > br[nb]) nrs = rs + 0.8 * (br[nb] - rs);
        else if (nrs < br[0]) nrs = rs + 0.8 * (br[0] - rs);
        float nc = chi2_scale(nrs, br, w, nb);
        if (cr < nc) { nc = cr; nrs = rs + drs; }
        if (cl < nc) { nc = cl; nrs = rs - drs; }
        if (lc < nc) { drs *= 0.5; continue; }
        drs = fabs(rs - nrs) / 10.0;
        rs = nrs; chi2 = nc; it++;
    }
    *chi2o = chi2;
    return rs;
}
static void scale_radius(struct halo *h, float mvir, float rvir, float vmax, float rvmax, float scale,
                         int64_t tot, int bound) {
    float br[51] = {0}, w[50] = {0};
    int64_t nb = 0, an = 0, pp = 0, i, j;
    float rs = h->klypin_rs = klypin_rs(mvir, rvir, vmax, rvmax, scale);
    for (i = 0; i < tot - 1; i++) { if (bound && (po[i].pe < po[i].ke)) continue; an++; }
    if (an < 100) { h->rs = rs; return; }
    pp = ceil(((double)an / (double)50));
    if (pp < 15) pp = (an) / ((int64_t)(an / 15));
    br[0] = 0;
    for (i = 0, j = 0; i < tot - 1; i++) {
        if (bound && (po[i].pe < po[i].ke)) continue;
        if (++j == pp) {
            nb++;
            br[nb] = 1e3 * 0.5 * (sqrt(po[i].r2) + sqrt(po[i + 1].r2));
            w[nb - 1] = 1;
            j = 0;
        }
    }
    for (i = 0; i < nb; i++) if (br[i] * 1e-3 < 3 * C.force_res) w[i] = 0.1;
    float chi2 = 0.0;
    h->rs = fit_bins(rs, br, w, nb, &chi2);
    h->chi2 = chi2;
}
static void add_L(double L[3], const float c[6], const float p[6]) {
    L[0] += (p[1] - c[1]) * (p[2 + 3] - c[2 + 3]);
    L[0] -= (p[2] - c[2]) * (p[1 + 3] - c[1 + 3]);
    L[1] += (p[2] - c[2]) * (p[0 + 3] - c[0 + 3]);
    L[1] -= (p[0] - c[0]) * (p[2 + 3] - c[2 + 3]);
    L[2] += (p[0] - c[0]) * (p[1 + 3] - c[1 + 3]);
    L[2] -= (p[1] - c[1]) * (p[0 + 3] - c[0 + 3]);
}
/* _calc_additional_halo_props, src/properties.c:384-510 */
static void more_props(struct halo *h, int64_t tot, int bound) {
    int64_t j, pmd = 0, np_ = 0, npa[4] = {0}, npv = 0, dtot = 0, avg = 0, nhalf = 0;
    float scale = C.scale_now;
    double dth = thresh_dens[0] * (4.0 * M_PI / 3.0);
    double d1 = thresh_dens[1] * (4.0 * M_PI / 3.0), d2 = thresh_dens[2] * (4.0 * M_PI / 3.0);
    double d3 = thresh_dens[3] * (4.0 * M_PI / 3.0), d4 = thresh_dens[4] * (4.0 * M_PI / 3.0);
    double rth = rvir_dens * (4.0 * M_PI / 3.0), vconv = C.particle_mass / scale;
    double r, cv, vmax = 0, rvmax = 0, L[3] = {0}, Jh, m = 0, ds;
    double vrms[3] = {0}, xa[3] = {0}, va[3] = {0}, md, cd, rvir, mvir;
    for (j = 0; j < tot; j++) {
        if (bound && (po[j].pe < po[j].ke)) continue;
        np_++;
        r = sqrt(po[j].r2);
        if (r < C.force_res) r = C.force_res;
        cd = ((double)np_ / (r * r * r));
        if (cd > dth) { pmd = np_; dtot = j; }
        if (cd > d1) npa[0] = np_;
        if (cd > d2) npa[1] = np_;
        if (cd > d3) npa[2] = np_;
        if (cd > d4) npa[3] = np_;
        if (cd > rth) {
            cv = (double)np_ / r;
            npv = np_;
            if (pmd && cv > vmax) { vmax = cv; rvmax = r; }
        }
    }
    for (j = 0; j < dtot; j++) {
        if (bound && (po[j].pe < po[j].ke)) continue;
        add_L(L, h->pos, po[j].pos);
        avg++;
        if (avg * 2 >= pmd && !nhalf) nhalf = j;
        for (int k = 0; k < 3; k++) {
            xa[k] += (po[j].pos[k] - xa[k]) / ((double)avg);
            md = po[j].pos[k + 3] - va[k];
            va[k] += md / (double)avg;
            vrms[k] += md * (po[j].pos[k + 3] - va[k]);
        }
    }
    m = pmd * C.particle_mass;
    if (!bound) h->m = m; else h->mgrav = m;
    for (int k = 0; k < 3; k++) vrms[k] = (avg > 0) ? (vrms[k] / avg) : 0;
    if ((!bound) == (!C.bound_props)) {
        h->Xoff = h->Voff = 0;
        for (int k = 0; k < 3; k++) {
            ds = xa[k] - h->pos[k]; h->Xoff += ds * ds;
            ds = va[k] - h->pos[k + 3]; h->Voff += ds * ds;
        }
        for (int k = 0; k < 4; k++) h->alt_m[k] = npa[k] * C.particle_mass;
        h->Xoff = sqrt(h->Xoff) * 1e3;
        h->Voff = sqrt(h->Voff);
        h->vrms = sqrt(vrms[0] + vrms[1] + vrms[2]);
        h->vmax = VMAX_CONST * sqrt(vmax * vconv);
        h->rvmax = rvmax * 1e3;
        h->halfmass_radius = sqrt(po[nhalf].r2) * 1e3;
        h->r = cbrt((3.0 / (4.0 * M_PI)) * npa[2] / thresh_dens[3]) * 1e3;
        shape(h, npa[2], bound);
        h->b_to_a2 = h->b_to_a; h->c_to_a2 = h->c_to_a;
        memcpy(h->A2, h->A, sizeof(float) * 3);
        memcpy(h->inertia_tensor2, h->inertia_tensor, sizeof(float) * 6);
        h->r = cbrt((3.0 / (4.0 * M_PI)) * pmd / thresh_dens[0]) * 1e3;
        shape(h, dtot, bound);
        rvir = cbrt((3.0 / (4.0 * M_PI)) * npv / rvir_dens) * 1e3;
        mvir = npv * C.particle_mass;
        scale_radius(h, m, h->r, h->vmax, h->rvmax, scale, dtot, bound);
        for (j = 0; j < 3; j++) h->J[j] = C.particle_mass * scale * L[j];
        h->energy = total_energy(dtot, &(h->kin_to_pot));
        Jh = C.particle_mass * scale * sqrt(L[0] * L[0] + L[1] * L[1] + L[2] * L[2]);
        h->spin = (m > 0) ? (Jh * sqrt(fabs(h->energy)) / (GC * pow(m, 2.5))) : 0;
        h->bullock_spin = (m > 0) ? (Jh / (mvir * sqrt(2.0 * GC * mvir * rvir * scale / 1e3))) : 0;
        pseudo_masses(h, tot, bound);
    }
}
/* calc_additional_halo_props, src/properties.c:513-556 (BOUND_OUT_TO_HALO_EDGE = 0) */
static void add_props(struct hinfo *hi, int64_t hidx) {
    struct halo *h = hi->h + hidx;
    if (h->num_p < 1) return;
    int64_t tot = particle_radii(hi, h, h, h->pos, 0, 0, 0);
    if (tot > 1) oracle_compute_potential(po, tot);
    for (int64_t j = 0; j < tot; j++)
        if (po[j].ke < 0) { tot--; po[j] = po[tot]; j--; }
    qsort(po, tot, sizeof(struct potential), cmp_r2);
    corevel(h, po, tot);
    if (hi->e[hidx].sub_of > -1) oracle_kinetic_energy(po, tot, h->corevel, h->pos, C.scale_now);
    else oracle_kinetic_energy(po, tot, h->bulkvel, h->pos, C.scale_now);
    more_props(h, tot, 0);
    more_props(h, tot, 1);
}

/* find_subs, src/groupies.c:669-708, for one group of `pa` (the caller's
 * particle array, which plays the role of the global p).  Appends halos to
 * *hi with p_start relative to pa. */
static void find_subs_one(struct particle *pa, int64_t off, int64_t n, struct hinfo *hi) {
    int64_t h0 = hi->n;
    if (!n) return;
    P = pa;
    cp = realloc(cp, sizeof(struct particle) * n);
    phalo = realloc(phalo, sizeof(int64_t) * n);
    prad = realloc(prad, sizeof(float) * (n < SAMPLE_MAX ? SAMPLE_MAX : n));
    po = realloc(po, sizeof(struct potential) * n);
    memcpy(cp, pa + off, sizeof(struct particle) * n);
    for (int64_t i = 0; i < n; i++) cp[i].id = off + i;
    ncopies = n;
    struct fofrec cf = {n, cp};
    nsubf = 0;
    find_subs_rec(&cf, -1, 0, hi);
    nsubf = 0;
    for (int64_t i = 0; i < n; i++) cp[i] = pa[cp[i].id];
    calc_nchild(hi, h0);
    for (int64_t i = h0; i < hi->n; i++) basic_props(hi->h + i);
    for (int64_t i = h0; i < hi->n; i++) add_props(hi, i);
    memcpy(pa + off, cp, sizeof(struct particle) * n);
    for (int64_t i = h0; i < hi->n; i++) hi->h[i].p_start += off;
}

/* Runs find_subs over every group (offsets/sizes into pa), in order, and
 * returns the halos (malloc'd; free with oracle_free) with links already
 * global, as copy_halos (src/mpi_main.cpp:1335-1361) leaves them. */
int64_t oracle_find_subs(struct particle *pa, const int64_t *off, const int64_t *sz, int64_t nf,
                         struct halo **ho, struct extra **eo) {
    struct hinfo hi = {0};
    rec_cnt = 0;
    for (int64_t i = 0; i < nf; i++) find_subs_one(pa, off[i], sz[i], &hi);
    *ho = hi.h; *eo = hi.e;
    return hi.n;
}

/* Test hook: the in-place permutation of fast3tree_init (src/fast3tree.c:225-240)
 * over particle records, for dim 3 or 6 and the given leaf size. */
void oracle_tree_order(struct particle *pa, int64_t n, int dim, int leaf) {
    struct ktree t = {0};
    kbuild(&t, pa, sizeof(struct particle), 8, dim, leaf, n);
    kfree(&t);
}

/* ------------------------------------------------- catalogue output ----
 * _within_bounds / _should_print (src/io/meta_io.c:266-286), output_ascii
 * with print_ascii_header_info (:288-371) and output_binary with
 * fill_binary_header (src/io/io_internal.c:16-41,104-186; header
 * src/io/io_internal.h:6-27), with the file name given by the caller.  The
 * reference's meta_io.c does not compile here (its reader headers need the
 * tirpc library's rpc/types.h), so the ascii writer is pinned by this
 * restatement alone; output_binary itself is compiled from io_internal.c into
 * oracle/_ref and pins the binary writer where the reference is present. */
#include <inttypes.h>
#define ORC_ALWAYS_PRINT 16                      /* src/groupies.h:12 */
static const char *orc_mass_def[5] = {"vir", "200b", "200c", "500c", "2500c"};

static int orc_within_bounds(const struct halo *h, const float *bounds) {
    int64_t i;
    if (!bounds) return 1;
    for (i = 0; i < 3; i++)
        if (h->pos[i] < bounds[i] || h->pos[i] > bounds[i + 3]) return 0;
    return 1;
}
int oracle_should_print(const struct halo *h, const float *bounds) {
    if (!orc_within_bounds(h, bounds)) return 0;
    if (h->flags & ORC_ALWAYS_PRINT) return 1;
    if ((h->num_p < C.min_halo_output_size) || (h->m * C.unbound_threshold >= h->mgrav) ||
        ((h->mgrav < 1.5 * C.particle_mass) && C.unbound_threshold > 0))
        return 0;
    return 1;
}

static void orc_header_info(FILE *output, const float *bounds, int64_t np, int64_t strict_so) {
    fprintf(output, "#a = %f\n", C.scale_now);
    if (bounds)
        fprintf(output, "#Bounds: (%f, %f, %f) - (%f, %f, %f)\n", bounds[0], bounds[1],
                bounds[2], bounds[3], bounds[4], bounds[5]);
    fprintf(output, "#Om = %f; Ol = %f; h = %f\n", C.om, C.ol, C.h0);
    fprintf(output, "#FOF linking length: %f\n", C.fof_linking_length);
    fprintf(output, "#Unbound Threshold: %f; FOF Refinement Threshold: %f\n",
            C.unbound_threshold, C.fof_fraction);
    fprintf(output, "#Particle mass: %.5e Msun/h\n", C.particle_mass);
    fprintf(output, "#Box size: %f Mpc/h\n", C.box_size);
    if (np) fprintf(output, "#Total particles processed: %" PRId64 "\n", np);
    fprintf(output, "#Force resolution assumed: %g Mpc/h\n", C.force_res);
    if (strict_so && !np) fprintf(output, "#Using Strict Spherical Overdensity Masses\n");
    fprintf(output,
            "#Units: Masses in Msun / h\n"
            "#Units: Positions in Mpc / h (comoving)\n"
            "#Units: Velocities in km / s (physical, peculiar)\n"
            "#Units: Halo Distances, Lengths, and Radii in kpc / h (comoving)\n"
            "#Units: Angular Momenta in (Msun/h) * (Mpc/h) * km/s (physical)\n"
            "#Units: Spins are dimensionless\n");
    if (np)
        fprintf(output,
                "#Units: Total energy in (Msun/h)*(km/s)^2"
                " (physical)\n"
                "#Note: idx, i_so, and i_ph are internal debugging quantities\n");
    fprintf(output, "#Np is an internal debugging quantity.\n");
    fprintf(output, "#MPI-Rockstar Version: %s\n", "1.0.0RC");   /* src/version.h:4 */
}

int oracle_write_ascii(const char *path, const struct halo *halos, const struct extra *ex,
                       int64_t num_halos, int64_t id_offset, const float *bounds, int64_t np,
                       int64_t strict_so) {
    int64_t i, id = 0;
    const struct halo *th;
    const char **M = orc_mass_def;
    FILE *output = fopen(path, "w");
    if (!output) return -1;
    fprintf(output,
            "#id num_p m%s mbound_%s r%s vmax rvmax vrms x y z vx vy vz Jx Jy "
            "Jz E Spin PosUncertainty VelUncertainty bulk_vx bulk_vy bulk_vz "
            "BulkVelUnc n_core m%s m%s m%s m%s Xoff Voff spin_bullock b_to_a "
            "c_to_a A[x] A[y] A[z] b_to_a(%s) c_to_a(%s) A[x](%s) A[y](%s) "
            "A[z](%s) Rs Rs_Klypin T/|U| M_pe_Behroozi M_pe_Diemer "
            "Halfmass_Radius idx i_so i_ph num_cp mmetric\n",
            M[0], M[0], M[0], M[1], M[2], M[3], M[4], M[3], M[3], M[3], M[3], M[3]);
    orc_header_info(output, bounds, np, strict_so);
    for (i = 0; i < num_halos; i++) {
        if (!oracle_should_print(halos + i, bounds)) continue;
        th = halos + i;
        fprintf(output,
                "%" PRId64 " %" PRId64 " %.3e %.3e"
                " %f %f %f %f %f %f %f %f %f %f %g %g %g %g %g %f %f %f %f %f "
                "%f %" PRId64 " %e %e %e %e %f %f %f %f %f %f %f %f %f %f %f "
                "%f %f %f %f %f %e %e %f %" PRId64 " %" PRId64 " %" PRId64
                " %" PRId64 " %f\n",
                id + id_offset, th->num_p, th->m, th->mgrav, th->r, th->vmax, th->rvmax,
                th->vrms, th->pos[0], th->pos[1], th->pos[2], th->pos[3], th->pos[4],
                th->pos[5], th->J[0], th->J[1], th->J[2], th->energy, th->spin,
                sqrt(th->min_pos_err), sqrt(th->min_vel_err), th->bulkvel[0], th->bulkvel[1],
                th->bulkvel[2], sqrt(th->min_bulkvel_err), th->n_core, th->alt_m[0],
                th->alt_m[1], th->alt_m[2], th->alt_m[3], th->Xoff, th->Voff,
                th->bullock_spin, th->b_to_a, th->c_to_a, th->A[0], th->A[1], th->A[2],
                th->b_to_a2, th->c_to_a2, th->A2[0], th->A2[1], th->A2[2], th->rs,
                th->klypin_rs, th->kin_to_pot, th->m_pe_b, th->m_pe_d, th->halfmass_radius, i,
                ex[i].sub_of, ex[i].ph, th->num_child_particles, ex[i].max_metric);
        id++;
    }
    fclose(output);
    return 0;
}

struct orc_bin_header {                           /* src/io/io_internal.h:15-27 */
    uint64_t magic;
    int64_t snap, chunk;
    float scale, Om, Ol, h0;
    float bounds[6];
    int64_t num_halos, num_particles;
    float box_size, particle_mass;
    int64_t particle_type;
    int32_t format_revision;
    char rockstar_version[12];
    int32_t add_flag;
    char unused[256 - 12 - 4 * 12 - 4 * 2 - 8 * 6];
};

int oracle_write_binary(const char *path, const struct halo *halos, int64_t num_halos,
                        const struct particle *p, int64_t id_offset, int64_t snap,
                        int64_t chunk, const float *bounds) {
    float max[3] = {0}, min[3] = {0};
    struct halo tmp;
    int64_t i, j, id = 0;
    struct orc_bin_header bh;
    FILE *output = fopen(path, "wb");
    if (!output) return -1;
    memset(&bh, 0, sizeof bh);
    fwrite(&bh, sizeof bh, 1, output);
    if (num_halos) {
        memcpy(min, halos[0].pos, sizeof(float) * 3);
        memcpy(max, halos[0].pos, sizeof(float) * 3);
    }
    for (i = 0; i < num_halos; i++) {
        if (!oracle_should_print(halos + i, bounds)) continue;
        for (j = 0; j < 3; j++) {
            if (min[j] > halos[i].pos[j]) min[j] = halos[i].pos[j];
            if (max[j] < halos[i].pos[j]) max[j] = halos[i].pos[j];
        }
        tmp = halos[i];
        tmp.id = id + id_offset;
        tmp.p_start = bh.num_particles;
        fwrite(&tmp, sizeof tmp, 1, output);
        bh.num_halos++;
        bh.num_particles += tmp.num_p;
        id++;
    }
    for (i = 0; i < num_halos; i++) {
        if (!oracle_should_print(halos + i, bounds)) continue;
        for (j = 0; j < halos[i].num_p; j++)
            fwrite(&(p[halos[i].p_start + j].id), sizeof(int64_t), 1, output);
    }
    bh.magic = 0xfadedacec0c0d0d0ULL;
    bh.snap = snap;
    bh.chunk = chunk;
    bh.scale = C.scale_now;
    bh.Om = C.om;
    bh.Ol = C.ol;
    bh.h0 = C.h0;
    bh.box_size = C.box_size;
    bh.particle_mass = C.particle_mass;
    snprintf(bh.rockstar_version, 12, "%s", "1.0.0RC");
    bh.format_revision = 2;                       /* HALO_FORMAT_REVISION, src/halo.h:4 */
    bh.add_flag = 1 | 4;                          /* OUTPUT_NFW_CHI2 | OUTPUT_INERTIA_TENSOR */
    bh.particle_type = 1;                         /* PARTICLE_TYPE_IDS */
    if (bounds)
        memcpy(bh.bounds, bounds, sizeof(float) * 6);
    else {
        memcpy(bh.bounds, min, sizeof(float) * 3);
        memcpy(&(bh.bounds[3]), max, sizeof(float) * 3);
    }
    rewind(output);
    fwrite(&bh, sizeof bh, 1, output);
    fclose(output);
    return 0;
}

/* output_full_particles with print_child_particles (src/io/meta_io.c:378-461)
 * to the caller's file name: the halo table (ids assigned to the printable
 * halos from id_offset, -1 for the others, printed only with
 * UNFILTERED_HALO_OUTPUT), then every listed halo's particles followed,
 * recursively, by its children's.  ids_out receives the ids the reference
 * writes back into halos[].id. */
static void orc_child_particles(FILE *output, const struct halo *halos, const struct extra *ex,
                                const struct particle *p, int64_t i, int64_t pid, int64_t eid,
                                int64_t every_n) {
    int64_t j, child;
    const struct particle *p2;
    for (j = 0; j < halos[i].num_p; j++) {
        p2 = p + halos[i].p_start + j;
        if (every_n <= 1 || !(p2->id % every_n))
            fprintf(output,
                    "%f %f %f %f %f %f %" PRId64 " %" PRId64 " %" PRId64 " %" PRId64 "\n",
                    p2->pos[0], p2->pos[1], p2->pos[2], p2->pos[3], p2->pos[4], p2->pos[5],
                    p2->id, i, pid, eid);
    }
    child = ex[i].child;
    while (child > -1) {
        orc_child_particles(output, halos, ex, p, child, pid, eid, every_n);
        child = ex[child].next_cochild;
    }
}

int oracle_write_particles(const char *path, const struct halo *halos, const struct extra *ex,
                           int64_t num_halos, const struct particle *p, int64_t id_offset,
                           const float *bounds, int64_t np, int64_t strict_so, int64_t unfiltered,
                           int64_t every_n, int64_t *ids_out) {
    int64_t i, id = 0;
    const struct halo *th;
    const char **M = orc_mass_def;
    FILE *output = fopen(path, "w");
    if (!output) return -1;
    fprintf(output, "#Halo table:\n");
    fprintf(output,
            "#id internal_id num_p m%s mbound_%s r%s vmax rvmax vrms x y z vx "
            "vy vz Jx Jy Jz energy spin\n",
            M[0], M[0], M[0]);
    fprintf(output, "#Particle table:\n");
    fprintf(output, "#x y z vx vy vz particle_id assigned_internal_haloid "
                    "internal_haloid external_haloid\n");
    if (every_n > 1)
        fprintf(output, "#Notes: Only particles with IDs divisible by %" PRId64 " are printed.\n",
                every_n);
    fprintf(output,
            "#Notes: As not all halos are printed, some halos may not have "
            "external halo ids.  (Hence the need to print internal halo ids).  "
            "Each particle is assigned to a unique halo; however, some "
            "properties (such as halo bound mass) are calculated including all "
            "substructure.  As such, particles belonging to subhalos are "
            "included in outputs; to exclude substructure, verify that the "
            "internal halo id is the same as the assigned internal halo id.\n");
    orc_header_info(output, bounds, np, strict_so);
    fprintf(output, "#Halo table begins here:\n");
    for (i = 0; i < num_halos; i++) {
        th = halos + i;
        if (oracle_should_print(th, bounds)) {
            ids_out[i] = id + id_offset;
            id++;
        } else {
            ids_out[i] = -1;
            if (!unfiltered) continue;
        }
        fprintf(output,
                "#%" PRId64 " %" PRId64 " %" PRId64 " %.3e %.3e"
                " %f %f %f %f %f %f %f %f %f %f %g %g %g %g %g\n",
                ids_out[i], i, th->num_p, th->m, th->mgrav, th->r, th->vmax, th->rvmax, th->vrms,
                th->pos[0], th->pos[1], th->pos[2], th->pos[3], th->pos[4], th->pos[5], th->J[0],
                th->J[1], th->J[2], th->energy, th->spin);
    }
    fprintf(output, "#Particle table begins here:\n");
    for (i = 0; i < num_halos; i++)
        if (unfiltered || ids_out[i] > -1)
            orc_child_particles(output, halos, ex, p, i, i, ids_out[i], every_n);
    fclose(output);
    return 0;
}

/* ------------------------------------------------------- merger trees ----
 * The descendant rule of src/merger.c:45-101 (connect_particle_ids_to_halo_ids
 * + calculate_descendants): every particle id listed by a halo of the later
 * catalogue (halos2 in order, each halo's ids in order) maps to that halo's
 * id, a later listing replacing an earlier one; a halo of the earlier
 * catalogue takes as descendant the id that most of its particles map to,
 * the smallest such id on a tie, or -1 when none maps.  Restated here as a
 * sort-based join over (particle id, listing order). */
struct orc_pid_hid { int64_t pid, ord, hid; };
static int orc_cmp_pid_ord(const void *a, const void *b) {
    const struct orc_pid_hid *x = a, *y = b;
    if (x->pid != y->pid) return x->pid < y->pid ? -1 : 1;
    return (x->ord > y->ord) - (x->ord < y->ord);
}
static int orc_cmp_i64(const void *a, const void *b) {
    int64_t x = *(const int64_t *)a, y = *(const int64_t *)b;
    return (x > y) - (x < y);
}
void oracle_descendants(const struct halo *h1, int64_t nh1, const int64_t *p1,
                        const struct halo *h2, int64_t nh2, const int64_t *p2,
                        int64_t *desc_out) {
    int64_t i, j, n = 0, m = 0, k;
    for (i = 0; i < nh2; i++) n += h2[i].num_p > 0 ? h2[i].num_p : 0;
    struct orc_pid_hid *map = malloc(sizeof *map * (n ? n : 1));
    for (i = 0; i < nh2; i++)
        for (j = h2[i].p_start; j < h2[i].p_start + h2[i].num_p; j++) {
            map[m].pid = p2[j];
            map[m].ord = m;
            map[m].hid = h2[i].id;
            m++;
        }
    qsort(map, m, sizeof *map, orc_cmp_pid_ord);
    /* keep the last listing of each id */
    for (i = 0, k = 0; i < m; i++)
        if (i + 1 == m || map[i + 1].pid != map[i].pid) map[k++] = map[i];
    m = k;
    int64_t cap = 1;
    for (i = 0; i < nh1; i++) if (h1[i].num_p > cap) cap = h1[i].num_p;
    int64_t *hits = malloc(sizeof(int64_t) * cap);
    for (i = 0; i < nh1; i++) {
        desc_out[i] = -1;
        for (j = 0, k = 0; j < h1[i].num_p; j++) {
            int64_t pid = p1[h1[i].p_start + j], lo = 0, hi = m;
            while (lo < hi) {
                int64_t mid = lo + (hi - lo) / 2;
                if (map[mid].pid < pid) lo = mid + 1; else hi = mid;
            }
            if (lo < m && map[lo].pid == pid) hits[k++] = map[lo].hid;
        }
        if (!k) continue;
        qsort(hits, k, sizeof(int64_t), orc_cmp_i64);
        int64_t best = -1, best_n = 0, run = 1;
        for (j = 1; j <= k; j++) {
            if (j < k && hits[j] == hits[j - 1]) { run++; continue; }
            if (run > best_n) { best_n = run; best = hits[j - 1]; }
            run = 1;
        }
        desc_out[i] = best;
    }
    free(hits);
    free(map);
}
