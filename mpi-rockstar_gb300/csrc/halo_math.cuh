// Per-halo device math shared by the find_subs pipeline: phase-space metric,
// Poisson / force-resolution test, 3x3 Jacobi, NFW pieces.  Expressions keep
// the float/double conversions of the reference expressions they follow.
#pragma once
#include "common.cuh"

namespace rsg {

// Loops that the reference runs until convergence carry an iteration limit
// here; one that reaches it sets this flag (one copy per translation unit),
// which the host reads at the end of the call and turns into RSG_ERR_LIMIT.
static __device__ int g_loop_limit_hit;
__device__ __forceinline__ void loop_limit_hit() { atomicExch(&g_loop_limit_hit, 1); }
static inline void loop_limit_reset(cudaStream_t st) {
    const int z = 0;
    RSG_CUDA(cudaMemcpyToSymbolAsync(g_loop_limit_hit, &z, sizeof(int), 0, cudaMemcpyHostToDevice,
                                     st));
}
// After the stream has been synchronised: fails the call if a limit was hit.
static inline void loop_limit_check(cudaStream_t st, const char *where) {
    int h = 0;
    RSG_CUDA(cudaMemcpyFromSymbolAsync(&h, g_loop_limit_hit, sizeof(int), 0,
                                       cudaMemcpyDeviceToHost, st));
    RSG_CUDA(cudaStreamSynchronize(st));
    if (h) {
        set_error(RSG_ERR_LIMIT, "%s: an iterative step (quickselect, Jacobi, parent walk or "
                  "NFW concentration) hit its iteration limit", where);
        throw Failure();
    }
}

#define RSG_GROWING 1
#define RSG_GC 4.30117902e-9          // src/universal_constants.h:4
#define RSG_VMAX_CONST 6.55833746e-5  // src/universal_constants.h:6
#define RSG_RMAX_TO_RS 2.1626
#define RSG_RS_CONSTANT 0.216216595

// Parameters every kernel needs, copied from rsg_config once per call.
struct DevCfg {
    double particle_mass, force_res, scale_now, initial_metric_scaling;
    double include_host_potential_ratio, fof_fraction;
    double thresh_dens[5], rvir_dens, rvir_dens_z0, dyn_time, om, ol, w0, wa;
    // 100 * hubble_scaling(1/SCALE_NOW - 1) with SCALE_NOW rounded to float, as
    // compute_kinetic_energy receives it (src/potential.c:194-199); evaluated on
    // the host with the C library's pow/log/sqrt, as the reference does
    double hub;
    int64_t min_halo_particles, bound_props, shape_iterations, weighted_shapes, exact_ll_calc;
};

// calc_particle_dist, src/subhalo_metric.c:51-65
__device__ __forceinline__ float pdist(const rsg_halo &h, const float *pos) {
    if (h.vrms <= 0 || h.r <= 0) return 1e20f;
    float r2 = 0.f, v2 = 0.f;
#pragma unroll
    for (int i = 0; i < 3; i++) {
        float dx = fsub(h.pos[i], pos[i]);
        r2 = fadd(r2, fmul(dx, dx));
    }
#pragma unroll
    for (int i = 3; i < 6; i++) {
        float dx = fsub(h.bulkvel[i - 3], pos[i]);
        v2 = fadd(v2, fmul(dx, dx));
    }
    float a = __fdiv_rn(r2, fmul(h.r, h.r));
    float b = __fdiv_rn(v2, fmul(h.vrms, h.vrms));
    return sqrt_fd(fadd(a, b));
}
// could_be_poisson_or_force_res, src/groupies.c:333-360
__device__ __forceinline__ int poisson_or_force(const rsg_halo &h1, const rsg_halo &h2,
                                                double force_res, int *force) {
    *force = 0;
    if (!h1.min_pos_err || !h1.min_vel_err) return 1;
    float r = 0.f, v = 0.f, dx;
    for (int k = 0; k < 3; k++) {
        dx = fsub(h1.pos[k], h2.pos[k]);
        r = fadd(r, fmul(dx, dx));
        dx = fsub(h1.pos[k + 3], h2.pos[k + 3]);
        v = fadd(v, fmul(dx, dx));
    }
    float mpe = h1.min_pos_err, mve = h1.min_vel_err;
    dx = (float)((double)fadd(__fdiv_rn(r, mpe), __fdiv_rn(v, mve)) / 2.0);
    if (!(dx > 100)) return 1;
    r = sqrt_fd(r);
    v = sqrt_fd(v);
    if ((fadd(h1.r, h2.r) > r) && (1.5 * (double)fadd(h1.vrms, h2.vrms)) > (double)v &&
        ((double)r < 1.5 * force_res)) {
        *force = 1;
        return 1;
    }
    return 0;
}

// round_to_double(a + sqrt(x)) with the sum taken before rounding, as the
// reference's `fabsl(a) + sqrtl(x)` in a wide long double does: sqrt(x) is
// carried as hi + lo (lo from the exact FMA residual), the sum with a is
// formed by an error-free transformation and rounded once.
__device__ __forceinline__ double abs_plus_sqrt(double a, double x) {
    double hi = sqrt(x);
    if (!(hi > 0) || isinf(hi)) return a + hi;
    double lo = fma(-hi, hi, x) / (2.0 * hi);
    double sum = a + hi;
    double bb = sum - a;
    double err = (a - (sum - bb)) + (hi - bb);
    return sum + (err + lo);
}

// Cyclic 3x3 Jacobi with the 1e-6 change rule, src/jacobi.c:9-138; the
// rotation's t is rounded once from an extended sum as the reference's
// long double expression is, s = sqrt of a double needs no extension.
__device__ inline void jacobi3(double a[3][3], double eig[3], double v[3][3]) {
    int maxc[3], chg[3], n = 3, state = 0;
    double mx, c, s, t, u, w;
    for (int i = 0; i < n; i++) {
        mx = 0;
        maxc[i] = i + 1;
        for (int j = i + 1; j < n; j++)
            if (fabs(a[i][j]) > mx) {
                maxc[i] = j;
                mx = fabs(a[i][j]);
            }
    }
    for (int i = 0; i < n; i++)
        for (int j = 0; j < n; j++) v[i][j] = (i == j) ? 1 : 0;
    for (int i = 0; i < n; i++) {
        eig[i] = a[i][i];
        chg[i] = 1;
        int j;
        for (j = 0; j < n; j++)
            if (j != i && a[i][j]) break;
        if (j == n) {
            state--;
            chg[i] = 0;
        }
    }
    state += n;
    int guard = 0;
    while (state) {
        if (++guard > 10000) {  // the reference's loop ends after a few sweeps
            loop_limit_hit();
            break;
        }
        mx = fabs(a[0][maxc[0]]);
        int mr = 0;
        for (int i = 1; i < n - 1; i++)
            if (fabs(a[i][maxc[i]]) > mx) {
                mx = fabs(a[i][maxc[i]]);
                mr = i;
            }
        int k = mr, l = maxc[k];
        mx = a[k][l];
        if (mx == 0) break;
        w = (eig[l] - eig[k]) * 0.5;
        t = abs_plus_sqrt(fabs(w), mx * mx + w * w);
        s = sqrt(mx * mx + t * t);
        c = t / s;
        s = mx / s;
        t = mx * mx / t;
        if (w < 0) {
            s = -s;
            t = -t;
        }
        double ys[2] = {-t, t};
        int xs[2] = {k, l};
        for (int z = 0; z < 2; z++) {
            int x = xs[z];
            double y = ys[z];
            eig[x] += y;
            if (chg[x] && (fabs(y) < 1e-6 * fabs(eig[x]))) {
                chg[x] = 0;
                state--;
            } else if (!chg[x] && (fabs(y) > 1e-6 * fabs(eig[x]))) {
                chg[x] = 1;
                state++;
            }
        }
        a[k][l] = 0;
#define RSG_ROT(m, p1, q1, p2, q2, upd)                                          \
    {                                                                            \
        t = m[p1][q1];                                                           \
        u = m[p2][q2];                                                           \
        m[p1][q1] = t * c - s * u;                                               \
        m[p2][q2] = s * t + c * u;                                               \
        if (upd) {                                                               \
            if (fabs(m[p1][q1]) > fabs(m[p1][maxc[p1]])) maxc[p1] = q1;          \
            if (p2 < 3 && fabs(m[p2][q2]) > fabs(m[p2][maxc[p2]])) maxc[p2] = q2; \
        }                                                                        \
    }
        for (int i = 0; i < k; i++) RSG_ROT(a, i, k, i, l, 1);
        for (int i = k + 1; i < l; i++) RSG_ROT(a, k, i, i, l, 1);
        for (int i = l + 1; i < n; i++) RSG_ROT(a, k, i, l, i, 1);
        for (int i = 0; i < n; i++) RSG_ROT(v, k, i, l, i, 0);
#undef RSG_ROT
    }
    for (int k = 0; k < n - 1; k++)
        for (int l = k + 1; l < n; l++) a[k][l] = a[l][k];
}

// set_eig, src/jacobi.c:140-154
__device__ inline double min_eig_sqrt(double in[3][3]) {
    double v[3][3], e[3];
    jacobi3(in, e, v);
    double r = e[0];
    if (e[1] < r) r = e[1];
    if (e[2] < r) r = e[2];
    if (r <= 0) r = sqrt(in[0][0] + in[1][1] + in[2][2]);
    else r = sqrt(r);
    return r;
}

}  // namespace rsg
