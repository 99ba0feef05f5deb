// Batched form of the per-halo property scans (calculate_corevel,
// compute_kinetic_energy, _calc_additional_halo_props x2, calc_shape,
// estimate_total_energy, calc_scale_radius, _calc_pseudo_evolution_masses;
// src/properties.c:165-556, src/nfw.c:130-173) as a sequence of segmented
// passes over the radius-sorted potential records of ALL halos at once.
//
// The records of every halo are cut into chunks of RSG_CH records that never
// span two halos; one block processes one chunk per pass, so a halo of 3e5
// records spreads over ~150 blocks instead of one.  Each pass writes one
// partial per chunk; a thread per halo combines its chunks in order (the
// result is deterministic) and takes the halo's decisions (thresholds,
// Jacobi, NFW fit).  Prefix counts ("number of kept particles up to j") are
// chunk-offset block scans.  The reference's running means and variances in
// calculate_corevel become prefix sums, and its running-minimum test picks
// the first minimum of tv / ((i-3) i).  Results equal the sequential ones
// up to FP64 rounding of the sums.
#pragma once
#include <limits.h>
#include <math.h>

#include <cub/block/block_reduce.cuh>
#include <cub/block/block_scan.cuh>

namespace rsg {

#define RSG_CH 2048               // records per chunk
#define RSG_CT 256                // threads per chunk block
#define RSG_CI (RSG_CH / RSG_CT)  // records per thread

struct Chunk {
    int32_t halo, start, n, first;  // start: record index; first: index within the halo
};

// per-halo state carried between passes
struct HS {
    int64_t rmax, cmax;
    double x0[3];
    int64_t pmd, dtot, j0, npa[4], npv;
    double vmax, rvmax, m;
    double L[3], xa[3], va[3];
    int64_t avg, nhalf;
    double orth[3][3], eig[3];
    float minr;
    int32_t it, iter, done, set;
    double kes, ts;
    int64_t an, pp;
    float br[51], w[50];
};

// per-chunk partial results of one pass
struct CP {
    double d[9];
    long long i[8];
};

// ---- small block reductions ----------------------------------------------
struct I8 {
    long long v[8];
};
struct MaxMin8 {  // v[0..6] max, v[7] min
    __device__ I8 operator()(const I8 &a, const I8 &b) const {
        I8 r;
        for (int k = 0; k < 7; k++) r.v[k] = a.v[k] > b.v[k] ? a.v[k] : b.v[k];
        r.v[7] = a.v[7] < b.v[7] ? a.v[7] : b.v[7];
        return r;
    }
};
struct MaxLL {
    __device__ long long operator()(long long a, long long b) const { return a > b ? a : b; }
};
struct D9 {
    double v[9];
};
struct SumD9 {
    __device__ D9 operator()(const D9 &a, const D9 &b) const {
        D9 r;
        for (int k = 0; k < 9; k++) r.v[k] = a.v[k] + b.v[k];
        return r;
    }
};
struct VI {  // value with index; ties go to the smaller index
    double v;
    long long j;
};
struct ArgMax {
    __device__ VI operator()(const VI &a, const VI &b) const {
        return (b.v > a.v || (b.v == a.v && b.j < a.j)) ? b : a;
    }
};
struct ArgMin {
    __device__ VI operator()(const VI &a, const VI &b) const {
        return (b.v < a.v || (b.v == a.v && b.j < a.j)) ? b : a;
    }
};
struct D6 {
    double v[6];
};
struct SumD6 {
    __device__ D6 operator()(const D6 &a, const D6 &b) const {
        D6 r;
        for (int k = 0; k < 6; k++) r.v[k] = a.v[k] + b.v[k];
        return r;
    }
};

// ---- chunk table -----------------------------------------------------------
__global__ void k_sg_nch(const rsg_halo *H, int32_t NH, const int32_t *kept, int32_t *nch) {
    int h = blockIdx.x * blockDim.x + threadIdx.x;
    if (h > NH) return;
    nch[h] = (h < NH && H[h].num_p >= 1) ? (kept[h] + RSG_CH - 1) / RSG_CH : 0;
}
__global__ void k_sg_fill(int32_t NH, const int32_t *toff, const int32_t *kept,
                          const int32_t *c0, const int32_t *nch, Chunk *CH) {
    int h = blockIdx.x * blockDim.x + threadIdx.x;
    if (h >= NH) return;
    for (int c = 0; c < nch[h]; c++) {
        Chunk k;
        k.halo = h;
        k.first = c * RSG_CH;
        k.start = toff[h] + k.first;
        k.n = min(RSG_CH, kept[h] - k.first);
        CH[c0[h] + c] = k;
    }
}

// ---- segmented inclusive counts of a per-record flag -----------------------
__global__ void __launch_bounds__(RSG_CT) k_sg_cnt_chunk(const Chunk *CH, const uint8_t *flag,
                                                         CP *cp) {
    typedef cub::BlockReduce<int, RSG_CT> R;
    __shared__ typename R::TempStorage tmp;
    Chunk c = CH[blockIdx.x];
    int s = 0;
    for (int k = threadIdx.x; k < c.n; k += RSG_CT) s += flag[c.start + k];
    s = R(tmp).Sum(s);
    if (threadIdx.x == 0) cp[blockIdx.x].i[0] = s;
}
// exclusive prefix over each halo's chunks, in chunk order
__global__ void k_sg_cnt_off(int32_t NH, const int32_t *c0, const int32_t *nch, CP *cp) {
    int h = blockIdx.x * blockDim.x + threadIdx.x;
    if (h >= NH) return;
    long long run = 0;
    for (int c = c0[h]; c < c0[h] + nch[h]; c++) {
        long long t = cp[c].i[0];
        cp[c].i[0] = run;
        run += t;
    }
}
__global__ void __launch_bounds__(RSG_CT) k_sg_cnt_scan(const Chunk *CH, const uint8_t *flag,
                                                        const CP *cp, int32_t *cnt) {
    typedef cub::BlockScan<int, RSG_CT> S;
    __shared__ typename S::TempStorage tmp;
    Chunk c = CH[blockIdx.x];
    int b = threadIdx.x * RSG_CI, e = min(b + RSG_CI, c.n), loc = 0;
    for (int k = b; k < e; k++) loc += flag[c.start + k];
    int ex;
    S(tmp).ExclusiveSum(loc, ex);
    int run = (int)cp[blockIdx.x].i[0] + ex;
    for (int k = b; k < e; k++) {
        run += flag[c.start + k];
        cnt[c.start + k] = run;
    }
}

// ---- calculate_corevel (src/properties.c:165-214) --------------------------
// rmax: the largest j with j^2 > r2_j^3 (4/3 pi rvir_dens)^2
__global__ void __launch_bounds__(RSG_CT) k_cv_rmax(const Chunk *CH, const PotRec *PO,
                                                    const DevCfg *Cp, CP *cp) {
    typedef cub::BlockReduce<long long, RSG_CT> R;
    __shared__ typename R::TempStorage tmp;
    Chunk c = CH[blockIdx.x];
    double rt = Cp->rvir_dens * (4.0 * M_PI / 3.0);
    long long best = 0;  // j + 1
    for (int k = threadIdx.x; k < c.n; k += RSG_CT) {
        int64_t j = c.first + k;
        float r2 = PO[c.start + k].r2;
        if ((double)(j * j) > (double)fmul(fmul(r2, r2), r2) * (rt * rt)) best = j + 1;
    }
    best = R(tmp).Reduce(best, MaxLL());
    if (threadIdx.x == 0) cp[blockIdx.x].i[0] = best;
}
__global__ void k_cv_fin1(int32_t NH, const rsg_halo *H, const int32_t *c0, const int32_t *nch,
                          const CP *cp, HS *S) {
    int h = blockIdx.x * blockDim.x + threadIdx.x;
    if (h >= NH || H[h].num_p < 1) return;
    long long b = 0;
    for (int c = c0[h]; c < c0[h] + nch[h]; c++) b = max(b, cp[c].i[0]);
    S[h].rmax = b - 1;
}
// cmax: the largest j with 100 r2_j < r2_rmax
__global__ void __launch_bounds__(RSG_CT) k_cv_cmax(const Chunk *CH, const PotRec *PO,
                                                    const int32_t *toff, const HS *S, CP *cp) {
    typedef cub::BlockReduce<long long, RSG_CT> R;
    __shared__ typename R::TempStorage tmp;
    Chunk c = CH[blockIdx.x];
    int64_t rmax = S[c.halo].rmax;
    if (rmax < 1) return;
    double thr = (double)PO[toff[c.halo] + rmax].r2;
    long long best = 0;
    for (int k = threadIdx.x; k < c.n; k += RSG_CT)
        if ((double)PO[c.start + k].r2 * 100.0 < thr) best = c.first + k + 1;
    best = R(tmp).Reduce(best, MaxLL());
    if (threadIdx.x == 0) cp[blockIdx.x].i[0] = best;
}
__global__ void k_cv_fin2(int32_t NH, const rsg_halo *H, const int32_t *c0, const int32_t *nch,
                          const CP *cp, const PotRec *PO, const int32_t *toff, HS *S) {
    int h = blockIdx.x * blockDim.x + threadIdx.x;
    if (h >= NH || H[h].num_p < 1 || S[h].rmax < 1) return;
    long long b = 0;
    for (int c = c0[h]; c < c0[h] + nch[h]; c++) b = max(b, cp[c].i[0]);
    S[h].cmax = b - 1 < 100 ? 100 : b - 1;
    for (int k = 0; k < 3; k++) S[h].x0[k] = (double)PO[toff[h]].pos[k + 3];
}
// sums of y = v - v_0 and y^2 over i < rmax, per chunk
__global__ void __launch_bounds__(RSG_CT) k_cv_sums(const Chunk *CH, const PotRec *PO,
                                                    const HS *S, CP *cp) {
    typedef cub::BlockReduce<D6, RSG_CT> R;
    __shared__ typename R::TempStorage tmp;
    Chunk c = CH[blockIdx.x];
    const HS &s = S[c.halo];
    if (s.rmax < 1) return;
    D6 a = {{0, 0, 0, 0, 0, 0}};
    for (int k = threadIdx.x; k < c.n; k += RSG_CT) {
        if (c.first + k >= s.rmax) break;
        for (int d = 0; d < 3; d++) {
            double y = (double)PO[c.start + k].pos[d + 3] - s.x0[d];
            a.v[d] += y;
            a.v[d + 3] += y * y;
        }
    }
    a = R(tmp).Reduce(a, SumD6());
    if (threadIdx.x == 0)
        for (int d = 0; d < 6; d++) cp[blockIdx.x].d[d] = a.v[d];
}
__global__ void k_cv_off(int32_t NH, const rsg_halo *H, const int32_t *c0, const int32_t *nch,
                         const HS *S, CP *cp) {
    int h = blockIdx.x * blockDim.x + threadIdx.x;
    if (h >= NH || H[h].num_p < 1 || S[h].rmax < 1) return;
    double run[6] = {0, 0, 0, 0, 0, 0};
    for (int c = c0[h]; c < c0[h] + nch[h]; c++)
        for (int d = 0; d < 6; d++) {
            double t = cp[c].d[d];
            cp[c].d[d] = run[d];
            run[d] += t;
        }
}
// running mean and variance at every i < rmax from prefix sums, the test
// value g_i = tv_i / ((i-3) i) (0 for i <= 3), and per chunk the first
// minimum of g over [9, rmax) and over [9, min(cmax, rmax))
__global__ void __launch_bounds__(RSG_CT) k_cv_scan(const Chunk *CH, const PotRec *PO,
                                                    const HS *S, CP *cp, double *g,
                                                    float *vel) {
    typedef cub::BlockScan<D6, RSG_CT> Sc;
    typedef cub::BlockReduce<VI, RSG_CT> R;
    __shared__ union {
        typename Sc::TempStorage s;
        typename R::TempStorage r;
    } tmp;
    Chunk c = CH[blockIdx.x];
    const HS &s = S[c.halo];
    if (s.rmax < 1) return;
    int64_t rmax = s.rmax, rc = s.cmax < rmax ? s.cmax : rmax;
    int b = threadIdx.x * RSG_CI, e = min(b + RSG_CI, c.n);
    D6 loc = {{0, 0, 0, 0, 0, 0}};
    for (int k = b; k < e && c.first + k < rmax; k++)
        for (int d = 0; d < 3; d++) {
            double y = (double)PO[c.start + k].pos[d + 3] - s.x0[d];
            loc.v[d] += y;
            loc.v[d + 3] += y * y;
        }
    D6 ex;
    D6 zero = {{0, 0, 0, 0, 0, 0}};
    Sc(tmp.s).ExclusiveScan(loc, ex, zero, SumD6());
    __syncthreads();  // tmp is reused by the reductions below
    double run[6];
    for (int d = 0; d < 6; d++) run[d] = cp[blockIdx.x].d[d] + ex.v[d];
    VI ba = {INFINITY, LLONG_MAX}, bc = {INFINITY, LLONG_MAX};
    for (int k = b; k < e; k++) {
        int64_t i = c.first + k;
        if (i >= rmax) break;
        double n = (double)(i + 1), tv = 0;
        for (int d = 0; d < 3; d++) {
            double y = (double)PO[c.start + k].pos[d + 3] - s.x0[d];
            run[d] += y;
            run[d + 3] += y * y;
            double m2 = run[d + 3] - run[d] * run[d] / n;
            tv = (d == 0) ? m2 : tv + m2;
            vel[3 * (int64_t)(c.start + k) + d] = (float)(s.x0[d] + run[d] / n);
        }
        double gi = (i > 3) ? tv / (double)((i - 3) * i) : 0.0;
        g[c.start + k] = gi;
        if (i >= 9) {
            if (gi < ba.v) { ba.v = gi; ba.j = i; }
            if (i < rc && gi < bc.v) { bc.v = gi; bc.j = i; }
        }
    }
    ba = R(tmp.r).Reduce(ba, ArgMin());
    __syncthreads();
    bc = R(tmp.r).Reduce(bc, ArgMin());
    if (threadIdx.x == 0) {
        cp[blockIdx.x].d[6] = ba.v;
        cp[blockIdx.x].i[0] = ba.j;
        cp[blockIdx.x].d[7] = bc.v;
        cp[blockIdx.x].i[1] = bc.j;
    }
}
// the last update of the reference's loop is the first minimum of g after
// the forced updates of i < 10 (strict test: equal values do not update)
__global__ void k_cv_fin3(int32_t NH, rsg_halo *H, const int32_t *c0, const int32_t *nch,
                          const CP *cp, const HS *S, const int32_t *toff, const double *g,
                          const float *vel) {
    int h = blockIdx.x * blockDim.x + threadIdx.x;
    if (h >= NH || H[h].num_p < 1 || S[h].rmax < 1) return;
    int64_t rmax = S[h].rmax, ua = rmax - 1, uc = rmax - 1;
    if (rmax > 10) {
        VI a = {INFINITY, LLONG_MAX}, b = {INFINITY, LLONG_MAX};
        for (int c = c0[h]; c < c0[h] + nch[h]; c++) {
            VI x = {cp[c].d[6], cp[c].i[0]}, y = {cp[c].d[7], cp[c].i[1]};
            a = ArgMin()(a, x);
            b = ArgMin()(b, y);
        }
        // no comparable value after i = 9 (NaN): the forced update at 9 is the last
        ua = (a.j == LLONG_MAX) ? 9 : a.j;
        uc = (b.j == LLONG_MAX) ? 9 : b.j;
    }
    rsg_halo &hh = H[h];
    int64_t ra = toff[h] + ua, rc = toff[h] + uc;
    hh.n_core = uc;
    hh.min_vel_err = (float)g[rc];
    hh.min_bulkvel_err = (float)g[ra];
    for (int k = 0; k < 3; k++) {
        hh.corevel[k] = vel[3 * rc + k];
        hh.bulkvel[k] = vel[3 * ra + k];
        hh.pos[k + 3] = hh.corevel[k];
    }
}

// compute_kinetic_energy about the core (subhalos) or bulk velocity
__global__ void __launch_bounds__(RSG_CT) k_sg_kinetic(const Chunk *CH, PotRec *PO,
                                                       const rsg_halo *H,
                                                       const rsg_extra_halo_info *E,
                                                       const DevCfg *Cp) {
    Chunk c = CH[blockIdx.x];
    const DevCfg &C = *Cp;
    const rsg_halo &hh = H[c.halo];
    float sn = (float)C.scale_now;
    const float *vc = (E[c.halo].sub_of > -1) ? hh.corevel : hh.bulkvel;
    double conv = 0.5 * (double)sn / RSG_GC;
    double hub = C.hub;
    float vv[3] = {vc[0], vc[1], vc[2]}, pp[3] = {hh.pos[0], hh.pos[1], hh.pos[2]};
    for (int k = threadIdx.x; k < c.n; k += RSG_CT) {
        PotRec &q = PO[c.start + k];
        if (q.ke < 0) continue;
        float ke = 0;
        for (int j = 0; j < 3; j++) {
            double dv = (double)fsub(q.pos[j + 3], vv[j]) +
                        hub * (double)sn * (double)fsub(q.pos[j], pp[j]);
            ke = (float)((double)ke + dv * dv);
        }
        q.ke = (float)((double)ke * conv);
    }
}

// ---- _calc_additional_halo_props (src/properties.c:384-510) ----------------
// per-record flag: mode 0 = analysed in this bound pass (!(bound && pe < ke)),
// mode 1 = counted by estimate_total_energy (j < dtot && pe > ke)
__global__ void __launch_bounds__(RSG_CT) k_sg_flag(const Chunk *CH, const PotRec *PO,
                                                    const HS *S, int bound, int mode,
                                                    uint8_t *flag) {
    Chunk c = CH[blockIdx.x];
    int64_t dtot = S[c.halo].dtot;
    for (int k = threadIdx.x; k < c.n; k += RSG_CT) {
        const PotRec &q = PO[c.start + k];
        uint8_t f;
        if (mode == 0) f = !(bound && unbound(q));
        else f = (c.first + k < dtot) && q.pe > (double)q.ke;
        flag[c.start + k] = f;
    }
}
// pass 1: densities at every analysed particle; the thresholds keep the
// largest running count (counts grow with j), dtot the last qualifying j and
// j0 the first one
__global__ void __launch_bounds__(RSG_CT) k_sg_p1(const Chunk *CH, const PotRec *PO,
                                                  const uint8_t *flag, const int32_t *cnt,
                                                  const DevCfg *Cp, CP *cp) {
    typedef cub::BlockReduce<I8, RSG_CT> R;
    __shared__ typename R::TempStorage tmp;
    const DevCfg &C = *Cp;
    Chunk c = CH[blockIdx.x];
    const double f43 = 4.0 * M_PI / 3.0;
    const double th[6] = {C.thresh_dens[0] * f43, C.thresh_dens[1] * f43, C.thresh_dens[2] * f43,
                          C.thresh_dens[3] * f43, C.thresh_dens[4] * f43, C.rvir_dens * f43};
    I8 a = {{0, 0, 0, 0, 0, 0, 0, LLONG_MAX}};
    for (int k = threadIdx.x; k < c.n; k += RSG_CT) {
        int64_t rec = c.start + k, j = c.first + k;
        if (!flag[rec]) continue;
        long long np_ = cnt[rec];
        double r = sqrt((double)PO[rec].r2);
        if (r < C.force_res) r = C.force_res;
        double cd = ((double)np_ / (r * r * r));
        if (cd > th[0]) {
            a.v[0] = max(a.v[0], np_);
            a.v[1] = max(a.v[1], (long long)j);
            a.v[7] = min(a.v[7], (long long)j);
        }
        for (int t = 1; t < 6; t++)
            if (cd > th[t]) a.v[1 + t] = max(a.v[1 + t], np_);
    }
    a = R(tmp).Reduce(a, MaxMin8());
    if (threadIdx.x == 0)
        for (int t = 0; t < 8; t++) cp[blockIdx.x].i[t] = a.v[t];
}
__global__ void k_sg_p1_fin(int32_t NH, rsg_halo *H, const int32_t *c0, const int32_t *nch,
                            const CP *cp, const DevCfg *Cp, int bound, HS *S) {
    int h = blockIdx.x * blockDim.x + threadIdx.x;
    if (h >= NH || H[h].num_p < 1) return;
    I8 a = {{0, 0, 0, 0, 0, 0, 0, LLONG_MAX}};
    for (int c = c0[h]; c < c0[h] + nch[h]; c++) {
        I8 b;
        for (int t = 0; t < 8; t++) b.v[t] = cp[c].i[t];
        a = MaxMin8()(a, b);
    }
    HS &s = S[h];
    s.pmd = a.v[0];
    s.dtot = a.v[0] > 0 ? a.v[1] : 0;
    for (int k = 0; k < 4; k++) s.npa[k] = a.v[2 + k];
    s.npv = a.v[6];
    s.j0 = a.v[7];
    s.m = s.pmd * Cp->particle_mass;
    if (!bound) H[h].m = (float)s.m;
    else H[h].mgrav = (float)s.m;
}
// Vmax: the first maximum of np/r over analysed particles at or after j0
// above the virial density
__global__ void __launch_bounds__(RSG_CT) k_sg_vmax(const Chunk *CH, const PotRec *PO,
                                                    const uint8_t *flag, const int32_t *cnt,
                                                    const HS *S, const DevCfg *Cp, CP *cp) {
    typedef cub::BlockReduce<VI, RSG_CT> R;
    __shared__ typename R::TempStorage tmp;
    const DevCfg &C = *Cp;
    Chunk c = CH[blockIdx.x];
    const double rth = C.rvir_dens * (4.0 * M_PI / 3.0);
    int64_t j0 = S[c.halo].j0;
    VI b = {-1.0, LLONG_MAX};
    for (int k = threadIdx.x; k < c.n; k += RSG_CT) {
        int64_t rec = c.start + k, j = c.first + k;
        if (!flag[rec] || j < j0) continue;
        double r = sqrt((double)PO[rec].r2);
        if (r < C.force_res) r = C.force_res;
        double np_ = (double)cnt[rec], cd = np_ / (r * r * r);
        if (cd > rth) {
            VI x = {np_ / r, (long long)j};
            b = ArgMax()(b, x);
        }
    }
    b = R(tmp).Reduce(b, ArgMax());
    if (threadIdx.x == 0) {
        cp[blockIdx.x].d[0] = b.v;
        cp[blockIdx.x].i[0] = b.j;
    }
}
__global__ void k_sg_vmax_fin(int32_t NH, const rsg_halo *H, const int32_t *c0,
                              const int32_t *nch, const CP *cp, const PotRec *PO,
                              const int32_t *toff, const DevCfg *Cp, HS *S) {
    int h = blockIdx.x * blockDim.x + threadIdx.x;
    if (h >= NH || H[h].num_p < 1) return;
    VI b = {-1.0, LLONG_MAX};
    for (int c = c0[h]; c < c0[h] + nch[h]; c++) {
        VI x = {cp[c].d[0], cp[c].i[0]};
        b = ArgMax()(b, x);
    }
    S[h].vmax = 0;
    S[h].rvmax = 0;
    if (b.v > 0 && b.j != LLONG_MAX) {
        S[h].vmax = b.v;
        double r = sqrt((double)PO[toff[h] + b.j].r2);
        if (r < Cp->force_res) r = Cp->force_res;
        S[h].rvmax = r;
    }
}
struct CN {
    long long c, nh;
};
struct SumMin {
    __device__ CN operator()(const CN &a, const CN &b) const {
        CN r = {a.c + b.c, a.nh < b.nh ? a.nh : b.nh};
        return r;
    }
};
// pass 2 over [0, dtot): angular momentum, mean position and velocity, the
// half-mass index
__global__ void __launch_bounds__(RSG_CT) k_sg_p2(const Chunk *CH, const PotRec *PO,
                                                  const rsg_halo *H, const uint8_t *flag,
                                                  const int32_t *cnt, const HS *S, CP *cp) {
    typedef cub::BlockReduce<D9, RSG_CT> R;
    typedef cub::BlockReduce<CN, RSG_CT> R2;
    __shared__ union {
        typename R::TempStorage a;
        typename R2::TempStorage b;
    } tmp;
    Chunk c = CH[blockIdx.x];
    const HS &s = S[c.halo];
    float ce[6];
    for (int k = 0; k < 6; k++) ce[k] = H[c.halo].pos[k];
    D9 a = {{0, 0, 0, 0, 0, 0, 0, 0, 0}};
    CN n = {0, LLONG_MAX};
    for (int k = threadIdx.x; k < c.n; k += RSG_CT) {
        int64_t rec = c.start + k, j = c.first + k;
        if (j >= s.dtot) break;
        if (!flag[rec]) continue;
        const float *p = PO[rec].pos;
        for (int d = 0; d < 3; d++) {
            int x = (d + 1) % 3, y = (d + 2) % 3;
            a.v[d] += (double)fmul(fsub(p[x], ce[x]), fsub(p[y + 3], ce[y + 3]));
            a.v[d] -= (double)fmul(fsub(p[y], ce[y]), fsub(p[x + 3], ce[x + 3]));
            a.v[3 + d] += (double)p[d];
            a.v[6 + d] += (double)p[d + 3];
        }
        n.c++;
        if (j >= 1 && (long long)cnt[rec] * 2 >= s.pmd && j < n.nh) n.nh = j;
    }
    a = R(tmp.a).Reduce(a, SumD9());
    __syncthreads();
    n = R2(tmp.b).Reduce(n, SumMin());
    if (threadIdx.x == 0) {
        for (int d = 0; d < 9; d++) cp[blockIdx.x].d[d] = a.v[d];
        cp[blockIdx.x].i[0] = n.c;
        cp[blockIdx.x].i[1] = n.nh;
    }
}
__global__ void k_sg_p2_fin(int32_t NH, const rsg_halo *H, const int32_t *c0, const int32_t *nch,
                            const CP *cp, HS *S) {
    int h = blockIdx.x * blockDim.x + threadIdx.x;
    if (h >= NH || H[h].num_p < 1) return;
    double a[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
    long long cn = 0, nh = LLONG_MAX;
    for (int c = c0[h]; c < c0[h] + nch[h]; c++) {
        for (int d = 0; d < 9; d++) a[d] += cp[c].d[d];
        cn += cp[c].i[0];
        nh = min(nh, cp[c].i[1]);
    }
    HS &s = S[h];
    double tc = (double)cn;
    for (int k = 0; k < 3; k++) {
        s.L[k] = a[k];
        s.xa[k] = tc > 0 ? a[3 + k] / tc : 0;
        s.va[k] = tc > 0 ? a[6 + k] / tc : 0;
    }
    s.avg = cn;
    s.nhalf = (nh == LLONG_MAX) ? 0 : nh;
}
// second moments of the velocities about their mean, over [0, dtot)
__global__ void __launch_bounds__(RSG_CT) k_sg_v2(const Chunk *CH, const PotRec *PO,
                                                  const uint8_t *flag, const HS *S, CP *cp) {
    typedef cub::BlockReduce<D6, RSG_CT> R;
    __shared__ typename R::TempStorage tmp;
    Chunk c = CH[blockIdx.x];
    const HS &s = S[c.halo];
    D6 a = {{0, 0, 0, 0, 0, 0}};
    for (int k = threadIdx.x; k < c.n; k += RSG_CT) {
        int64_t rec = c.start + k;
        if (c.first + k >= s.dtot) break;
        if (!flag[rec]) continue;
        for (int d = 0; d < 3; d++) {
            double x = (double)PO[rec].pos[d + 3] - s.va[d];
            a.v[d] += x * x;
        }
    }
    a = R(tmp).Reduce(a, SumD6());
    if (threadIdx.x == 0)
        for (int d = 0; d < 3; d++) cp[blockIdx.x].d[d] = a.v[d];
}
// the halo fields of the analysed bound pass (src/properties.c:452-475)
__global__ void k_sg_v2_fin(int32_t NH, rsg_halo *H, const int32_t *c0, const int32_t *nch,
                            const CP *cp, const PotRec *PO, const int32_t *toff,
                            const DevCfg *Cp, HS *S) {
    int h = blockIdx.x * blockDim.x + threadIdx.x;
    if (h >= NH || H[h].num_p < 1) return;
    const DevCfg &C = *Cp;
    HS &s = S[h];
    rsg_halo &hh = H[h];
    double v2[3] = {0, 0, 0};
    for (int c = c0[h]; c < c0[h] + nch[h]; c++)
        for (int d = 0; d < 3; d++) v2[d] += cp[c].d[d];
    double vr[3];
    for (int k = 0; k < 3; k++) vr[k] = (s.avg > 0) ? (v2[k] / s.avg) : 0;
    float scale = (float)C.scale_now;
    double ds;
    hh.Xoff = hh.Voff = 0;
    for (int k = 0; k < 3; k++) {
        ds = s.xa[k] - (double)hh.pos[k];
        hh.Xoff = (float)((double)hh.Xoff + ds * ds);
        ds = s.va[k] - (double)hh.pos[k + 3];
        hh.Voff = (float)((double)hh.Voff + ds * ds);
    }
    for (int k = 0; k < 4; k++) hh.alt_m[k] = (float)(s.npa[k] * C.particle_mass);
    hh.Xoff = (float)(sqrt((double)hh.Xoff) * 1e3);
    hh.Voff = sqrt_fd(hh.Voff);
    hh.vrms = (float)sqrt(vr[0] + vr[1] + vr[2]);
    hh.vmax = (float)(RSG_VMAX_CONST * sqrt(s.vmax * (C.particle_mass / (double)scale)));
    hh.rvmax = (float)(s.rvmax * 1e3);
    hh.halfmass_radius = (float)(sqrt((double)PO[toff[h] + s.nhalf].r2) * 1e3);
    hh.r = (float)(cbrt((3.0 / (4.0 * M_PI)) * s.npa[2] / C.thresh_dens[3]) * 1e3);
}

// ---- calc_shape (src/properties.c:216-326) ---------------------------------
// which = 0: the R_500c set [0, npa[2]); which = 1: the R_Delta set
// [0, dtot), after the first set's results move to the *2 fields
// Sets of at most this many records run the reference's loop itself, one
// thread per halo (shape(), in the records' order): with a handful of
// particles the inertia tensor is close to singular and its smallest
// eigenvalue is rounding noise, so only the reference's own summation order
// reproduces its axis ratios.
#define RSG_SHAPE_SEQ 256
__global__ void k_sh_init(int32_t NH, rsg_halo *H, const int32_t *cnt, const int32_t *toff,
                          const DevCfg *Cp, int which, HS *S) {
    int h = blockIdx.x * blockDim.x + threadIdx.x;
    if (h >= NH || H[h].num_p < 1) return;
    const DevCfg &C = *Cp;
    HS &s = S[h];
    rsg_halo &hh = H[h];
    int64_t set = s.npa[2];
    if (which) {
        hh.b_to_a2 = hh.b_to_a;
        hh.c_to_a2 = hh.c_to_a;
        for (int k = 0; k < 3; k++) hh.A2[k] = hh.A[k];
        for (int k = 0; k < 6; k++) hh.inertia_tensor2[k] = hh.inertia_tensor[k];
        hh.r = (float)(cbrt((3.0 / (4.0 * M_PI)) * s.pmd / C.thresh_dens[0]) * 1e3);
        set = s.dtot;
    }
    s.set = (int32_t)set;
    if (set <= RSG_SHAPE_SEQ) {  // k_sh_small's
        s.done = 1;
        return;
    }
    int64_t an = (set > 0) ? cnt[toff[h] + set - 1] : 0, it = C.shape_iterations;
    s.iter = 0;
    s.done = 0;
    float minr = fmul((float)C.force_res, (float)C.force_res);
    hh.b_to_a = hh.c_to_a = 0;
    hh.A[0] = hh.A[1] = hh.A[2] = 0;
    if (!(hh.r > 0)) {
        s.done = 1;
        return;
    }
    minr = (float)((double)minr * (1e6 / (double)fmul(hh.r, hh.r)));
    if (an < 3) s.done = 1;
    if (an < it) it = an;
    for (int i = 0; i < 3; i++) {
        for (int k = 0; k < 3; k++) s.orth[i][k] = 0;
        s.orth[i][i] = 1;
        s.eig[i] = (double)fmul(hh.r, hh.r) * 1e-6;
    }
    s.minr = minr;
    s.it = (int32_t)it;
    if (it <= 0) s.done = 1;
}
// The small sets of k_sh_init: shape_batch, 32 halos per warp.
__global__ void __launch_bounds__(128) k_sh_small(int32_t NH, rsg_halo *H, const int32_t *toff,
                                                  const PotRec *PO, const DevCfg *Cp,
                                                  const HS *S, int bound) {
    __shared__ ShapeBatch sb[4];
    ShapeBatch &B = sb[threadIdx.x >> 5];
    const int32_t base = ((blockIdx.x * blockDim.x + threadIdx.x) >> 5) * 32;
    if (base >= NH) return;
    const int lane = threadIdx.x & 31;
    const int32_t h = base + lane;
    B.set[lane] = (h < NH && H[h].num_p >= 1 && S[h].set <= RSG_SHAPE_SEQ) ? S[h].set : -1;
    __syncwarp();
    shape_batch(H, toff, PO, base, NH, bound, *Cp, B);
}
__global__ void __launch_bounds__(RSG_CT) k_sh_sum(const Chunk *CH, const PotRec *PO,
                                                   const rsg_halo *H, const uint8_t *flag,
                                                   const HS *S, const DevCfg *Cp, CP *cp) {
    typedef cub::BlockReduce<D9, RSG_CT> R;
    __shared__ typename R::TempStorage tmp;
    Chunk c = CH[blockIdx.x];
    const HS &s = S[c.halo];
    if (s.done) return;
    const float hp0 = H[c.halo].pos[0], hp1 = H[c.halo].pos[1], hp2 = H[c.halo].pos[2];
    const int ws = (int)Cp->weighted_shapes;
    // The ellipsoidal radius r = sum_q (o_q . d)^2 / eig_q as the quadratic
    // form d^T M d with M = O^T diag(1/eig) O, formed once per block, on the
    // six products d_k d_l the tensor sums need anyway (about 40 FP64
    // operations per record instead of 90: GB300's FP64 pipe bounds this
    // pass).  The value differs from the reference's expression by rounding
    // only, as the batched form's order of summation does already.
    double Mq[6] = {0, 0, 0, 0, 0, 0};  // M00 M11 M22 2M01 2M02 2M12
    for (int q = 0; q < 3; q++) {
        const double iq = 1.0 / s.eig[q];
        const double o0 = s.orth[q][0], o1 = s.orth[q][1], o2 = s.orth[q][2];
        Mq[0] += iq * o0 * o0;
        Mq[1] += iq * o1 * o1;
        Mq[2] += iq * o2 * o2;
        Mq[3] += 2.0 * iq * o0 * o1;
        Mq[4] += 2.0 * iq * o0 * o2;
        Mq[5] += 2.0 * iq * o1 * o2;
    }
    const double minr = (double)s.minr;
    D9 a = {{0, 0, 0, 0, 0, 0, 0, 0, 0}};
    for (int k = threadIdx.x; k < c.n; k += RSG_CT) {
        int64_t rec = c.start + k;
        if (c.first + k >= s.set) break;
        if (!flag[rec]) continue;
        const float *p = PO[rec].pos;
        const double d0 = (double)fsub(p[0], hp0), d1 = (double)fsub(p[1], hp1),
                     d2 = (double)fsub(p[2], hp2);
        const double p00 = d0 * d0, p11 = d1 * d1, p22 = d2 * d2, p01 = d0 * d1, p02 = d0 * d2,
                     p12 = d1 * d2;
        double r = Mq[0] * p00 + Mq[1] * p11 + Mq[2] * p22 + Mq[3] * p01 + Mq[4] * p02 +
                   Mq[5] * p12;
        if (r < minr) r = minr;
        if (r > 0 && r <= 1) {
            double tw = 1.0;
            if (ws) {
                // 1/r: an FP32 estimate and two Newton steps in FP64 (about
                // 2^-52 relative, for an FP64 divide's many operations)
                if (r > 1e-30) {
                    tw = (double)__frcp_rn((float)r);
                    tw = fma(tw, fma(-r, tw, 1.0), tw);
                    tw = fma(tw, fma(-r, tw, 1.0), tw);
                } else {
                    tw = 1.0 / r;
                }
            }
            a.v[0] += tw;
            a.v[1] += p00 * tw;
            a.v[2] += p11 * tw;
            a.v[3] += p22 * tw;
            a.v[4] += p01 * tw;
            a.v[5] += p02 * tw;
            a.v[6] += p12 * tw;
        }
    }
    a = R(tmp).Reduce(a, SumD9());
    if (threadIdx.x == 0)
        for (int d = 0; d < 7; d++) cp[blockIdx.x].d[d] = a.v[d];
}
__global__ void k_sh_fin(int32_t NH, rsg_halo *H, const int32_t *c0, const int32_t *nch,
                         const CP *cp, HS *S) {
    int h = blockIdx.x * blockDim.x + threadIdx.x;
    if (h >= NH || H[h].num_p < 1) return;
    HS &s = S[h];
    if (s.done) return;
    rsg_halo &hh = H[h];
    double acc[7] = {0, 0, 0, 0, 0, 0, 0};
    for (int c = c0[h]; c < c0[h] + nch[h]; c++)
        for (int d = 0; d < 7; d++) acc[d] += cp[c].d[d];
    double w = acc[0];
    if (!w) {
        s.done = 1;
        return;
    }
    double m[3][3] = {{acc[1], acc[4], acc[5]}, {acc[4], acc[2], acc[6]}, {acc[5], acc[6], acc[3]}};
    for (int k = 0; k < 3; k++)
        for (int l = 0; l < 3; l++) m[k][l] /= (double)w;
    double mt2[3][3], o2[3][3], e2[3];
    for (int k = 0; k < 3; k++)
        for (int l = 0; l < 3; l++) mt2[k][l] = m[k][l];
    jacobi3(m, e2, o2);
    int a2 = 0, b = 1, c = 2;
    if (e2[1] > e2[0]) { b = 0; a2 = 1; }
    if (e2[2] > e2[b]) { c = b; b = 2; }
    if (e2[b] > e2[a2]) { int t = a2; a2 = b; b = t; }
    for (int k = 0; k < 3; k++) {
        s.eig[k] = e2[k];
        for (int l = 0; l < 3; l++) s.orth[k][l] = o2[k][l];
    }
    if (!e2[a2] || !e2[b] || !e2[c]) {
        s.done = 1;
        return;
    }
    float ba = (float)sqrt(e2[b] / e2[a2]);
    float ca = (float)sqrt(e2[c] / e2[a2]);
    if ((fabs((double)fsub(ba, hh.b_to_a)) < 0.01 * (double)hh.b_to_a) &&
        (fabs((double)fsub(ca, hh.c_to_a)) < 0.01 * (double)hh.c_to_a)) {
        s.done = 1;
        return;
    }
    hh.b_to_a = (ba > 0) ? ba : 0;
    hh.c_to_a = (ca > 0) ? ca : 0;
    double rr = sqrt(e2[a2]);
    for (int k = 0; k < 3; k++) {
        hh.A[k] = (float)(1e3 * rr * o2[a2][k]);
        s.eig[k] *= ((double)fmul(hh.r, hh.r) * 1e-6) / (rr * rr);
    }
    hh.inertia_tensor[0] = (float)mt2[0][0];
    hh.inertia_tensor[1] = (float)mt2[1][1];
    hh.inertia_tensor[2] = (float)mt2[2][2];
    hh.inertia_tensor[3] = (float)mt2[0][1];
    hh.inertia_tensor[4] = (float)mt2[1][2];
    hh.inertia_tensor[5] = (float)mt2[2][0];
    if (++s.iter >= s.it) s.done = 1;
}

// ---- estimate_total_energy (src/properties.c:328-349) ----------------------
// tphi = sum_i m i / r_i + sum_i (m / r_i) (number of counted particles
// before i): the reference's descending running sum, regrouped
__global__ void __launch_bounds__(RSG_CT) k_sg_energy(const Chunk *CH, const PotRec *PO,
                                                      const uint8_t *flag, const int32_t *cnt,
                                                      const DevCfg *Cp, CP *cp) {
    typedef cub::BlockReduce<D6, RSG_CT> R;
    __shared__ typename R::TempStorage tmp;
    const DevCfg &C = *Cp;
    Chunk c = CH[blockIdx.x];
    D6 a = {{0, 0, 0, 0, 0, 0}};
    for (int k = threadIdx.x; k < c.n; k += RSG_CT) {
        int64_t rec = c.start + k, i = c.first + k;
        if (!flag[rec]) continue;
        double r = sqrt((double)PO[rec].r2);
        if (r < C.force_res) r = C.force_res;
        a.v[0] += (double)PO[rec].ke;
        a.v[1] += C.particle_mass * i / r + (C.particle_mass / r) * (double)(cnt[rec] - 1);
    }
    a = R(tmp).Reduce(a, SumD6());
    if (threadIdx.x == 0) {
        cp[blockIdx.x].d[0] = a.v[0];
        cp[blockIdx.x].d[1] = a.v[1];
    }
}
__global__ void k_sg_energy_fin(int32_t NH, const rsg_halo *H, const int32_t *c0,
                                const int32_t *nch, const CP *cp, HS *S) {
    int h = blockIdx.x * blockDim.x + threadIdx.x;
    if (h >= NH || H[h].num_p < 1) return;
    double a = 0, b = 0;
    for (int c = c0[h]; c < c0[h] + nch[h]; c++) {
        a += cp[c].d[0];
        b += cp[c].d[1];
    }
    S[h].kes = a;
    S[h].ts = b;
}

// ---- calc_scale_radius (src/nfw.c:130-173) ---------------------------------
// bins of pp analysed particles over [0, dtot - 1): the bin edge after the
// k-th group of pp sits between the particle whose running count is k pp and
// the next particle
__global__ void k_nfw_init(int32_t NH, rsg_halo *H, const int32_t *cnt, const int32_t *toff,
                           const DevCfg *Cp, HS *S) {
    int h = blockIdx.x * blockDim.x + threadIdx.x;
    if (h >= NH || H[h].num_p < 1) return;
    HS &s = S[h];
    rsg_halo &hh = H[h];
    float scale = (float)Cp->scale_now;
    float rs = hh.klypin_rs = klypin_rs((float)s.m, hh.r, hh.vmax, hh.rvmax, scale);
    int64_t an = (s.dtot >= 2) ? cnt[toff[h] + s.dtot - 2] : 0;
    s.an = an;
    s.pp = 0;
    if (an < 100) {
        hh.rs = rs;
        return;
    }
    int64_t pp = (int64_t)ceil(((double)an / (double)50));
    if (pp < 15) pp = (an) / ((int64_t)(an / 15));
    s.pp = pp;
    for (int i = 0; i < 51; i++) s.br[i] = 0;
    for (int i = 0; i < 50; i++) s.w[i] = 0;
}
__global__ void __launch_bounds__(RSG_CT) k_nfw_bins(const Chunk *CH, const PotRec *PO,
                                                     const uint8_t *flag, const int32_t *cnt,
                                                     HS *S) {
    Chunk c = CH[blockIdx.x];
    HS &s = S[c.halo];
    int64_t pp = s.pp;
    if (pp <= 0) return;
    for (int k = threadIdx.x; k < c.n; k += RSG_CT) {
        int64_t rec = c.start + k;
        if (c.first + k >= s.dtot - 1) break;
        if (!flag[rec]) continue;
        int64_t n = cnt[rec];
        if (n % pp) continue;
        int64_t b = n / pp;
        if (b < 1 || b > 50) continue;
        s.br[b] = (float)(1e3 * 0.5 * (sqrt((double)PO[rec].r2) + sqrt((double)PO[rec + 1].r2)));
        s.w[b - 1] = 1;
    }
}
__global__ void k_nfw_fit(int32_t NH, rsg_halo *H, const DevCfg *Cp, const HS *S) {
    int h = blockIdx.x * blockDim.x + threadIdx.x;
    if (h >= NH || H[h].num_p < 1) return;
    const HS &s = S[h];
    if (s.pp <= 0) return;
    int64_t nb = s.an / s.pp;
    if (nb > 50) nb = 50;
    float br[51], w[50];
    for (int i = 0; i < 51; i++) br[i] = s.br[i];
    for (int i = 0; i < 50; i++) w[i] = s.w[i];
    br[0] = 0;
    for (int64_t i = 0; i < nb; i++)
        if ((double)br[i] * 1e-3 < 3 * Cp->force_res) w[i] = 0.1f;
    float chi2 = 0.0f;
    H[h].rs = fit_bins(H[h].klypin_rs, br, w, nb, &chi2);
    H[h].chi2 = chi2;
}

// ---- _calc_pseudo_evolution_masses (src/properties.c:351-382) and the last
// fields of _calc_additional_halo_props --------------------------------------
__global__ void __launch_bounds__(RSG_CT) k_sg_pseudo(const Chunk *CH, const PotRec *PO,
                                                      const rsg_halo *H, const uint8_t *flag,
                                                      const int32_t *cnt, CP *cp) {
    Chunk c = CH[blockIdx.x];
    const rsg_halo &hh = H[c.halo];
    double rpd = (double)hh.rs * 4.0;
    if (rpd < (double)hh.r / 5.0) rpd = (double)hh.r / 5.0;
    rpd *= 1e-3;
    VI a = {0.0, 0};  // v: max of np^2 / r^1.5, j: largest count inside rpd
    for (int k = threadIdx.x; k < c.n; k += RSG_CT) {
        int64_t rec = c.start + k;
        if (!flag[rec]) continue;
        long long np_ = cnt[rec];
        double r = sqrt((double)PO[rec].r2), r32 = sqrt(r);
        r32 = r32 * r32 * r32;
        double v = (double)(np_ * np_) / r32;
        if (v > a.v) a.v = v;
        if (r < rpd && np_ > a.j) a.j = np_;
    }
    __shared__ double smx[RSG_CT / 32];
    __shared__ long long snp[RSG_CT / 32];
    for (int o = 16; o; o >>= 1) {
        double v = __shfl_down_sync(0xffffffffu, a.v, o);
        long long j = __shfl_down_sync(0xffffffffu, a.j, o);
        if (v > a.v) a.v = v;
        if (j > a.j) a.j = j;
    }
    if ((threadIdx.x & 31) == 0) {
        smx[threadIdx.x >> 5] = a.v;
        snp[threadIdx.x >> 5] = a.j;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        for (int w = 1; w < RSG_CT / 32; w++) {
            if (smx[w] > a.v) a.v = smx[w];
            if (snp[w] > a.j) a.j = snp[w];
        }
        cp[blockIdx.x].d[0] = a.v;
        cp[blockIdx.x].i[0] = a.j;
    }
}
__global__ void k_sg_final(int32_t NH, rsg_halo *H, const int32_t *c0, const int32_t *nch,
                           const CP *cp, const DevCfg *Cp, const HS *S) {
    int h = blockIdx.x * blockDim.x + threadIdx.x;
    if (h >= NH || H[h].num_p < 1) return;
    const DevCfg &C = *Cp;
    const HS &s = S[h];
    rsg_halo &hh = H[h];
    double mx = 0;
    long long npd = 0;
    for (int c = c0[h]; c < c0[h] + nch[h]; c++) {
        if (cp[c].d[0] > mx) mx = cp[c].d[0];
        if (cp[c].i[0] > npd) npd = cp[c].i[0];
    }
    float scale = (float)C.scale_now;
    double rvir = cbrt((3.0 / (4.0 * M_PI)) * s.npv / C.rvir_dens) * 1e3;
    double mvir = s.npv * C.particle_mass, m = s.m;
    for (int j = 0; j < 3; j++) hh.J[j] = (float)(C.particle_mass * (double)scale * s.L[j]);
    {
        double ke = s.kes, tphi = s.ts / 2.0;
        hh.kin_to_pot = 0;
        if (tphi) hh.kin_to_pot = (float)(ke / tphi);
        float sn = (float)C.scale_now;
        hh.energy = (float)((ke - tphi) * C.particle_mass * RSG_GC / (double)sn);
    }
    double Jh = C.particle_mass * (double)scale *
                sqrt(s.L[0] * s.L[0] + s.L[1] * s.L[1] + s.L[2] * s.L[2]);
    hh.spin = (float)((m > 0) ? (Jh * sqrt(fabs((double)hh.energy)) / (RSG_GC * pow(m, 2.5))) : 0);
    hh.bullock_spin = (float)((m > 0) ? (Jh / (mvir * sqrt(2.0 * RSG_GC * mvir * rvir * (double)scale / 1e3))) : 0);
    hh.m_pe_d = (float)(npd * C.particle_mass);
    hh.m_pe_b = (float)(C.particle_mass * pow(mx, 2.0 / 3.0) /
                        cbrt(4.0 * M_PI * C.rvir_dens_z0 / 3.0));
}

}  // namespace rsg
