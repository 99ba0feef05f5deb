// Batched find_subs (src/groupies.c:520-708) on the GPU.
//
// The reference recurses depth first through the 6D subgroup hierarchy of one
// FOF group at a time.  Here all groups of a call are processed together and
// the recursion is unrolled by level:
//   descending, level L = 0, 1, ...: for every node of level L
//     norm_sd (FP64 moments + 3x3 Jacobi), 6D kd-tree (exact fast3tree
//     permutation), nearest-neighbour distances of the sample (glibc rand_r
//     stream, exact traversal order), the FOF_FRACTION quantile by the
//     reference's own randomised quickselect, 6D FOF at that length, and the
//     kept subgroups (>= MIN_HALO_PARTICLES) become level L+1 nodes when
//     MIN_HALO_PARTICLES < n < parent n (src/groupies.c:535-537);
//   halos: every node without recursed children creates one seed halo;
//     halo order is the depth-first order of those nodes, which is the order
//     of their first particle;
//   ascending, level L = max .. 0: for every node, the post-recursion part
//     of _find_subs (src/groupies.c:539-666): seed merging, particle
//     assignment by the phase-space metric, regrouping by halo, basic
//     properties and parent links.
// A node's work at a level only touches its own particle range, so running
// all nodes of a level at once performs the same operations, in the same
// order per range, as the reference's depth-first walk.
#include <cooperative_groups.h>
#include <cub/cub.cuh>

#include "kdtree_impl.cuh"
#include "lsort.cuh"
#include "subs.cuh"
#include "df64.cuh"
#include "uflabels.cuh"

// Ranges up to this size are summed by one thread in array order, so FP64
// sums round exactly as the reference's sequential loops do.
#define RSG_SEQ_MAX 65536
// Below this size one thread does all of a node's or halo's work.
#define RSG_SMALL 2048

namespace rsg {

namespace cg = cooperative_groups;

// Hierarchy record of the last find_subs call (level, first position, size,
// 6D linking length per node), kept for the test hooks.
std::vector<int32_t> g_dbg_level, g_dbg_start, g_dbg_n;
std::vector<float> g_dbg_target;

void additional_props(Arena &ar, const DevCfg &dc, const DevCfg *d_dc, const Rec *W,
                      int64_t M, rsg_halo *H, rsg_extra_halo_info *E, int32_t NH,
                      cudaStream_t st, int exact);

// ---- reductions -------------------------------------------------------------
__device__ __forceinline__ double warp_sum_d(double v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    return v;
}
// Deterministic block sum (fixed shuffle tree, then warp totals in order).
// All threads must call; the result is valid in every thread.
__device__ double block_sum_d(double v, double *sm) {
    int lane = threadIdx.x & 31, w = threadIdx.x >> 5, nw = (blockDim.x + 31) >> 5;
    v = warp_sum_d(v);
    __syncthreads();
    if (lane == 0) sm[w] = v;
    __syncthreads();
    double t = 0;
    if (threadIdx.x == 0) {
        for (int i = 0; i < nw; i++) t += sm[i];
        sm[32] = t;
    }
    __syncthreads();
    return sm[32];
}

// glibc's published rand_r (three steps of the ANSI C LCG, 31-bit result).
__device__ __forceinline__ int rand_r_glibc(unsigned *seed) {
    unsigned next = *seed;
    int result;
    next *= 1103515245u;
    next += 12345u;
    result = (unsigned)(next / 65536u) % 2048u;
    next *= 1103515245u;
    next += 12345u;
    result <<= 10;
    result ^= (unsigned)(next / 65536u) % 1024u;
    next *= 1103515245u;
    next += 12345u;
    result <<= 10;
    result ^= (unsigned)(next / 65536u) % 1024u;
    *seed = next;
    return result;
}

// ---- descending phase ---------------------------------------------------------

// norm_sd (src/groupies.c:788-830) + calc_deviations (src/jacobi.c:156-172).
// Moments go to mom[node * 27]: 6 means then the 21 upper-triangular
// second moments of the centred coordinates; sig[node * 2] gets sig_x, sig_v.
__device__ void norm_sigmas(const double *corr, int level0, double ims, double *sig) {
    double full[6][6];
    int k = 0;
    for (int a = 0; a < 6; a++)
        for (int b = a; b < 6; b++) full[a][b] = full[b][a] = corr[k++];
    double in[3][3];
    for (int a = 0; a < 3; a++)
        for (int b = 0; b < 3; b++) in[a][b] = full[a][b];
    double sx = min_eig_sqrt(in);
    for (int a = 0; a < 3; a++)
        for (int b = 0; b < 3; b++) in[a][b] = full[a + 3][b + 3];
    double sv = min_eig_sqrt(in);
    if (level0) sx *= ims;  // n == num_copies holds for the group itself only
    sig[0] = sx;
    sig[1] = sv;
}

// Nodes up to RSG_SEQ_MAX particles: one thread, array order, so every FP64
// sum rounds as the reference's loop does.
__global__ void k_norm_seq(Rec *W, HierNodes N, int32_t base, int32_t count, int level0,
                           double ims, double *sig) {
    int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= count) return;
    int node = base + k;
    int s = N.start[node], n = N.n[node];
    if (n <= 0 || n > RSG_SMALL) return;
    double mean[6] = {0, 0, 0, 0, 0, 0};
    for (int i = 0; i < n; i++)
        for (int d = 0; d < 6; d++) mean[d] += (double)W[s + i].pos[d];
    for (int d = 0; d < 6; d++) mean[d] /= (double)n;
    double c[21];
    for (int j = 0; j < 21; j++) c[j] = 0;
    for (int i = 0; i < n; i++) {
        float q[6];
        for (int d = 0; d < 6; d++) {
            q[d] = __double2float_rn((double)W[s + i].pos[d] - mean[d]);
            W[s + i].pos[d] = q[d];
        }
        int j = 0;
        for (int x = 0; x < 6; x++)
            for (int y = x; y < 6; y++) c[j++] += (double)fmul(q[x], q[y]);
    }
    for (int j = 0; j < 21; j++) c[j] /= (double)n;
    norm_sigmas(c, level0, ims, sig + 2 * k);
}

// Batched form, nodes up to RSG_SMALL particles: 32 nodes per warp.  For
// each node in turn the lanes stride over its particles: the means and the
// centred coordinates float((double)x - mean) in FP64, as the reference
// forms them (a double-float mean or centring moved coordinates by an ulp
// measurably more often), and the 21 second moments of the float products as
// float pairs on the FP32 pipe (hi + lo, Knuth's two-sum: about 48 bits,
// enough for RSG_SMALL terms); the lanes' sums are combined by shuffles
// (deterministic).  Then the 32 nodes' sigmas (two 3x3 eigenvalue
// problems each, in FP64) run side by side, one node per lane, instead of on
// lane 0 of a warp per node.
#define RSG_NORM_WARPS 4
__global__ void __launch_bounds__(RSG_NORM_WARPS * 32)
    k_norm_warp(Rec *W, HierNodes N, int32_t base, int32_t count, int level0, double ims,
                double *sig) {
    __shared__ double cs[RSG_NORM_WARPS][32][21];
    const unsigned FULL = 0xffffffffu;
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int32_t k0 = ((blockIdx.x * blockDim.x + threadIdx.x) >> 5) * 32;
    if (k0 >= count) return;
    for (int q = 0; q < 32; q++) {
        const int32_t k = k0 + q;
        if (k >= count) break;
        const int node = base + k;
        const int s = N.start[node], n = N.n[node];
        if (n <= 0 || n > RSG_SMALL) continue;
        double acc[6] = {0, 0, 0, 0, 0, 0};
        for (int i = lane; i < n; i += 32)
#pragma unroll
            for (int d = 0; d < 6; d++) acc[d] += (double)W[s + i].pos[d];
        double mean[6];
#pragma unroll
        for (int d = 0; d < 6; d++) {
            for (int o = 16; o; o >>= 1) acc[d] += __shfl_xor_sync(FULL, acc[d], o);
            mean[d] = acc[d] / (double)n;
        }
        float ch[21], cl[21];
        for (int jj = 0; jj < 21; jj++) ch[jj] = cl[jj] = 0.f;
        for (int i = lane; i < n; i += 32) {
            float qv[6];
#pragma unroll
            for (int d = 0; d < 6; d++) {
                qv[d] = __double2float_rn((double)W[s + i].pos[d] - mean[d]);
                W[s + i].pos[d] = qv[d];
            }
            int jj = 0;
            for (int x = 0; x < 6; x++)
                for (int y = x; y < 6; y++, jj++) two_sum_acc(ch[jj], cl[jj], fmul(qv[x], qv[y]));
        }
        for (int jj = 0; jj < 21; jj++) {
            for (int o = 16; o; o >>= 1) {
                float h2 = __shfl_xor_sync(FULL, ch[jj], o);
                float l2 = __shfl_xor_sync(FULL, cl[jj], o);
                two_sum_acc(ch[jj], cl[jj], h2);
                cl[jj] = fadd(cl[jj], l2);
            }
        }
        if (lane < 21) {
            double v = 0;
            for (int jj = 0; jj < 21; jj++)
                if (jj == lane) v = ((double)ch[jj] + (double)cl[jj]) / (double)n;
            cs[w][q][lane] = v;
        }
    }
    __syncwarp();
    const int32_t k = k0 + lane;
    if (k < count) {
        const int n = N.n[base + k];
        if (n > 0 && n <= RSG_SMALL) norm_sigmas(cs[w][lane], level0, ims, sig + 2 * k);
    }
}

// Mid-size nodes: the block stages particles in shared memory and computes
// the per-particle products; thread 0 adds them in array order.
__global__ void __launch_bounds__(256) k_norm_blk(Rec *W, HierNodes N, int32_t base, int level0,
                                                  double ims, double *sig, int lo, int hi) {
    __shared__ float q[256][6];
    __shared__ float pr[256][21];
    __shared__ double mean[6], corr[21];
    int k = blockIdx.x;
    int node = base + k;
    int s = N.start[node], n = N.n[node];
    if (n <= lo || n > hi) return;
    // lane d of warp 0 owns the running sum of coordinate d
    double a = 0;
    for (int b0 = 0; b0 < n; b0 += 256) {
        int i = b0 + threadIdx.x;
        if (i < n)
            for (int d = 0; d < 6; d++) q[threadIdx.x][d] = W[s + i].pos[d];
        __syncthreads();
        if (threadIdx.x < 6) {
            int m = min(256, n - b0), d = threadIdx.x;
            for (int t = 0; t < m; t++) a += (double)q[t][d];
        }
        __syncthreads();
    }
    if (threadIdx.x < 6) mean[threadIdx.x] = a / (double)n;
    __syncthreads();
    double c = 0;  // lane j of warp 0 owns second moment j
    for (int b0 = 0; b0 < n; b0 += 256) {
        int i = b0 + threadIdx.x;
        if (i < n) {
            float v[6];
            for (int d = 0; d < 6; d++) {
                v[d] = __double2float_rn((double)W[s + i].pos[d] - mean[d]);
                W[s + i].pos[d] = v[d];
            }
            int j = 0;
            for (int x = 0; x < 6; x++)
                for (int y = x; y < 6; y++) pr[threadIdx.x][j++] = fmul(v[x], v[y]);
        }
        __syncthreads();
        if (threadIdx.x < 21) {
            int m = min(256, n - b0), j = threadIdx.x;
            for (int t = 0; t < m; t++) c += (double)pr[t][j];
        }
        __syncthreads();
    }
    if (threadIdx.x < 21) corr[threadIdx.x] = c / (double)n;
    __syncthreads();
    if (threadIdx.x == 0) norm_sigmas(corr, level0, ims, sig + 2 * k);
}

// Batched form, nodes above RSG_SMALL particles: cut into chunks of
// Tuning::norm_chunk records, one block per chunk; per-chunk partial sums
// are added per node in chunk order (deterministic).
struct NChunk {
    int32_t node, start, n, pad;  // node: level-local index
};
struct NPart {
    double d[21];
};
__global__ void k_nch_count(HierNodes N, int32_t base, int32_t cnt, int chunk, int seq_lo,
                            int seq_hi, int32_t *nch) {
    int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k > cnt) return;
    int n = (k < cnt) ? N.n[base + k] : 0;
    bool seq = n > seq_lo && n <= seq_hi;  // summed in order by k_norm_blk instead
    nch[k] = (n > RSG_SMALL && !seq) ? (n + chunk - 1) / chunk : 0;
}
__global__ void k_nch_fill(HierNodes N, int32_t base, int32_t cnt, int chunk, const int32_t *nch,
                           const int32_t *c0, NChunk *C) {
    int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= cnt) return;
    int s = N.start[base + k], n = N.n[base + k];
    for (int c = 0; c < nch[k]; c++) {
        NChunk x;
        x.node = k;
        x.start = s + c * chunk;
        x.n = min(chunk, n - c * chunk);
        x.pad = 0;
        C[c0[k] + c] = x;
    }
}
__global__ void __launch_bounds__(256) k_nch_sum6(const Rec *W, const NChunk *C, NPart *P) {
    __shared__ double sm[40];
    NChunk c = C[blockIdx.x];
    double a[6] = {0, 0, 0, 0, 0, 0};
    for (int i = threadIdx.x; i < c.n; i += blockDim.x)
        for (int d = 0; d < 6; d++) a[d] += (double)W[c.start + i].pos[d];
    for (int d = 0; d < 6; d++) {
        double t = block_sum_d(a[d], sm);
        if (threadIdx.x == 0) P[blockIdx.x].d[d] = t;
    }
}
__global__ void k_nch_mean(HierNodes N, int32_t base, int32_t cnt, const int32_t *nch,
                           const int32_t *c0, const NPart *P, double *mean) {
    int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= cnt || nch[k] == 0) return;
    double a[6] = {0, 0, 0, 0, 0, 0};
    for (int c = c0[k]; c < c0[k] + nch[k]; c++)
        for (int d = 0; d < 6; d++) a[d] += P[c].d[d];
    for (int d = 0; d < 6; d++) mean[6 * k + d] = a[d] / (double)N.n[base + k];
}
__global__ void __launch_bounds__(256) k_nch_mom(Rec *W, const NChunk *C, const double *mean,
                                                 NPart *P) {
    __shared__ double sm[40];
    NChunk c = C[blockIdx.x];
    double mu[6];
    for (int d = 0; d < 6; d++) mu[d] = mean[6 * c.node + d];
    double cc[21];
    for (int j = 0; j < 21; j++) cc[j] = 0;
    for (int i = threadIdx.x; i < c.n; i += blockDim.x) {
        float q[6];
        for (int d = 0; d < 6; d++) {
            q[d] = __double2float_rn((double)W[c.start + i].pos[d] - mu[d]);
            W[c.start + i].pos[d] = q[d];
        }
        int j = 0;
        for (int x = 0; x < 6; x++)
            for (int y = x; y < 6; y++) cc[j++] += (double)fmul(q[x], q[y]);
    }
    for (int j = 0; j < 21; j++) {
        double t = block_sum_d(cc[j], sm);
        if (threadIdx.x == 0) P[blockIdx.x].d[j] = t;
    }
}
__global__ void k_nch_fin(HierNodes N, int32_t base, int32_t cnt, const int32_t *nch,
                          const int32_t *c0, const NPart *P, int level0, double ims,
                          double *sig) {
    int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= cnt || nch[k] == 0) return;
    double cc[21];
    for (int j = 0; j < 21; j++) cc[j] = 0;
    for (int c = c0[k]; c < c0[k] + nch[k]; c++)
        for (int j = 0; j < 21; j++) cc[j] += P[c].d[j];
    for (int j = 0; j < 21; j++) cc[j] /= (double)N.n[base + k];
    norm_sigmas(cc, level0, ims, sig + 2 * k);
}

// Larger nodes: one block, deterministic tree reductions.
__global__ void k_norm_par(Rec *W, HierNodes N, int32_t base, int level0, double ims,
                           double *sig, int seq_max) {
    __shared__ double sm[40];
    __shared__ double mean[6], corr[21];
    int k = blockIdx.x;
    int node = base + k;
    int s = N.start[node], n = N.n[node];
    if (n <= seq_max) return;
    double acc[6] = {0, 0, 0, 0, 0, 0};
    for (int i = threadIdx.x; i < n; i += blockDim.x)
        for (int d = 0; d < 6; d++) acc[d] += (double)W[s + i].pos[d];
    for (int d = 0; d < 6; d++) {
        double t = block_sum_d(acc[d], sm);
        if (threadIdx.x == 0) mean[d] = t / (double)n;
    }
    __syncthreads();
    double cc[21];
    for (int j = 0; j < 21; j++) cc[j] = 0;
    for (int i = threadIdx.x; i < n; i += blockDim.x) {
        float q[6];
        for (int d = 0; d < 6; d++) {
            q[d] = __double2float_rn((double)W[s + i].pos[d] - mean[d]);
            W[s + i].pos[d] = q[d];
        }
        int j = 0;
        for (int x = 0; x < 6; x++)
            for (int y = x; y < 6; y++) cc[j++] += (double)fmul(q[x], q[y]);
    }
    for (int j = 0; j < 21; j++) {
        double t = block_sum_d(cc[j], sm);
        if (threadIdx.x == 0) corr[j] = t / (double)n;
    }
    __syncthreads();
    if (threadIdx.x == 0) norm_sigmas(corr, level0, ims, sig + 2 * k);
}

// Divide by the dispersions unless one of them is zero (src/groupies.c:825-829),
// one thread per record.
__global__ void k_norm_div_el(Rec *W, int64_t M, const int32_t *eln, const double *sig) {
    int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= M) return;
    int k = eln[i];
    if (k < 0) return;
    double sx = sig[2 * k], sv = sig[2 * k + 1];
    if (!sx || !sv) return;
    for (int d = 0; d < 6; d++)
        W[i].pos[d] = __double2float_rn((double)W[i].pos[d] / (d < 3 ? sx : sv));
}

// x advanced by m steps of rand_r's generator (x <- 1103515245 x + 12345
// mod 2^32), by squaring the affine step.
__device__ __forceinline__ unsigned lcg_jump(unsigned x, uint64_t m) {
    unsigned a = 1103515245u, c = 12345u, ra = 1u, rc = 0u;
    while (m) {
        if (m & 1) {
            ra = a * ra;
            rc = a * rc + c;
        }
        c = a * c + c;
        a = a * a;
        m >>= 1;
    }
    return ra * x + rc;
}

// Sample list (src/groupies.c:295-308): all particles when n <= 10000
// (or EXACT_LL_CALC), else 10000 indices drawn by two rand_r calls each
// from a stream seeded with n.  A rand_r call is three generator steps, so
// sample t starts from the seed advanced by 6 t steps: every sample is
// drawn on its own thread.  The node's stream continues into
// find_median_r from the state after all its samples.
__global__ void k_sample_seed(HierNodes N, int32_t base, int32_t count, unsigned *seed_out,
                              int exact) {
    int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= count) return;
    int n = N.n[base + k];
    int nt = exact ? n : (n < 10000 ? n : 10000);
    seed_out[k] = (nt != n) ? lcg_jump((unsigned)n, 6ull * (uint64_t)nt) : (unsigned)n;
}
__global__ void k_sample_idx(HierNodes N, int32_t base, int32_t count, const int32_t *soff,
                             int32_t *sidx, int64_t total, int exact) {
    int64_t g = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (g >= total) return;
    int lo = 0, hi = count - 1;  // node of sample g: last k with soff[k] <= g
    while (lo < hi) {
        int mid = (lo + hi + 1) >> 1;
        if (soff[mid] <= g) lo = mid;
        else hi = mid - 1;
    }
    int n = N.n[base + lo];
    int nt = exact ? n : (n < 10000 ? n : 10000);
    if (nt == n) return;
    int64_t t = g - soff[lo];
    unsigned seed = lcg_jump((unsigned)n, 6ull * (uint64_t)t);
    int64_t j = rand_r_glibc(&seed);
    j <<= 31;
    j += rand_r_glibc(&seed);
    j %= n;
    sidx[g] = (int32_t)j;
}

// The squared 6D distance of the reference's searches: dx = c[j] - p[j],
// d += dx * dx for j = 0..5 in order, each operation rounded to float
// (src/fast3tree.c:401-405 with FAST3TREE_DIM 6).
// dist6_p computes it with the subtractions and squares done two dimensions
// per instruction (Blackwell's packed FP32 arithmetic, each lane rounded as
// the scalar operation): c2 and q2 hold coordinates (0,1), (2,3), (4,5) as
// float pairs, the lower-addressed coordinate in the low half.  The sum runs
// over j = 0..5 in order as in dist6, so the result is the same float.
__device__ __forceinline__ float dist6_p(const unsigned long long *c2, const unsigned long long *q2) {
    float p0, p1, p2, p3, p4, p5;
    f2_split(f2_sqr(f2_sub(c2[0], q2[0])), p0, p1);
    f2_split(f2_sqr(f2_sub(c2[1], q2[1])), p2, p3);
    f2_split(f2_sqr(f2_sub(c2[2], q2[2])), p4, p5);
    float d = fadd(0.f, p0);
    d = fadd(d, p1);
    d = fadd(d, p2);
    d = fadd(d, p3);
    d = fadd(d, p4);
    return fadd(d, p5);
}
// A record's coordinates as three float pairs (two 16-byte loads).
__device__ __forceinline__ void rec_pairs(const Rec *w, unsigned long long *q2) {
    const ulonglong2 a = reinterpret_cast<const ulonglong2 *>(w)[0];
    const ulonglong2 b = reinterpret_cast<const ulonglong2 *>(w)[1];
    q2[0] = a.x;
    q2[1] = a.y;
    q2[2] = b.x;
}
__device__ __forceinline__ bool box_out6(const KNode<6> &nd, const float *c, float r) {
    float d = 0.f, e;
    const float r2 = fmul(r, r);
#pragma unroll
    for (int i = 0; i < 6; i++) {
        if ((e = fsub(c[i], nd.mn[i])) < 0) {
            d = fadd(d, fmul(e, e));
            if (d >= r2) return true;
        } else if ((e = fsub(c[i], nd.mx[i])) > 0) {
            d = fadd(d, fmul(e, e));
            if (d >= r2) return true;
        }
    }
    return false;
}

// fast3tree_find_next_closest_distance (src/fast3tree.c:956-1030), with the
// recursion unrolled onto an explicit stack; the running radius threads
// through the visits in the reference's order.
__device__ float next_closest(const KNode<6> *nodes, int root, const Rec *W, const float *c,
                              bool valid, int *err) {
    const unsigned FULL = 0xffffffffu;
    int nd = root;
    float r = 0.f;
    int stack[RSG_STACK6];
    int sp = 0;
    if (valid) {
        while (nodes[nd].div >= 0) {
            const KNode<6> &x = nodes[nd];
            nd = (c[x.div] <= nodes[x.left].mx[x.div]) ? x.left : x.left + 1;
        }
        while (nd != root) {
            int pdv = nodes[nodes[nd].parent].div;
            if (nodes[nd].mn[pdv] == nodes[nd].mx[pdv]) nd = nodes[nd].parent;
            else break;
        }
        const KNode<6> &o = nodes[nd];
        float md = 0.f;
        for (int j = 0; j < 6; j++) {
            float dx = fsub(o.mx[j], o.mn[j]);
            md = fadd(md, fmul(dx, dx));
        }
        const unsigned long long c2[3] = {f2_pack(c[0], c[1]), f2_pack(c[2], c[3]),
                                          f2_pack(c[4], c[5])};
        for (int i = 0; i < o.n; i++) {
            unsigned long long q2[3];
            rec_pairs(W + o.start + i, q2);
            float d = dist6_p(c2, q2);
            if (d && d < md) md = d;
        }
        r = sqrt_fd(md);
        stack[sp++] = root;
    }
    // Each lane walks its own depth-first order (the reference's, with its
    // own pruning radius) until it reaches its next leaf; then the lanes
    // holding a leaf test their leaves together.  A lane's sequence of node
    // tests and leaf updates is unchanged; only its interleaving with the
    // other lanes is.
    while (__any_sync(FULL, sp > 0)) {
        int leaf = -1;
        while (sp) {
            const int ni = stack[--sp];
            const KNode<6> &x = nodes[ni];
            if (box_out6(x, c, r) || ni == nd) continue;
            if (x.div < 0) {
                leaf = ni;
                break;
            }
            int a = x.left, b = x.left + 1;
            if (c[x.div] > fmul(0.5f, fadd(x.mn[x.div], x.mx[x.div]))) {
                a = x.left + 1;
                b = x.left;
            }
            if (sp + 2 > RSG_STACK6) {
                atomicExch(err, 1);
                sp = 0;
                break;
            }
            stack[sp++] = b;
            stack[sp++] = a;
        }
        if (leaf >= 0) {
            const KNode<6> &x = nodes[leaf];
            const unsigned long long c2[3] = {f2_pack(c[0], c[1]), f2_pack(c[2], c[3]),
                                              f2_pack(c[4], c[5])};
            float r2 = fmul(r, r);
            for (int i = 0; i < x.n; i++) {
                unsigned long long q2[3];
                rec_pairs(W + x.start + i, q2);
                float d = dist6_p(c2, q2);
                if (d < r2) r2 = d;
            }
            r = sqrt_fd(r2);
        }
    }
    return r;
}

// Sample queries in tree order: key (node, position in the node) of every
// sample (random positions for nodes above 10000 particles), so neighbouring
// threads search from neighbouring particles.
__global__ void k_nn_keys(HierNodes N, int32_t base, int32_t count, const int32_t *soff,
                          const int32_t *sidx, int64_t total, int exact, uint64_t *key,
                          uint32_t *val) {
    int64_t g = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (g >= total) return;
    int lo = 0, hi = count - 1;
    while (lo < hi) {
        int mid = (lo + hi + 1) >> 1;
        if (soff[mid] <= g) lo = mid;
        else hi = mid - 1;
    }
    int n = N.n[base + lo];
    int nt = exact ? n : (n < 10000 ? n : 10000);
    int t = (int)(g - soff[lo]);
    int j = (nt == n) ? t : sidx[g];
    key[g] = ((uint64_t)(uint32_t)lo << 32) | (uint32_t)j;
    val[g] = (uint32_t)g;
}
// The next-closest distance of every sample, queries taken in `order`
// (sample indices; null: as stored), results stored by sample index.
__global__ void k_nn(const KNode<6> *nodes, const Rec *W, HierNodes N, int32_t base,
                     int32_t count, const int32_t *soff, const int32_t *sidx, float *prad,
                     int64_t total, int exact, int *err, const uint32_t *order) {
    int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    // lanes past the end stay (next_closest synchronises the warp)
    const bool valid = q < total;
    if (!valid) q = total - 1;
    int64_t g = order ? (int64_t)order[q] : q;
    // node of sample g: last k with soff[k] <= g
    int lo = 0, hi = count - 1;
    while (lo < hi) {
        int mid = (lo + hi + 1) >> 1;
        if (soff[mid] <= g) lo = mid;
        else hi = mid - 1;
    }
    int k = lo;
    int node = base + k;
    int s = N.start[node], n = N.n[node];
    int nt = exact ? n : (n < 10000 ? n : 10000);
    int t = (int)(g - soff[k]);
    int j = (nt == n) ? t : sidx[soff[k] + t];
    float c[6];
#pragma unroll
    for (int d = 0; d < 6; d++) c[d] = W[s + j].pos[d];
    const float rr = next_closest(nodes, k, W, c, valid, err);
    if (valid) prad[g] = rr;
}

// find_median_r / rad_partition (src/groupies.c:735-786), run as is on the
// sample's distances in sample order with the continuing rand_r stream.
__device__ float median_r(float *a, int nt, unsigned seed, float frac) {
    int64_t kk = (int64_t)__float2ll_rz(fmul(__ll2float_rn(nt), frac));
    if (nt < 2) return a[0];
    int64_t left = 0, right = nt;
    int guard = 0;
    while (true) {
        float u = __fdiv_rn(__int2float_rn(rand_r_glibc(&seed) % 2147483647), 2147483648.0f);
        float pf = fadd(__ll2float_rn(left), fmul(u, __ll2float_rn(right - left)));
        int64_t pi = (int64_t)__float2ll_rz(pf);
        if (pi >= right) pi = right - 1;  // keeps the access in range (u == 1 edge)
        float piv = a[pi], t;
        t = a[pi]; a[pi] = a[right - 1]; a[right - 1] = t;
        int64_t si = right - 2, i;
        for (i = left; i < si; i++)
            if (a[i] > piv) {
                t = a[i]; a[i] = a[si]; a[si] = t;
                si--;
                i--;
            }
        if (a[si] <= piv) si++;
        t = a[right - 1]; a[right - 1] = a[si]; a[si] = t;
        int64_t p = si;
        if (kk == p || (a[left] == a[right - 1])) return a[kk];
        if (kk < p) right = p;
        else left = p + 1;
        if (++guard > 100000000) {  // cannot happen for finite input: report it
            loop_limit_hit();
            return a[kk];
        }
    }
}
// Nodes whose sample fits in shared memory (RSG_TARGET_SMEM distances): one
// block per node runs find_median_r with every rad_partition done by the
// whole block.  rad_partition's loop over [left, right - 1) is the same
// two-pointer swap as the kd-tree split (kdtree.cuh), so each element's
// destination follows in closed form from prefix counts of the elements
// above the pivot; thread 0 draws the pivots from the rand_r stream in the
// reference's order.  The result is the sequential one element for element.
#define RSG_TARGET_SMEM 10000
#define RSG_TGT_T 256
__global__ void __launch_bounds__(RSG_TGT_T) k_target_par(HierNodes N, int32_t base,
                                                          const int32_t *soff, const float *prad,
                                                          const unsigned *seed_in, float frac,
                                                          int exact) {
    extern __shared__ float sm_f[];
    typedef cub::BlockScan<int, RSG_TGT_T> Scan;
    typedef cub::BlockReduce<int, RSG_TGT_T> Red;
    __shared__ union {
        typename Scan::TempStorage s;
        typename Red::TempStorage r;
    } tmp;
    __shared__ int sh_pi, sh_done, sh_q;
    __shared__ float sh_res;
    const int k = blockIdx.x, node = base + k, tid = threadIdx.x;
    const int n = N.n[node];
    const int nt = exact ? n : (n < 10000 ? n : 10000);
    if (nt > RSG_TARGET_SMEM || nt < 1) return;
    float *a = sm_f, *b = sm_f + nt;
    int *fb = (int *)(sm_f + 2 * nt), *bs = fb + nt;
    const float *src = prad + soff[k];
    for (int i = tid; i < nt; i += RSG_TGT_T) a[i] = src[i];
    const int kk = (int)__float2ll_rz(fmul(__ll2float_rn(nt), frac));
    if (nt < 2) {
        if (tid == 0) N.target_r[node] = a[0];
        return;
    }
    unsigned seed = seed_in[k];
    int left = 0, right = nt;
    __syncthreads();
    for (int guard = 0;; guard++) {
        if (tid == 0) {
            float u = __fdiv_rn(__int2float_rn(rand_r_glibc(&seed) % 2147483647), 2147483648.0f);
            float pf = fadd(__int2float_rn(left), fmul(u, __int2float_rn(right - left)));
            int pi = (int)__float2ll_rz(pf);
            if (pi >= right) pi = right - 1;
            float t = a[pi];
            a[pi] = a[right - 1];
            a[right - 1] = t;
            sh_pi = pi;
        }
        __syncthreads();
        const float piv = a[right - 1];
        const int L = right - 1 - left;  // the swap loop runs over [left, right - 1)
        int m;
        if (L == 0) {
            // one element: the reference compares a[left - 1] (left >= 1 here,
            // since kk >= 1) and may swap it in; done as written
            m = 0;
            if (tid == 0) {
                int si = left - 1;
                if (a[si] <= piv) si++;
                float t = a[right - 1];
                a[right - 1] = a[si];
                a[si] = t;
                sh_q = si;
            }
            __syncthreads();
        } else {
            const int per = (L + RSG_TGT_T - 1) / RSG_TGT_T;
            const int c0 = min(L, tid * per), c1 = min(L, c0 + per);
            int cnt = 0;
            for (int l = c0; l < c1; l++) cnt += a[left + l] > piv;
            int before, B;
            Scan(tmp.s).ExclusiveSum(cnt, before, B);
            __syncthreads();
            m = L - B;  // elements <= pivot
            int br = before, qb = 0;
            for (int l = c0; l < c1; l++) {
                bool big = a[left + l] > piv;
                int sr = l - br;
                if (big && l < m) fb[br] = l;
                if (!big && l >= m) bs[m - 1 - sr] = l;
                if (big && l < m) qb++;
                br += big;
            }
            int q = Red(tmp.r).Sum(qb);
            if (tid == 0) sh_q = q;
            __syncthreads();
            q = sh_q;
            br = before;
            for (int l = c0; l < c1; l++) {
                float v = a[left + l];
                bool big = v > piv;
                int sr = l - br, d;
                if (!big && l < m) d = l;
                else if (big && l < m) d = (br == 0) ? L - 1 : bs[br - 1] - 1;
                else if (!big) d = fb[m - 1 - sr];
                else {
                    int pos_last = (q > 0) ? bs[q - 1] : L;
                    if (l > pos_last) d = l - 1;
                    else if (pos_last - m >= 2) d = (l == m) ? pos_last - 1 : l - 1;
                    else d = l;
                }
                b[d] = v;
                br += big;
            }
            __syncthreads();
            for (int l = tid; l < L; l += RSG_TGT_T) a[left + l] = b[l];
            __syncthreads();
            if (tid == 0) {
                int si = left + m;
                float t = a[right - 1];
                a[right - 1] = a[si];
                a[si] = t;
                sh_q = si;
            }
            __syncthreads();
        }
        const int p = sh_q;
        if (tid == 0) {
            sh_done = (kk == p || a[left] == a[right - 1]);
            if (sh_done) sh_res = a[kk];
            if (guard > 100000000) {  // cannot happen for finite input: report it
                loop_limit_hit();
                sh_done = 1;
                sh_res = a[kk];
            }
        }
        __syncthreads();
        if (sh_done) break;
        if (kk < p) right = p;
        else left = p + 1;
    }
    if (tid == 0) N.target_r[node] = sh_res;
}
// Larger samples (EXACT_LL_CALC): in place in global memory.
__global__ void k_target(HierNodes N, int32_t base, int32_t count, const int32_t *soff,
                         float *prad, const unsigned *seed_in, float frac, int exact) {
    int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= count) return;
    int node = base + k;
    int n = N.n[node];
    int nt = exact ? n : (n < 10000 ? n : 10000);
    if (nt <= RSG_TARGET_SMEM) return;
    N.target_r[node] = median_r(prad + soff[k], nt, seed_in[k], frac);
}

// element -> level-local node index for the nodes [base, base + count)
__global__ void k_fill_eln(HierNodes N, int32_t base, int32_t *eln) {
    int k = blockIdx.x;
    int s = N.start[base + k], n = N.n[base + k];
    for (int i = threadIdx.x; i < n; i += blockDim.x) eln[s + i] = k;
}

// _find_subfofs_at_r (src/groupies.c:274-284): every particle links to
// itself and to the later particles within target_r (6D, strict <), which
// the skip search returns in ascending order.
// The search runs for 32 consecutive particles at a time: the warp walks
// each node's tree once with a shared stack, entering a node when any
// lane's own box test admits it; at a leaf every lane tests
// every point with its own distance test.  A lane meets exactly the points
// of its own search, in ascending order.  MODE 2 counts every list, keeps
// its first RSG_SLOT6 entries in a fixed slot per particle and the rest in
// chunks of RSG_SLOT6 entries taken from a pool and chained per particle
// (Chains); a particle whose chunk the pool could not give is flagged
// (Chains::redo) and MODE 1 fills its CSR list with a second search.
#define RSG_SLOT6 32
struct Chains {
    int32_t *pool;     // cap chunks of RSG_SLOT6 entries
    int32_t *next;     // next chunk of a chain, -1 at the end
    int32_t *head;     // first chunk of a particle's chain, -1 for none
    int32_t *redo;     // 1: the list did not fit (MODE 1 refills it)
    unsigned *cursor;  // chunks taken
    int32_t cap;
};
template <int MODE>
__global__ void __launch_bounds__(128, 16) k_fof6_w(const KNode<6> *nodes, const Rec *W, int64_t M,
                                                HierNodes N, int32_t base, const int32_t *eln,
                                                const int32_t *noff, int32_t *ncnt, int32_t *nbr,
                                                Chains CH, int *err, unsigned long long *near) {
    const unsigned FULL = 0xffffffffu;
    int64_t w0 = ((blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5) * 32;
    int lane = threadIdx.x & 31;
    if (w0 >= M) return;
    int i = (int)(w0 + lane);
    bool valid = w0 + lane < M;
    int k = valid ? eln[i] : -1;
    float c[6];
#pragma unroll
    for (int d = 0; d < 6; d++) c[d] = (valid && k >= 0) ? W[i].pos[d] : 0.f;
    const unsigned long long c2[3] = {f2_pack(c[0], c[1]), f2_pack(c[2], c[3]),
                                      f2_pack(c[4], c[5])};
    int cnt = 0;
    bool part = valid && k >= 0 && (MODE != 1 || CH.redo[i]);
    int o = (MODE == 1 && part) ? noff[i] : 0;
    int32_t *slot = (MODE == 2) ? nbr + (int64_t)i * RSG_SLOT6 : nullptr;
    int chunk = -1;     // MODE 2: the chunk being filled
    bool lost = false;  // MODE 2: the pool ran out for this list
    unsigned pending = __ballot_sync(FULL, part);
    int stack[RSG_STACK6];
    while (pending) {
        int leader = __ffs(pending) - 1;
        int kk = __shfl_sync(FULL, k, leader);
        bool mine = part && k == kk;
        pending &= ~__ballot_sync(FULL, mine);
        int imin = (int)w0 + leader;  // the segment's first particle
        float r = N.target_r[base + kk];
        const float r2 = fmul(r, r);
        int sp = 0;
        stack[sp++] = kk;
        while (sp) {
            const KNode<6> &x = nodes[stack[--sp]];
            if (x.start + x.n <= imin + 1) continue;
            bool need = mine && (x.start + x.n > i + 1) && !box_out6(x, c, r);
            if (!__ballot_sync(FULL, need)) continue;
            if (x.div < 0) {
                int j0 = x.start > imin + 1 ? x.start : imin + 1;
                for (int j = j0; j < x.start + x.n; j++) {
                    // the record as two 16-byte loads (the same address in
                    // every lane: one broadcast transaction each)
                    unsigned long long q2[3];
                    rec_pairs(W + j, q2);
                    float d = dist6_p(c2, q2);
                    if (need && j > i && d < r2) {
                        if (MODE == 1) nbr[o + cnt] = j;
                        if (MODE == 2) {
                            if (cnt < RSG_SLOT6) {
                                slot[cnt] = j;
                            } else if (!lost) {
                                const int e = (cnt - RSG_SLOT6) % RSG_SLOT6;
                                if (e == 0) {
                                    cg::coalesced_group g = cg::coalesced_threads();
                                    unsigned b = 0;
                                    if (g.thread_rank() == 0) b = atomicAdd(CH.cursor, g.size());
                                    const unsigned c2 = g.shfl(b, 0) + g.thread_rank();
                                    if (c2 < (unsigned)CH.cap) {
                                        CH.next[c2] = -1;
                                        if (chunk < 0) CH.head[i] = (int32_t)c2;
                                        else CH.next[chunk] = (int32_t)c2;
                                        chunk = (int32_t)c2;
                                    } else {
                                        lost = true;
                                    }
                                }
                                if (!lost) CH.pool[(int64_t)chunk * RSG_SLOT6 + e] = j;
                            }
                        }
                        cnt++;
                    }
                    // pairs within 1e-6 of the linking length (relative, in
                    // distance): where a last-bit change of a coordinate
                    // could decide the link
                    if (MODE == 2 && need && j > i && fabsf(d - r2) <= 2e-6f * r2)
                        atomicAdd(near, 1ull);
                }
                continue;
            }
            if (sp + 2 > RSG_STACK6) {
                if (lane == 0) atomicExch(err, 1);
                return;
            }
            stack[sp++] = x.left + 1;
            stack[sp++] = x.left;
        }
    }
    if (MODE == 2 && part) {
        ncnt[i] = cnt;
        CH.redo[i] = lost;
    }
}
// CSR lists from the fixed slots of the lists that fit in them.
__global__ void k_slots_csr(const int32_t *eln, int64_t M, const int32_t *ncnt,
                            const int32_t *noff, const int32_t *slots, Chains CH, int32_t *nbr) {
    int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= M || eln[i] < 0 || CH.redo[i]) return;
    const int n = ncnt[i];
    const int32_t *sl = slots + i * RSG_SLOT6;
    int32_t *dst = nbr + noff[i];
    const int ns = n < RSG_SLOT6 ? n : RSG_SLOT6;
    for (int t = 0; t < ns; t++) dst[t] = sl[t];
    int c = n > RSG_SLOT6 ? CH.head[i] : -1;
    for (int t = RSG_SLOT6; t < n; t += RSG_SLOT6) {
        const int32_t *src = CH.pool + (int64_t)c * RSG_SLOT6;
        const int m = (n - t) < RSG_SLOT6 ? (n - t) : RSG_SLOT6;
        for (int u = 0; u < m; u++) dst[t + u] = src[u];
        c = CH.next[c];
    }
}

template <class T>
__global__ void k_gather(const T *src, const uint32_t *perm, int64_t M, T *dst) {
    int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i < M) dst[i] = src[perm[i]];
}

// Runs of equal labels after the partition sort: the kept ones (>= 0 and at
// least MIN_HALO_PARTICLES long) are the subgroups of build_fullfofs
// (src/fof.c:226-255), in array order.
__global__ void k_run_heads(const int32_t *eln, int64_t M, HierNodes N, int32_t base,
                            const int32_t *lab, int32_t *flag) {
    int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= M) return;
    int k = eln[i];
    int f = 0;
    if (k >= 0) {
        int s = N.start[base + k];
        f = (i == s) || lab[i] != lab[i - 1];
    }
    flag[i] = f;
}
__global__ void k_run_children(const int32_t *heads, int32_t nh, const int32_t *eln,
                               HierNodes N, int32_t base, const int32_t *lab, int64_t minsz,
                               int32_t *cflag, int32_t *clen) {
    int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= nh) return;
    int p = heads[t];
    int k = eln[p];
    int node = base + k;
    int end = N.start[node] + N.n[node];
    if (t + 1 < nh && heads[t + 1] < end) end = heads[t + 1];
    int len = end - p;
    clen[t] = len;
    cflag[t] = lab[p] >= 0 && len >= minsz && len > minsz && len < N.n[node];
}
__global__ void k_make_children2(const int32_t *cidx, int32_t nc, const int32_t *heads,
                                 const int32_t *clen, const int32_t *eln, HierNodes N,
                                 int32_t base, int32_t nbase) {
    int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= nc) return;
    int h = cidx[t];
    int p = heads[h];
    int par = base + eln[p];
    int c = nbase + t;
    N.start[c] = p;
    N.n[c] = clen[h];
    N.parent[c] = par;
    N.group[c] = N.group[par];
    N.level[c] = N.level[par] + 1;
    N.nchild[c] = 0;
    atomicAdd(&N.nchild[par], 1);
}

// ---- halos -----------------------------------------------------------------

__global__ void k_leaf_flags(HierNodes N, int32_t nn, int32_t *flag) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < nn) flag[i] = N.nchild[i] == 0;
}
__global__ void k_leaf_keys(HierNodes N, const int32_t *leaves, int32_t nl, int32_t *key) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < nl) key[i] = N.start[leaves[i]];
}
__device__ int lower_bound_i(const int32_t *a, int n, int v) {
    int lo = 0, hi = n;
    while (lo < hi) {
        int mid = (lo + hi) >> 1;
        if (a[mid] < v) lo = mid + 1;
        else hi = mid;
    }
    return lo;
}
__global__ void k_halo_ranges(HierNodes N, int32_t nn, const int32_t *lstart, int32_t nl) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nn) return;
    N.h0[i] = lower_bound_i(lstart, nl, N.start[i]);
    N.h1[i] = lower_bound_i(lstart, nl, N.start[i] + N.n[i]);
}
// add_new_halo (src/groupies.c:164-187)
__global__ void k_halo_init(rsg_halo *H, rsg_extra_halo_info *E, int32_t nh) {
    int h = blockIdx.x * blockDim.x + threadIdx.x;
    if (h >= nh) return;
    rsg_halo z;
    memset(&z, 0, sizeof(z));
    z.flags = RSG_GROWING;
    H[h] = z;
    E[h].child = E[h].next_cochild = E[h].ph = E[h].prev_cochild = E[h].sub_of = -1;
    E[h].max_metric = 0;
}

// src/groupies.c:542-551: particle -> halo from the children's halos, and
// real coordinates restored from the caller's particles.  The restore runs
// one thread per particle of the level; the marks one warp per halo (block
// (k, y) takes every gridDim.y-th group of warps of node k's halos).  The
// reference's loop over the halos in index order leaves a particle listed by
// several halos with the largest index, which atomicMax gives in any order.
__global__ void k_asc_restore(Rec *W, const rsg_particle *P, const int32_t *eln, int64_t M,
                              int32_t *phalo) {
    int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= M || eln[i] < 0) return;
    phalo[i] = -1;
    const rsg_particle &q = P[W[i].ridx];
#pragma unroll
    for (int d = 0; d < 6; d++) W[i].pos[d] = q.pos[d];
}
__global__ void k_asc_halo_mark(HierNodes N, int32_t base, const rsg_halo *H, int32_t *phalo) {
    int node = base + blockIdx.x;
    int h0 = N.h0[node], h1 = N.h1[node];
    const int wpb = blockDim.x >> 5, w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    for (int h = h0 + blockIdx.y * wpb + w; h < h1; h += gridDim.y * wpb) {
        int ps = (int)H[h].p_start, np = (int)H[h].num_p;
        for (int j = lane; j < np; j += 32) atomicMax(&phalo[ps + j], h);
    }
}

// _find_biggest_parent without temporal information (src/groupies.c:362-380)
// is a running strict maximum of (vmax, num_p) from a start halo: the first
// index holding the largest pair, except that a NaN vmax never replaces and
// a NaN at the start is never replaced.  big_gt: candidate a beats b.
__device__ __forceinline__ bool big_gt(const rsg_halo &a, const rsg_halo &b) {
    return a.vmax > b.vmax || (a.vmax == b.vmax && a.num_p > b.num_p);
}
// That choice over halos h0..h1 (growing ones only, starting from `first`,
// or all, starting from h0) as a block reduction (blockDim 256).
__device__ int biggest_blk(const rsg_halo *H, int h0, int h1, int growing_only, int first) {
    __shared__ int red[256];
    int start = growing_only ? first : h0;
    int loc = -1;
    for (int i = h0 + threadIdx.x; i < h1; i += blockDim.x) {
        if (growing_only && !(H[i].flags & RSG_GROWING)) continue;
        if (H[i].vmax != H[i].vmax) continue;
        if (loc < 0 || big_gt(H[i], H[loc])) loc = i;
    }
    red[threadIdx.x] = loc;
    __syncthreads();
    for (int o = blockDim.x >> 1; o; o >>= 1) {
        if (threadIdx.x < o) {
            int a = red[threadIdx.x], b = red[threadIdx.x + o];
            if (a < 0 || (b >= 0 && (big_gt(H[b], H[a]) || (!big_gt(H[a], H[b]) && b < a))))
                red[threadIdx.x] = b;
        }
        __syncthreads();
    }
    int best = red[0];
    __syncthreads();
    if (best < 0 || H[start].vmax != H[start].vmax) return start;
    return big_gt(H[best], H[start]) ? best : (growing_only ? start : best);
}

// src/groupies.c:553-582: biggest seed, Poisson/force-resolution merges,
// growing list.  One block (256 threads) per node: the merge test of every
// halo against the biggest in parallel, the growing list compacted in index
// order.
__global__ void __launch_bounds__(256) k_asc_seed_blk(HierNodes N, int32_t base, rsg_halo *H,
                                                      rsg_extra_halo_info *E, int32_t *glist,
                                                      int32_t *redirect, double force_res) {
    typedef cub::BlockScan<int, 256> Scan;
    __shared__ typename Scan::TempStorage ts;
    __shared__ int run;
    int node = base + blockIdx.x;
    int h0 = N.h0[node], h1 = N.h1[node];
    int mi = biggest_blk(H, h0, h1, 0, 0);
    if (threadIdx.x == 0) {
        H[mi].flags |= RSG_GROWING;
        E[mi].sub_of = -1;
        glist[h0] = mi;
        run = 1;
    }
    __syncthreads();
    for (int c0 = h0; c0 < h1; c0 += 256) {
        int i = c0 + threadIdx.x, keep = 0;
        if (i < h1) {
            redirect[i] = -1;
            if (i != mi && (H[i].flags & RSG_GROWING)) {
                int force;
                if (poisson_or_force(H[i], H[mi], force_res, &force)) {
                    H[i].flags -= (H[i].flags & RSG_GROWING);
                    E[i].sub_of = mi;
                    if (!force) {
                        redirect[i] = mi;
                        H[i].num_p = 0;
                    }
                } else {
                    keep = 1;
                }
            }
        }
        int at, tot;
        Scan(ts).ExclusiveSum(keep, at, tot);
        if (keep) glist[h0 + run + at] = i;
        __syncthreads();
        if (threadIdx.x == 0) run += tot;
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        N.maxi[node] = mi;
        N.ng[node] = run;
    }
}

// src/groupies.c:584-609: particles of merged seeds go to the biggest halo;
// unassigned particles go to the halo of smallest phase-space metric among
// the growing ones, then up the sub_of chain while the metric exceeds the
// halo's max_metric.  The metric is calc_particle_dist's
// (float)sqrt((double)x) of the float sum x = r^2/h.r^2 + v^2/h.vrms^2,
// which is monotone in x: a candidate whose x is not below the best one's
// cannot win the strict comparison, so the square root is only taken for
// candidates that might (same choice, ties included).
struct AscHalo {
    float pos[6];
    float r, vrms;
};
__device__ __forceinline__ bool asc_valid(const AscHalo &h) { return !(h.vrms <= 0 || h.r <= 0); }
__device__ __forceinline__ float asc_x(const AscHalo &h, const float *pos) {
    float r2 = 0.f, v2 = 0.f;
#pragma unroll
    for (int i = 0; i < 3; i++) {
        float dx = fsub(h.pos[i], pos[i]);
        r2 = fadd(r2, fmul(dx, dx));
    }
#pragma unroll
    for (int i = 3; i < 6; i++) {
        float dx = fsub(h.pos[i], pos[i]);
        v2 = fadd(v2, fmul(dx, dx));
    }
    float a = __fdiv_rn(r2, fmul(h.r, h.r));
    float b = __fdiv_rn(v2, fmul(h.vrms, h.vrms));
    return fadd(a, b);
}
// Buckets of 32 consecutive candidates (k_asc_buckets_s) for nodes with more
// than Tuning::asc_bucket_min (bmin) of them: the box of their centres and the largest
// radius over the valid ones (inv: the bucket holds an invalid halo).  For a
// point, box distance^2 / rmax^2 is at most the float x of every valid halo
// in the bucket (every rounded operation of x is monotone in its inputs).
struct AscBucket {
    float mn[3], mx[3], rmax;
    int32_t inv;  // holds a halo without a valid metric
};
// lower bound of x over a bucket's valid halos
__device__ __forceinline__ float asc_bucket_lb(const AscBucket &B, const float *pos) {
    float d2 = 0.f;
#pragma unroll
    for (int i = 0; i < 3; i++) {
        float gap = 0.f;
        if (pos[i] < B.mn[i]) gap = fsub(B.mn[i], pos[i]);
        else if (pos[i] > B.mx[i]) gap = fsub(pos[i], B.mx[i]);
        d2 = fadd(d2, fmul(gap, gap));
    }
    return __fdiv_rn(d2, fmul(B.rmax, B.rmax));
}
// Nodes with more than bmin growing halos also get their halos in
// Morton order of position (within the node's box of halo centres), so that
// buckets of 32 and 1024 halos are compact in space.  The scan order then
// differs from the list order; the choice stays the list scan's because a
// candidate is taken on (metric, list position) lexicographically: the
// first list position among the smallest metrics, which is what the strict
// sequential comparison keeps.
__device__ __forceinline__ uint32_t morton10(uint32_t v) {
    v &= 1023u;
    v = (v | (v << 16)) & 0x030000FFu;
    v = (v | (v << 8)) & 0x0300F00Fu;
    v = (v | (v << 4)) & 0x030C30C3u;
    v = (v | (v << 2)) & 0x09249249u;
    return v;
}
// all = 0: the node's growing list glist[h0 ..]; all = 1: halos h0 .. h1.
__device__ __forceinline__ int asc_count(const HierNodes &N, int node, int all) {
    return all ? N.h1[node] - N.h0[node] : N.ng[node];
}
__global__ void k_asc_sort_keys(HierNodes N, int32_t base, const rsg_halo *H,
                                const int32_t *glist, int all, int bmin, uint32_t *key,
                                int32_t *val, int32_t *sb, int32_t *se) {
    __shared__ float mn[3], mx[3];
    int k = blockIdx.x, node = base + k;
    int ng = asc_count(N, node, all), h0 = N.h0[node];
    if (threadIdx.x == 0) {
        sb[k] = h0;
        se[k] = ng > bmin ? h0 + ng : h0;
        for (int d = 0; d < 3; d++) {
            mn[d] = INFINITY;
            mx[d] = -INFINITY;
        }
    }
    __syncthreads();
    if (ng <= bmin) return;
    float lmn[3] = {INFINITY, INFINITY, INFINITY}, lmx[3] = {-INFINITY, -INFINITY, -INFINITY};
    for (int g = threadIdx.x; g < ng; g += blockDim.x) {
        const float *p = H[all ? h0 + g : glist[h0 + g]].pos;
        for (int d = 0; d < 3; d++) {
            lmn[d] = fminf(lmn[d], p[d]);
            lmx[d] = fmaxf(lmx[d], p[d]);
        }
    }
    __shared__ float red[6][32];
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    for (int d = 0; d < 3; d++) {
        float a = lmn[d], b = lmx[d];
        for (int o = 16; o; o >>= 1) {
            a = fminf(a, __shfl_xor_sync(0xffffffffu, a, o));
            b = fmaxf(b, __shfl_xor_sync(0xffffffffu, b, o));
        }
        if (lane == 0) {
            red[d][w] = a;
            red[d + 3][w] = b;
        }
    }
    __syncthreads();
    if (threadIdx.x == 0)
        for (int v = 0; v < (int)(blockDim.x >> 5); v++)
            for (int d = 0; d < 3; d++) {
                mn[d] = fminf(mn[d], red[d][v]);
                mx[d] = fmaxf(mx[d], red[d + 3][v]);
            }
    __syncthreads();
    float sc[3];
    for (int d = 0; d < 3; d++) sc[d] = (mx[d] > mn[d]) ? 1023.99f / (mx[d] - mn[d]) : 0.f;
    for (int g = threadIdx.x; g < ng; g += blockDim.x) {
        const float *p = H[all ? h0 + g : glist[h0 + g]].pos;
        uint32_t q[3];
        for (int d = 0; d < 3; d++) {
            float t = (p[d] - mn[d]) * sc[d];
            q[d] = (t >= 0.f && t < 1024.f) ? (uint32_t)t : 0u;
        }
        key[h0 + g] = morton10(q[0]) | (morton10(q[1]) << 1) | (morton10(q[2]) << 2);
        val[h0 + g] = g;
    }
}
// Candidate records of the Morton-ordered nodes: ah[h0 + j] is the halo at
// sorted position j, gi[h0 + j] its (list position, halo index).
__global__ void k_asc_sorted_recs(HierNodes N, int32_t base, const rsg_halo *H,
                                  const int32_t *glist, int all, int bmin, const int32_t *sval,
                                  AscHalo *ah, int2 *gi) {
    int node = base + blockIdx.x;
    int ng = asc_count(N, node, all), h0 = N.h0[node];
    if (ng <= bmin) return;
    for (int j = threadIdx.x; j < ng; j += blockDim.x) {
        int g = sval[h0 + j], h = all ? h0 + g : glist[h0 + g];
        const rsg_halo &hh = H[h];
        AscHalo c;
        for (int d = 0; d < 3; d++) {
            c.pos[d] = hh.pos[d];
            c.pos[d + 3] = hh.bulkvel[d];
        }
        c.r = hh.r;
        c.vrms = hh.vrms;
        ah[h0 + j] = c;
        gi[h0 + j] = make_int2(g, h);
    }
}
// Buckets of 32 (and 1024) consecutive Morton-ordered candidates.
__global__ void k_asc_buckets_s(HierNodes N, int32_t base, int all, int bmin, const AscHalo *ah,
                                AscBucket *bk, AscBucket *bk2) {
    int node = base + blockIdx.x;
    int ng = asc_count(N, node, all), h0 = N.h0[node];
    if (ng <= bmin) return;
    int nb = (ng + 31) / 32;
    for (int b = threadIdx.x; b < nb; b += blockDim.x) {
        AscBucket B;
        for (int d = 0; d < 3; d++) {
            B.mn[d] = INFINITY;
            B.mx[d] = -INFINITY;
        }
        B.rmax = 0.f;
        B.inv = 0;
        for (int j = 32 * b; j < ng && j < 32 * b + 32; j++) {
            const AscHalo &c = ah[h0 + j];
            if (c.vrms <= 0 || c.r <= 0 || !(c.r == c.r)) {
                B.inv = 1;
                continue;
            }
            for (int d = 0; d < 3; d++) {
                B.mn[d] = fminf(B.mn[d], c.pos[d]);
                B.mx[d] = fmaxf(B.mx[d], c.pos[d]);
            }
            B.rmax = fmaxf(B.rmax, c.r);
        }
        bk[h0 + b] = B;
    }
    __syncthreads();
    int nsb = (nb + 31) / 32;
    for (int sb = threadIdx.x; sb < nsb; sb += blockDim.x) {
        AscBucket S = bk[h0 + 32 * sb];
        for (int b = 32 * sb + 1; b < nb && b < 32 * sb + 32; b++) {
            const AscBucket &B = bk[h0 + b];
            for (int d = 0; d < 3; d++) {
                S.mn[d] = fminf(S.mn[d], B.mn[d]);
                S.mx[d] = fmaxf(S.mx[d], B.mx[d]);
            }
            S.rmax = fmaxf(S.rmax, B.rmax);
            S.inv |= B.inv;
        }
        bk2[h0 + sb] = S;
    }
}
// Smallest float x whose metric (float)sqrt((double)x) can exceed `best`:
// any x at or above the square of best's float successor gives a metric of
// at least that successor, and for a float x, x >= nb^2 holds exactly when
// x >= nb^2 rounded up to a float (__fmul_ru).  The hot loops compare floats
// only (GB300's FP64 pipe is narrow).
__device__ __forceinline__ float asc_xcut(float best) {
    float nb = nextafterf(best, INFINITY);
    return __fmul_ru(nb, nb);
}
// calc_halo_dist's size test (double)h.r > (double)c.r * 0.99999 as a float
// comparison c.r < T: T is the smallest float t with (double)t * 0.99999 >=
// h.r (the product is monotone in t); -inf when no r is filtered (h.r NaN or
// -inf), +inf when every finite r is.  A NaN c.r is never filtered either way.
__device__ float rfilter_threshold(float hr) {
    if (hr != hr || hr == -INFINITY) return -INFINITY;
    if (hr == INFINITY) return INFINITY;
    const double h = hr;
    float t = (float)(h / 0.99999);
    for (int i = 0; i < 8 && !((double)t * 0.99999 >= h); i++) t = nextafterf(t, INFINITY);
    for (int i = 0; i < 8; i++) {
        float q = nextafterf(t, -INFINITY);
        if ((double)q * 0.99999 >= h) t = q;
        else break;
    }
    return t;
}

// One thread per particle of the level (the node from eln): a node of
// millions of particles spreads over the whole GPU.  Nodes with more than
// bmin growing halos scan their Morton-ordered candidates and skip
// a bucket (32) or super-bucket (1024 halos) whose lower bound of x reaches
// asc_xcut of the running best (and, unless the best is below 1e20, holds
// no invalid halo); the others scan the list in order.
__global__ void k_asc_assign_p(const Rec *W, int64_t M, const int32_t *eln, HierNodes N,
                               int32_t base, const rsg_halo *H, const rsg_extra_halo_info *E,
                               const int32_t *glist, const int32_t *redirect,
                               const AscBucket *bk, const AscBucket *bk2, const AscHalo *ah,
                               const int2 *gi, int bmin, int32_t *phalo) {
    int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= M) return;
    int k = eln[i];
    if (k < 0) return;
    int node = base + k;
    int ph = phalo[i];
    if (ph >= 0) {
        if (redirect[ph] >= 0) phalo[i] = redirect[ph];
        return;
    }
    int mi = N.maxi[node], ng = N.ng[node], h0 = N.h0[node];
    if (ng == 1) {
        phalo[i] = mi;
        return;
    }
    float pos[6];
#pragma unroll
    for (int d = 0; d < 6; d++) pos[d] = W[i].pos[d];
    AscHalo hm;
    for (int d = 0; d < 3; d++) {
        hm.pos[d] = H[mi].pos[d];
        hm.pos[d + 3] = H[mi].bulkvel[d];
    }
    hm.r = H[mi].r;
    hm.vrms = H[mi].vrms;
    bool bvalid = asc_valid(hm);
    float bx = bvalid ? asc_x(hm, pos) : 0.f;
    float best = bvalid ? sqrt_fd(bx) : 1e20f;
    int bh = mi;
    if (ng > bmin) {
        // Morton-ordered candidates, (metric, list position) lexicographic;
        // mi holds list position 0.
        int bpos = 0;
        float cut = asc_xcut(best);
        for (int j = 0; j < ng;) {
            if ((j & 1023) == 0) {
                const AscBucket &S = bk2[h0 + (j >> 10)];
                if ((!S.inv || best < 1e20f) && asc_bucket_lb(S, pos) >= cut) {
                    j += 1024;
                    continue;
                }
            }
            if ((j & 31) == 0) {
                const AscBucket &B = bk[h0 + (j >> 5)];
                if ((!B.inv || best < 1e20f) && asc_bucket_lb(B, pos) >= cut) {
                    j += 32;
                    continue;
                }
            }
            const AscHalo c = ah[h0 + j];
            float m;
            if (!asc_valid(c)) {
                m = 1e20f;
            } else {
                float x = asc_x(c, pos);
                if (x >= cut) {
                    j++;
                    continue;
                }
                m = sqrt_fd(x);
            }
            int gp = gi[h0 + j].x;
            if (m < best || (m == best && gp < bpos)) {
                best = m;
                bpos = gp;
                bh = gi[h0 + j].y;
                cut = asc_xcut(best);
            }
            j++;
        }
    } else {
        for (int g = 0; g < ng; g++) {
            const rsg_halo &hh = H[glist[h0 + g]];
            AscHalo c;
            for (int d = 0; d < 3; d++) {
                c.pos[d] = hh.pos[d];
                c.pos[d + 3] = hh.bulkvel[d];
            }
            c.r = hh.r;
            c.vrms = hh.vrms;
            if (!asc_valid(c)) {
                if (1e20f < best) {
                    best = 1e20f;
                    bh = glist[h0 + g];
                    bvalid = false;
                }
                continue;
            }
            float x = asc_x(c, pos);
            if (!(bvalid && !(x < bx))) {
                float m = sqrt_fd(x);
                if (m < best) {
                    best = m;
                    bx = x;
                    bvalid = true;
                    bh = glist[h0 + g];
                }
            }
        }
    }
    int h = bh;
    for (int guard = 0; E[h].sub_of > -1; guard++) {
        if (guard >= 100000) {  // sub_of links form a forest: deeper means a cycle
            loop_limit_hit();
            break;
        }
        if (pdist(H[h], pos) > E[h].max_metric) h = (int)E[h].sub_of;
        else break;
    }
    phalo[i] = h;
}

// Batched form: the records of every node grouped by label with one stable
// radix sort on (node start, label + 1); records outside the level's nodes
// keep their places.  (The plain form reproduces the reference's recursive
// midpoint partition instead, whose record order the reference's later
// sampling depends on.)
// Keys of label_sort_stable: the label inside each node of the level; val
// and val_out start as the identity, so elements outside the level's nodes
// (which the segmented sort leaves alone) keep their place.
__global__ void k_lsort_keys(const int32_t *eln, int64_t M, const int32_t *lab, uint32_t *key,
                             uint32_t *val, uint32_t *val_out) {
    int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= M) return;
    key[i] = eln[i] >= 0 ? (uint32_t)(lab[i] + 1) : 0u;
    val[i] = val_out[i] = (uint32_t)i;
}
// Keys of the whole-array form: (node start or own index, label + 1).
__global__ void k_lsort_keys64(const int32_t *eln, int64_t M, HierNodes N, int32_t base,
                               const int32_t *lab, uint64_t *key, uint32_t *val) {
    int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= M) return;
    int k = eln[i];
    uint64_t hi = (k >= 0) ? (uint64_t)N.start[base + k] : (uint64_t)i;
    key[i] = (hi << 32) | (uint64_t)(uint32_t)(k >= 0 ? lab[i] + 1 : 0);
    val[i] = (uint32_t)i;
}
__global__ void k_node_ends(HierNodes N, int32_t base, int32_t cnt, int32_t *end) {
    int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k < cnt) end[k] = N.start[base + k] + N.n[base + k];
}

// Regroup keys for reassign_halo_particles (src/groupies.c:316-331) and the
// core sort of src/fun_times.c:204-227 (by squared distance to the halo).
__global__ void k_halokeys(const int32_t *eln, int64_t M, HierNodes N, int32_t base,
                           const int32_t *phalo, uint64_t *key, uint32_t *val) {
    int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= M) return;
    int k = eln[i];
    uint64_t kk;
    if (k < 0) kk = (uint64_t)i << 32;
    else {
        int s = N.start[base + k], h0 = N.h0[base + k];
        kk = ((uint64_t)s << 32) | (uint64_t)(phalo[i] - h0);
    }
    key[i] = kk;
    val[i] = (uint32_t)i;
}
__global__ void k_halo_heads(const int32_t *eln, int64_t M, HierNodes N, int32_t base,
                             const int32_t *phalo, rsg_halo *H) {
    int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= M) return;
    int k = eln[i];
    if (k < 0) return;
    int s = N.start[base + k];
    if (i == s || phalo[i] != phalo[i - 1]) H[phalo[i]].p_start = i;
}
__global__ void k_halo_tails(const int32_t *eln, int64_t M, HierNodes N, int32_t base,
                             const int32_t *phalo, rsg_halo *H) {
    int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= M) return;
    int k = eln[i];
    if (k < 0) return;
    int s = N.start[base + k], n = N.n[base + k];
    if (i == s + n - 1 || phalo[i] != phalo[i + 1]) H[phalo[i]].num_p = i + 1 - H[phalo[i]].p_start;
}

// The halo fields of calc_basic_halo_props from the mean and the summed
// squared deviations (src/properties.c:88-125); returns whether the Vmax
// histogram is built and its scale.
__device__ void basic_decide(rsg_halo &hh, const double *mean, const double *p2, int np,
                             const DevCfg *C, int *do_bins, float *rsc_out) {
    hh.r = hh.vrms = 0;
    for (int k = 0; k < 6; k++) {
        if (k < 3) hh.r = (float)((double)hh.r + p2[k] / (double)np);
        else hh.vrms = (float)((double)hh.vrms + p2[k] / (double)np);
    }
    double pe = (double)hh.r / (double)np, ve = (double)hh.vrms / (double)np;
    if ((!hh.min_pos_err) || ((double)hh.min_pos_err > pe)) {
        hh.min_pos_err = (float)pe;
        hh.n_core = hh.num_p;
        for (int k = 0; k < 3; k++) hh.pos[k] = (float)mean[k];
    }
    if ((!hh.min_vel_err) || ((double)hh.min_vel_err > ve)) {
        hh.min_vel_err = (float)ve;
        for (int k = 3; k < 6; k++) hh.pos[k] = (float)mean[k];
    }
    for (int k = 3; k < 6; k++) hh.bulkvel[k - 3] = (float)mean[k];
    hh.m = (float)hh.num_p;
    if (!hh.num_child_particles) hh.num_child_particles = hh.num_p;
    hh.r = (float)cbrt((double)hh.num_p / ((4.0 * M_PI / 3.0) * C->rvir_dens));
    hh.child_r = (float)cbrt((double)hh.num_child_particles / ((4.0 * M_PI / 3.0) * C->rvir_dens));
    hh.vmax = hh.vmax_r = 0;
    *do_bins = (hh.child_r > 0);
    *rsc_out = (float)(50.0 / (double)hh.child_r);
}
// The Vmax histogram bin of one particle at squared distance ds:
// (int64_t)(sqrt((double)ds) * rsc) as the reference computes it, or -1 past
// bin 49.  The FP32 estimate is within 2e-5 of that product below 60, so it
// decides the bin unless it lies within 1e-4 of a bin edge; then the FP64
// expression is evaluated.
__device__ __forceinline__ int vmax_bin(float ds, float rsc) {
    float bf = sqrtf(ds) * rsc;
    if (!(bf < 60.f)) return -1;
    float fr = bf - floorf(bf);
    int64_t b = (fr < 1e-4f || fr > 1.f - 1e-4f) ? (int64_t)(sqrt((double)ds) * (double)rsc)
                                                  : (int64_t)bf;
    return (b < 50) ? (int)b : -1;
}
// Vmax and Rvmax from the 50-bin mass histogram (src/properties.c:39-69), then
// the final radius and vrms of calc_basic_halo_props.
__device__ void basic_vmax(rsg_halo &hh, const int *bins, int do_bins, float rsc_s,
                           const DevCfg *C) {
    if (do_bins) {
        float rsc = rsc_s, vm = 0.f;
        int64_t tp = 0;
        for (int i = 0; i < 50; i++) {
            // (float)((i + 1.0) / (double)rsc), src/properties.c:58, as one FP32
            // division: the exact quotient of a small integer by a float lies
            // either on a float rounding midpoint or more than 2^-48 (relative)
            // from every one, so the FP64 quotient rounds to the same float
            float r = __fdiv_rn((float)(i + 1), rsc);
            if ((double)r < C->force_res) r = (float)C->force_res;
            tp += bins[i];
            float vc = __fdiv_rn(__ll2float_rn(tp), r);
            if (vc > vm) vm = vc;
        }
        float sn = (float)C->scale_now;
        float v = (float)sqrt(RSG_GC * (double)vm * C->particle_mass / (double)sn);
        hh.vmax = v;
        hh.vmax_r = (float)(sqrt((double)sn) * (double)v * C->dyn_time);
    }
    if (hh.vmax_r) hh.r = hh.vmax_r;
    hh.vrms = sqrt_fd(hh.vrms);
}

// calc_basic_halo_props + estimate_vmax (src/properties.c:39-125); one
// block per listed halo.
__global__ void k_basic_props(const Rec *W, rsg_halo *H, const int32_t *list, const DevCfg *C,
                              int seq_max, int big, int small) {
    __shared__ double sm[40];
    __shared__ double mean[6], p2[6];
    __shared__ int bins[50];
    int h = list[blockIdx.x];
    rsg_halo &hh = H[h];
    int ps = (int)hh.p_start, np = (int)hh.num_p;
    // chunked and warp paths (batched form); halos emptied by the assignment
    // (num_p 0) are still processed, as the reference processes them
    if (np > big || np <= small) return;
    if (np <= seq_max) {
        // in array order (src/properties.c:76-87): the block stages values,
        // thread 0 adds them
        __shared__ double stage[256][6];
        double a = 0, b = 0;  // lane d of warp 0 owns coordinate d
        for (int b0 = 0; b0 < np; b0 += blockDim.x) {
            int i = b0 + threadIdx.x;
            if (i < np)
                for (int d = 0; d < 6; d++) stage[threadIdx.x][d] = (double)W[ps + i].pos[d];
            __syncthreads();
            if (threadIdx.x < 6) {
                int m = min((int)blockDim.x, np - b0), d = threadIdx.x;
                for (int t = 0; t < m; t++) a += stage[t][d];
            }
            __syncthreads();
        }
        if (threadIdx.x < 6) mean[threadIdx.x] = a / (double)np;
        __syncthreads();
        for (int b0 = 0; b0 < np; b0 += blockDim.x) {
            int i = b0 + threadIdx.x;
            if (i < np)
                for (int d = 0; d < 6; d++) {
                    double x = (double)W[ps + i].pos[d] - mean[d];
                    stage[threadIdx.x][d] = x * x;
                }
            __syncthreads();
            if (threadIdx.x < 6) {
                int m = min((int)blockDim.x, np - b0), d = threadIdx.x;
                for (int t = 0; t < m; t++) b += stage[t][d];
            }
            __syncthreads();
        }
        if (threadIdx.x < 6) p2[threadIdx.x] = b;
        __syncthreads();
    } else {
    double acc[6] = {0, 0, 0, 0, 0, 0};
    for (int i = threadIdx.x; i < np; i += blockDim.x)
#pragma unroll
        for (int d = 0; d < 6; d++) acc[d] += (double)W[ps + i].pos[d];
    for (int d = 0; d < 6; d++) {
        double t = block_sum_d(acc[d], sm);
        if (threadIdx.x == 0) mean[d] = t / (double)np;
    }
    __syncthreads();
    for (int d = 0; d < 6; d++) acc[d] = 0;
    for (int i = threadIdx.x; i < np; i += blockDim.x)
#pragma unroll
        for (int d = 0; d < 6; d++) {
            double x = (double)W[ps + i].pos[d] - mean[d];
            acc[d] += x * x;
        }
    for (int d = 0; d < 6; d++) {
        double t = block_sum_d(acc[d], sm);
        if (threadIdx.x == 0) p2[d] = t;
    }
    }
    if (threadIdx.x < 50) bins[threadIdx.x] = 0;
    __shared__ float rsc_s;
    __shared__ int do_bins;
    __syncthreads();
    if (threadIdx.x == 0) {
        int db;
        float rs;
        basic_decide(hh, mean, p2, np, C, &db, &rs);
        do_bins = db;
        rsc_s = rs;
    }
    __syncthreads();
    if (do_bins) {
        float rsc = rsc_s;
        float c0 = hh.pos[0], c1 = hh.pos[1], c2 = hh.pos[2];
        for (int i = threadIdx.x; i < np; i += blockDim.x) {
            float dx, ds = 0.f;
            dx = fsub(c0, W[ps + i].pos[0]); ds = fadd(ds, fmul(dx, dx));
            dx = fsub(c1, W[ps + i].pos[1]); ds = fadd(ds, fmul(dx, dx));
            dx = fsub(c2, W[ps + i].pos[2]); ds = fadd(ds, fmul(dx, dx));
            int key = vmax_bin(ds, rsc);
            // lanes with the same bin add once (shared-memory atomics on 50 bins
            // would otherwise serialise)
            unsigned peers = __match_any_sync(__activemask(), key);
            if (key >= 0 && (threadIdx.x & 31) == __ffs(peers) - 1) atomicAdd(&bins[key], __popc(peers));
        }
    }
    __syncthreads();
    if (threadIdx.x == 0) basic_vmax(hh, bins, do_bins, rsc_s, C);
}

// Batched form, halos of at most RSG_BP_WARP particles: the same steps with
// one warp per halo (a block per halo of tens of particles leaves most of
// its threads idle and spends its time in barriers).  Each lane sums in
// double-float on the FP32 pipe (df64.cuh; the FP64 pipe bound the FP64
// form), the lanes' sums are added in FP64 (the batched form's sums are not
// in the reference's order anyway); lane 0 takes the decisions.
#define RSG_BP_WARP 1024
__global__ void __launch_bounds__(256) k_basic_props_w(const Rec *W, rsg_halo *H,
                                                       const int32_t *list, int32_t nl,
                                                       const DevCfg *C) {
    __shared__ int bins_s[8][50];
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int t = blockIdx.x * 8 + w;
    if (t >= nl) return;
    rsg_halo &hh = H[list[t]];
    const int ps = (int)hh.p_start, np = (int)hh.num_p;
    if (np > RSG_BP_WARP) return;  // the block kernel's
    DF acc[6];
    double mean[6], p2[6];
#pragma unroll
    for (int d = 0; d < 6; d++) acc[d] = DF{0.f, 0.f};
    for (int i = lane; i < np; i += 32)
#pragma unroll
        for (int d = 0; d < 6; d++) acc[d] = df_add_f(acc[d], W[ps + i].pos[d]);
    DF md[6];
#pragma unroll
    for (int d = 0; d < 6; d++) {
        // warp_sum_d leaves the total in lane 0; every lane needs the mean
        mean[d] = __shfl_sync(0xffffffffu, warp_sum_d(df_to_double(acc[d])), 0) / (double)np;
        md[d] = df_from_double(mean[d]);
        acc[d] = DF{0.f, 0.f};
    }
    for (int i = lane; i < np; i += 32)
#pragma unroll
        for (int d = 0; d < 6; d++)
            acc[d] = df_add(acc[d], df_sqr(df_sub_from_f(W[ps + i].pos[d], md[d])));
#pragma unroll
    for (int d = 0; d < 6; d++) p2[d] = warp_sum_d(df_to_double(acc[d]));  // lane 0's are used
    int db = 0;
    float rs = 0.f;
    if (lane == 0) basic_decide(hh, mean, p2, np, C, &db, &rs);
    db = __shfl_sync(0xffffffffu, db, 0);
    rs = __shfl_sync(0xffffffffu, rs, 0);
    int *bins = bins_s[w];
    for (int k = lane; k < 50; k += 32) bins[k] = 0;
    __syncwarp();  // also orders lane 0's halo writes before the reads below
    if (db) {
        const float c0 = hh.pos[0], c1 = hh.pos[1], c2 = hh.pos[2];
        for (int i = lane; i < np; i += 32) {
            float dx, ds = 0.f;
            dx = fsub(c0, W[ps + i].pos[0]); ds = fadd(ds, fmul(dx, dx));
            dx = fsub(c1, W[ps + i].pos[1]); ds = fadd(ds, fmul(dx, dx));
            dx = fsub(c2, W[ps + i].pos[2]); ds = fadd(ds, fmul(dx, dx));
            const int key = vmax_bin(ds, rs);
            if (key >= 0) atomicAdd(&bins[key], 1);
        }
    }
    __syncwarp();
    if (lane == 0) basic_vmax(hh, bins, db, rs, C);
}

// Batched form, halos above Tuning::bp_big particles: calc_basic_halo_props
// over chunks of Tuning::bp_chunk particles, one block per chunk per pass;
// the partial sums and histograms are added per halo in chunk order
// (deterministic).
struct BPChunk {
    int32_t t, start, n, pad;  // t: entry of the halo list
};
struct BPPart {
    double d[6];
    int bins[50];
};
__global__ void k_bp_nch(const rsg_halo *H, const int32_t *list, int32_t nl, int big, int chunk,
                         int32_t *nch) {
    int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t > nl) return;
    int np = (t < nl) ? (int)H[list[t]].num_p : 0;
    nch[t] = (np > big) ? (np + chunk - 1) / chunk : 0;
}
__global__ void k_bp_fill(const rsg_halo *H, const int32_t *list, int32_t nl, int chunk,
                          const int32_t *nch, const int32_t *c0, BPChunk *C) {
    int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= nl) return;
    const rsg_halo &hh = H[list[t]];
    int ps = (int)hh.p_start, np = (int)hh.num_p;
    for (int c = 0; c < nch[t]; c++) {
        BPChunk x;
        x.t = t;
        x.start = ps + c * chunk;
        x.n = min(chunk, np - c * chunk);
        x.pad = 0;
        C[c0[t] + c] = x;
    }
}
__global__ void __launch_bounds__(256) k_bp_sum6(const Rec *W, const BPChunk *C,
                                                 const double *mean, BPPart *P) {
    __shared__ double sm[40];
    BPChunk c = C[blockIdx.x];
    double a[6] = {0, 0, 0, 0, 0, 0};
    for (int i = threadIdx.x; i < c.n; i += blockDim.x)
        for (int d = 0; d < 6; d++) {
            double x = (double)W[c.start + i].pos[d];
            if (mean) {  // second pass: squared deviations
                x -= mean[6 * c.t + d];
                x *= x;
            }
            a[d] += x;
        }
    for (int d = 0; d < 6; d++) {
        double t = block_sum_d(a[d], sm);
        if (threadIdx.x == 0) P[blockIdx.x].d[d] = t;
    }
}
__global__ void k_bp_mean(const rsg_halo *H, const int32_t *list, int32_t nl, const int32_t *nch,
                          const int32_t *c0, const BPPart *P, double *mean) {
    int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= nl || nch[t] == 0) return;
    double a[6] = {0, 0, 0, 0, 0, 0};
    for (int c = c0[t]; c < c0[t] + nch[t]; c++)
        for (int d = 0; d < 6; d++) a[d] += P[c].d[d];
    for (int d = 0; d < 6; d++) mean[6 * t + d] = a[d] / (double)H[list[t]].num_p;
}
__global__ void k_bp_decide(rsg_halo *H, const int32_t *list, int32_t nl, const int32_t *nch,
                            const int32_t *c0, const BPPart *P, const double *mean,
                            const DevCfg *C, int *dob, float *rsc) {
    int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= nl || nch[t] == 0) return;
    double p2[6] = {0, 0, 0, 0, 0, 0};
    for (int c = c0[t]; c < c0[t] + nch[t]; c++)
        for (int d = 0; d < 6; d++) p2[d] += P[c].d[d];
    rsg_halo &hh = H[list[t]];
    basic_decide(hh, mean + 6 * t, p2, (int)hh.num_p, C, &dob[t], &rsc[t]);
}
__global__ void __launch_bounds__(256) k_bp_hist(const Rec *W, const BPChunk *C,
                                                 const rsg_halo *H, const int32_t *list,
                                                 const int *dob, const float *rsc, BPPart *P) {
    __shared__ int bins[50];
    BPChunk c = C[blockIdx.x];
    if (threadIdx.x < 50) bins[threadIdx.x] = 0;
    __syncthreads();
    if (dob[c.t]) {
        const rsg_halo &hh = H[list[c.t]];
        float r = rsc[c.t], c0 = hh.pos[0], c1 = hh.pos[1], c2 = hh.pos[2];
        for (int i = threadIdx.x; i < c.n; i += blockDim.x) {
            float dx, ds = 0.f;
            dx = fsub(c0, W[c.start + i].pos[0]); ds = fadd(ds, fmul(dx, dx));
            dx = fsub(c1, W[c.start + i].pos[1]); ds = fadd(ds, fmul(dx, dx));
            dx = fsub(c2, W[c.start + i].pos[2]); ds = fadd(ds, fmul(dx, dx));
            int key = vmax_bin(ds, r);
            unsigned peers = __match_any_sync(__activemask(), key);
            if (key >= 0 && (threadIdx.x & 31) == __ffs(peers) - 1) atomicAdd(&bins[key], __popc(peers));
        }
    }
    __syncthreads();
    if (threadIdx.x < 50) P[blockIdx.x].bins[threadIdx.x] = bins[threadIdx.x];
}
__global__ void k_bp_vmax(rsg_halo *H, const int32_t *list, int32_t nl, const int32_t *nch,
                          const int32_t *c0, const BPPart *P, const int *dob, const float *rsc,
                          const DevCfg *C) {
    int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= nl || nch[t] == 0) return;
    int bins[50];
    for (int b = 0; b < 50; b++) bins[b] = 0;
    for (int c = c0[t]; c < c0[t] + nch[t]; c++)
        for (int b = 0; b < 50; b++) bins[b] += P[c].bins[b];
    basic_vmax(H[list[t]], bins, dob[t], rsc[t], C);
}

// growing-halo list of a level: node glist entries concatenated
// One block per node.
__global__ void k_list_growing(HierNodes N, int32_t base, const int32_t *goff,
                               const int32_t *glist, int32_t *list, int32_t *lnode) {
    int k = blockIdx.x;
    int node = base + k;
    for (int g = threadIdx.x; g < N.ng[node]; g += blockDim.x) {
        list[goff[k] + g] = glist[N.h0[node] + g];
        lnode[goff[k] + g] = k;
    }
}
__global__ void k_ng(HierNodes N, int32_t base, int32_t count, int32_t *out, int all) {
    int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k > count) return;
    if (k == count) { out[k] = 0; return; }
    int node = base + k;
    out[k] = all ? N.h1[node] - N.h0[node] : N.ng[node];
}
__global__ void k_list_all(HierNodes N, int32_t base, int32_t count, const int32_t *off,
                           int32_t *list) {
    int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= count) return;
    int node = base + k;
    for (int h = N.h0[node]; h < N.h1[node]; h++) list[off[k] + h - N.h0[node]] = h;
}

// Biggest halo among growing ones (all = 0) or all halos (all = 1); one
// block (256 threads) per node.
__global__ void __launch_bounds__(256) k_maxi(HierNodes N, int32_t base, const rsg_halo *H,
                                              const int32_t *glist, int all) {
    int node = base + blockIdx.x;
    int h0 = N.h0[node];
    int mi = all ? biggest_blk(H, h0, N.h1[node], 0, 0)
                 : biggest_blk(H, h0, N.h1[node], 1, glist[h0]);
    if (threadIdx.x == 0) N.maxi[node] = mi;
}

// calc_halo_dist(c, h) (src/subhalo_metric.c:73-77) and, when the value is
// a metric rather than the 1e20 of a too-small or invalid candidate, its
// float sum x before the square root (else x = inf).
__device__ __forceinline__ float hdist_x(const rsg_halo &c, const rsg_halo &h, float *x) {
    *x = INFINITY;
    if ((double)h.r > (double)c.r * 0.99999) return 1e20f;
    if (c.vrms <= 0 || c.r <= 0) return 1e20f;
    AscHalo a;
    for (int d = 0; d < 3; d++) {
        a.pos[d] = c.pos[d];
        a.pos[d + 3] = c.bulkvel[d];
    }
    a.r = c.r;
    a.vrms = c.vrms;
    *x = asc_x(a, h.pos);
    return sqrt_fd(*x);
}
// find_best_parent (src/subhalo_metric.c:185-191) over the node's listed
// halos: the first strict minimum of calc_halo_dist in list order, starting
// from the biggest halo (which therefore wins every tie).  Nodes listing
// more than bmin halos scan their Morton-ordered candidates
// (k_asc_sorted_recs over the same list) and take (metric, list position)
// lexicographically, the biggest halo holding position -1.  While the best
// is below 1e20 (the value of a too-small or invalid candidate), a bucket is
// skipped when every valid halo in it is too small (r * 0.99999 < h.r for
// its largest r) or its lower bound of x reaches the cut of the best.
__global__ void k_best_parent(HierNodes N, int32_t base, int32_t count, const int32_t *loff,
                              const int32_t *list, const int32_t *hnode, rsg_halo *H,
                              rsg_extra_halo_info *E, const AscBucket *bk, const AscBucket *bk2,
                              const AscHalo *ah, const int2 *gi, int bmin) {
    int t = blockIdx.x * blockDim.x + threadIdx.x;
    int tot = loff[count];
    if (t >= tot) return;
    int h = list[t];
    int k = hnode[t];
    int node = base + k;
    int mi = N.maxi[node];
    int res = h;
    if (h != mi) {
        const rsg_halo &hh = H[h];
        float bx;
        float best = hdist_x(H[mi], hh, &bx);
        res = mi;
        const int g0 = loff[k], n = loff[k + 1] - g0, h0 = N.h0[node];
        if (n > bmin) {
            int bpos = -1;
            float cut = asc_xcut(best);
            const float rt = rfilter_threshold(hh.r);
            for (int j = 0; j < n;) {
                if (best < 1e20f) {
                    if ((j & 1023) == 0) {
                        const AscBucket &S = bk2[h0 + (j >> 10)];
                        if (S.rmax < rt || asc_bucket_lb(S, hh.pos) >= cut) {
                            j += 1024;
                            continue;
                        }
                    }
                    if ((j & 31) == 0) {
                        const AscBucket &B = bk[h0 + (j >> 5)];
                        if (B.rmax < rt || asc_bucket_lb(B, hh.pos) >= cut) {
                            j += 32;
                            continue;
                        }
                    }
                }
                const AscHalo c = ah[h0 + j];
                float m;
                if (c.r < rt || c.vrms <= 0 || c.r <= 0) {
                    m = 1e20f;
                } else {
                    float x = asc_x(c, hh.pos);
                    if (x >= cut) {
                        j++;
                        continue;
                    }
                    m = sqrt_fd(x);
                }
                int gp = gi[h0 + j].x;
                if (m < best || (m == best && gp < bpos)) {
                    best = m;
                    bpos = gp;
                    res = gi[h0 + j].y;
                    cut = asc_xcut(best);
                }
                j++;
            }
        } else {
            for (int g = 0; g < n; g++) {
                int c = list[g0 + g];
                float x;
                float m = hdist_x(H[c], hh, &x);
                if (m < best) {
                    best = m;
                    res = c;
                }
            }
        }
    }
    E[h].sub_of = res;
}
__global__ void k_list_node(int32_t count, const int32_t *loff, int32_t *hnode) {
    int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= count) return;
    for (int g = loff[k]; g < loff[k + 1]; g++) hnode[g] = k;
}

// _fix_parents (src/groupies.c:425-485) and calc_num_child_particles
// (src/properties.c:139-163) for every node of a level in parallel.  Sequentially, each halo i (ascending) is pushed to the front of
// its parent's child list, so a parent's list runs from its largest child
// down: next_cochild(i) is the largest sibling below i, prev_cochild(i) the
// smallest sibling above it, child(P) the largest child.  Sorting (parent,
// index) pairs gives those neighbours directly.  num_child_particles is the
// sum of num_p over the halo's subtree: every halo adds its num_p to itself
// and each ancestor.
__global__ void k_fp_count(HierNodes N, int32_t base, int32_t cnt, int32_t *hc) {
    int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k > cnt) return;
    hc[k] = (k < cnt) ? N.h1[base + k] - N.h0[base + k] : 0;
}
__global__ void k_fp_reset(HierNodes N, int32_t base, rsg_extra_halo_info *E) {
    int node = base + blockIdx.x;
    for (int i = N.h0[node] + threadIdx.x; i < N.h1[node]; i += blockDim.x) {
        E[i].next_cochild = E[i].prev_cochild = E[i].child = -1;
        if (E[i].sub_of == i) E[i].sub_of = -1;
    }
}
__global__ void k_fp_keys(HierNodes N, int32_t base, const int32_t *hofs, const rsg_halo *H,
                          rsg_extra_halo_info *E, uint64_t *key, uint32_t *val) {
    int node = base + blockIdx.x;
    int h0 = N.h0[node];
    for (int i = h0 + threadIdx.x; i < N.h1[node]; i += blockDim.x) {
        int64_t so = E[i].sub_of;
        E[i].max_metric = (so < 0) ? 1e10f : pdist(H[i], H[so].pos);
        int64_t at = hofs[blockIdx.x] + (i - h0);
        key[at] = (so < 0) ? ~0ull : (((uint64_t)so << 32) | (uint64_t)(uint32_t)i);
        val[at] = (uint32_t)at;
    }
}
__global__ void k_fp_link(const uint64_t *key, int64_t n, rsg_extra_halo_info *E) {
    int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (e >= n || key[e] == ~0ull) return;
    uint64_t p = key[e] >> 32;
    int i = (int)(uint32_t)key[e];
    bool lo = e > 0 && (key[e - 1] >> 32) == p;
    bool hi = e + 1 < n && key[e + 1] != ~0ull && (key[e + 1] >> 32) == p;
    E[i].next_cochild = lo ? (int64_t)(uint32_t)key[e - 1] : -1;
    E[i].prev_cochild = hi ? (int64_t)(uint32_t)key[e + 1] : -1;
    if (!hi) E[p].child = i;
}
__global__ void k_nc_sum(HierNodes N, int32_t base, rsg_halo *H, const rsg_extra_halo_info *E,
                         int *err) {
    int node = base + blockIdx.x;
    int h0 = N.h0[node], h1 = N.h1[node];
    for (int i = h0 + threadIdx.x; i < h1; i += blockDim.x) H[i].num_child_particles = 0;
    __syncthreads();
    for (int i = h0 + threadIdx.x; i < h1; i += blockDim.x) {
        unsigned long long np = (unsigned long long)H[i].num_p;
        int64_t a = i;
        int guard = 0;
        while (a >= h0 && a < h1) {
            atomicAdd((unsigned long long *)&H[a].num_child_particles, np);
            a = E[a].sub_of;
            if (++guard > (h1 - h0)) {  // a cycle of sub_of links
                atomicExch(err, 1);
                break;
            }
        }
    }
}

// core sort keys: within each halo of the level-0 nodes, by float squared
// distance to the halo position (src/fun_times.c:204-214)
__global__ void k_corekeys(const Rec *W, const int32_t *eln, int64_t M, const int32_t *phalo,
                           const rsg_halo *H, uint64_t *key, uint32_t *val) {
    int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= M) return;
    uint64_t kk;
    if (eln[i] < 0) kk = ((uint64_t)i << 32);
    else {
        const rsg_halo &h = H[phalo[i]];
        float dx = 0.f, ds;
#pragma unroll
        for (int j = 0; j < 3; j++) {
            ds = fsub(h.pos[j], W[i].pos[j]);
            dx = fadd(dx, fmul(ds, ds));
        }
        kk = ((uint64_t)h.p_start << 32) | (uint64_t)f2ord(dx);
    }
    key[i] = kk;
    val[i] = (uint32_t)i;
}

// Output: caller particles in the final order, halo p_start relative to it.
__global__ void k_write_back(const Rec *W, int64_t M, const int32_t *wgroup,
                             const int64_t *goff, const int64_t *woff, const rsg_particle *Pin,
                             rsg_particle *Pout) {
    int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= M) return;
    int g = wgroup[i];
    Pout[goff[g] + (i - woff[g])] = Pin[W[i].ridx];
}
__global__ void k_halo_out(rsg_halo *H, rsg_extra_halo_info *E, int32_t nh, const int32_t *hgrp,
                           const int64_t *goff, const int64_t *woff) {
    int h = blockIdx.x * blockDim.x + threadIdx.x;
    if (h >= nh) return;
    int g = hgrp[h];
    H[h].p_start = goff[g] + (H[h].p_start - woff[g]);
}
__global__ void k_halo_group(HierNodes N, const int32_t *leaves, int32_t nl, int32_t *hgrp) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < nl) hgrp[i] = N.group[leaves[i]];
}
// Working records of every group: one thread per record, its group by a
// binary search over the record offsets (a group of millions of particles
// spreads over the GPU), and one thread per group for the level-0 nodes.
__global__ void k_make_w(const rsg_particle *P, int64_t ng, const int64_t *goff,
                         const int64_t *woff, int64_t M, Rec *W, int32_t *wgroup) {
    int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (e >= M) return;
    int64_t lo = 0, hi = ng;  // last g with woff[g] <= e
    while (hi - lo > 1) {
        int64_t mid = (lo + hi) >> 1;
        if (woff[mid] <= e) lo = mid;
        else hi = mid;
    }
    int64_t src = goff[lo] + (e - woff[lo]);
    Rec r;
#pragma unroll
    for (int d = 0; d < 6; d++) r.pos[d] = P[src].pos[d];
    r.ridx = (int32_t)src;
    r.aux = 0;
    W[e] = r;
    wgroup[e] = (int32_t)lo;
}
__global__ void k_make_nodes(int64_t ng, const int64_t *woff, const int64_t *gsz, HierNodes N) {
    int64_t g = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (g >= ng) return;
    N.start[g] = (int32_t)woff[g];
    N.n[g] = (int32_t)gsz[g];
    N.parent[g] = -1;
    N.group[g] = (int32_t)g;
    N.level[g] = 0;
    N.nchild[g] = 0;
}

// ---- host driver ------------------------------------------------------------

template <class K, class V>
static void sort_pairs(Arena &ar, K *k, K *k2, V *v, V *v2, int64_t n, int bits, cudaStream_t st) {
    size_t b = 0;
    cub::DeviceRadixSort::SortPairs(nullptr, b, k, k2, v, v2, (int)n, 0, bits, st);
    size_t m = ar.used;
    void *t = ar.take(b + 256);
    cub::DeviceRadixSort::SortPairs(t, b, k, k2, v, v2, (int)n, 0, bits, st);
    RSG_CHECK_LAUNCH();
    ar.used = m;
}
static int32_t excl_scan_i32(Arena &ar, const int32_t *in, int32_t *out, int32_t n,
                             cudaStream_t st);

// _fix_parents (+ calc_num_child_particles) for the nodes [base, base + cnt)
static void fix_parents_level(Arena &ar, HierNodes N, int32_t base, int32_t cnt, rsg_halo *H,
                              rsg_extra_halo_info *E, int *err, bool fix, cudaStream_t st) {
    const int T = 256;
    if (cnt <= 0) return;
    size_t mark = ar.used;
    if (fix) {
        int32_t *hofs = ar.get<int32_t>(cnt + 1);
        launch(k_fp_count, nblk(cnt + 1, T), T, 0, st, N, base, cnt, hofs);
        int32_t nh = excl_scan_i32(ar, hofs, hofs, cnt + 1, st);
        launch(k_fp_reset, cnt, T, 0, st, N, base, E);
        if (nh > 0) {
            uint64_t *k1 = ar.get<uint64_t>(nh), *k2 = ar.get<uint64_t>(nh);
            uint32_t *v1 = ar.get<uint32_t>(nh), *v2 = ar.get<uint32_t>(nh);
            launch(k_fp_keys, cnt, T, 0, st, N, base, (const int32_t *)hofs, (const rsg_halo *)H, E,
                   k1, v1);
            sort_pairs(ar, k1, k2, v1, v2, nh, 64, st);
            launch(k_fp_link, nblk(nh, T), T, 0, st, (const uint64_t *)k2, (int64_t)nh, E);
        }
    }
    launch(k_nc_sum, cnt, T, 0, st, N, base, H, (const rsg_extra_halo_info *)E, err);
    RSG_CHECK_LAUNCH();
    ar.used = mark;
}

// calc_basic_halo_props for the listed halos: one block per halo, and in the
// batched form the chunked passes for halos above Tuning::bp_big particles.
static void basic_props(Arena &ar, const Rec *W, rsg_halo *H, const int32_t *list, int32_t nl,
                        const DevCfg *d_dc, int seq_max, int exact, cudaStream_t st) {
    const int T = 256;
    if (nl <= 0) return;
    launch(k_basic_props, nl, T, 0, st, W, H, list, d_dc, exact ? seq_max : 0,
           exact ? 0x7fffffff : tuning().bp_big, exact ? -1 : RSG_BP_WARP);
    if (exact) return;
    launch(k_basic_props_w, nblk(nl, 8), 256, 0, st, W, H, list, nl, d_dc);
    size_t mark = ar.used;
    int32_t *nch = ar.get<int32_t>(nl + 1), *c0 = ar.get<int32_t>(nl + 1);
    const int bpbig = tuning().bp_big, bpch = tuning().bp_chunk;
    launch(k_bp_nch, nblk(nl + 1, T), T, 0, st, (const rsg_halo *)H, list, nl, bpbig, bpch, nch);
    int32_t nc = excl_scan_i32(ar, nch, c0, nl + 1, st);
    if (nc > 0) {
        BPChunk *C = ar.get<BPChunk>(nc);
        BPPart *P = ar.get<BPPart>(nc);
        double *mean = ar.get<double>(6 * (int64_t)nl);
        int *dob = ar.get<int>(nl);
        float *rsc = ar.get<float>(nl);
        launch(k_bp_fill, nblk(nl, T), T, 0, st, (const rsg_halo *)H, list, nl, bpch,
               (const int32_t *)nch, (const int32_t *)c0, C);
        launch(k_bp_sum6, nc, 256, 0, st, W, (const BPChunk *)C, (const double *)nullptr, P);
        launch(k_bp_mean, nblk(nl, T), T, 0, st, (const rsg_halo *)H, list, nl,
               (const int32_t *)nch, (const int32_t *)c0, (const BPPart *)P, mean);
        launch(k_bp_sum6, nc, 256, 0, st, W, (const BPChunk *)C, (const double *)mean, P);
        launch(k_bp_decide, nblk(nl, T), T, 0, st, H, list, nl, (const int32_t *)nch,
               (const int32_t *)c0, (const BPPart *)P, (const double *)mean, d_dc, dob, rsc);
        launch(k_bp_hist, nc, 256, 0, st, W, (const BPChunk *)C, (const rsg_halo *)H, list,
               (const int *)dob, (const float *)rsc, P);
        launch(k_bp_vmax, nblk(nl, T), T, 0, st, H, list, nl, (const int32_t *)nch,
               (const int32_t *)c0, (const BPPart *)P, (const int *)dob, (const float *)rsc, d_dc);
    }
    RSG_CHECK_LAUNCH();
    ar.used = mark;
}

// Batched regroup: every node's elements in label order, stable (the order
// the reference's sequential partition gives up to ties).  Levels whose
// nodes all hold at most RSG_SEGSORT_MAX elements use a segmented sort over
// the nodes on the labels alone; a level with a larger node (where the
// segmented sort's per-segment path is slow) sorts the whole array on
// (node start, label) keys.
#define RSG_SEGSORT_MAX (1 << 18)
static void label_sort_stable(Arena &ar, Rec *W, int32_t *lab, const int32_t *eln, HierNodes N,
                              int32_t base, int32_t cnt, int64_t M, cudaStream_t st) {
    const int T = 256;
    size_t mark = ar.used;
    int nmax = 0;
    {
        int *d = ar.get<int>(1);
        size_t mb = 0;
        cub::DeviceReduce::Max(nullptr, mb, N.n + base, d, cnt, st);
        void *mt = ar.take(mb + 256);
        cub::DeviceReduce::Max(mt, mb, N.n + base, d, cnt, st);
        RSG_CUDA(cudaMemcpyAsync(&nmax, d, sizeof(int), cudaMemcpyDeviceToHost, st));
        RSG_CUDA(cudaStreamSynchronize(st));
        ar.used = mark;
    }
    Rec *wt = ar.get<Rec>(M);
    int32_t *lt = ar.get<int32_t>(M);
    uint32_t *v1 = ar.get<uint32_t>(M), *v2 = ar.get<uint32_t>(M);
    if (nmax <= RSG_SEGSORT_MAX) {
        uint32_t *k1 = ar.get<uint32_t>(M), *k2 = ar.get<uint32_t>(M);
        int32_t *se = ar.get<int32_t>(cnt);
        launch(k_lsort_keys, nblk(M, T), T, 0, st, eln, M, (const int32_t *)lab, k1, v1, v2);
        launch(k_node_ends, nblk(cnt, T), T, 0, st, N, base, cnt, se);
        size_t b = 0;
        RSG_CUDA(cub::DeviceSegmentedSort::StableSortPairs(nullptr, b, k1, k2, v1, v2, (int)M, cnt,
                                                           N.start + base, se, st));
        void *t = ar.take(b + 256);
        RSG_CUDA(cub::DeviceSegmentedSort::StableSortPairs(t, b, k1, k2, v1, v2, (int)M, cnt,
                                                           N.start + base, se, st));
    } else {
        uint64_t *k1 = ar.get<uint64_t>(M), *k2 = ar.get<uint64_t>(M);
        launch(k_lsort_keys64, nblk(M, T), T, 0, st, eln, M, N, base, (const int32_t *)lab, k1, v1);
        int bits = 33;
        while (bits < 64 && (1ll << (bits - 32)) <= M) bits++;
        size_t b = 0;
        RSG_CUDA(cub::DeviceRadixSort::SortPairs(nullptr, b, k1, k2, v1, v2, (int)M, 0, bits, st));
        void *t = ar.take(b + 256);
        RSG_CUDA(cub::DeviceRadixSort::SortPairs(t, b, k1, k2, v1, v2, (int)M, 0, bits, st));
    }
    launch(k_gather<Rec>, nblk(M, T), T, 0, st, (const Rec *)W, (const uint32_t *)v2, M, wt);
    launch(k_gather<int32_t>, nblk(M, T), T, 0, st, (const int32_t *)lab, (const uint32_t *)v2, M,
           lt);
    RSG_CUDA(cudaMemcpyAsync(W, wt, sizeof(Rec) * M, cudaMemcpyDeviceToDevice, st));
    RSG_CUDA(cudaMemcpyAsync(lab, lt, sizeof(int32_t) * M, cudaMemcpyDeviceToDevice, st));
    RSG_CHECK_LAUNCH();
    ar.used = mark;
}

template <class T>
static int32_t excl_scan(Arena &ar, const T *in, T *out, int32_t n, cudaStream_t st) {
    size_t b = 0;
    cub::DeviceScan::ExclusiveSum(nullptr, b, in, out, n, st);
    size_t m = ar.used;
    void *t = ar.take(b + 256);
    cub::DeviceScan::ExclusiveSum(t, b, in, out, n, st);
    RSG_CHECK_LAUNCH();
    ar.used = m;
    T last = 0;
    RSG_CUDA(cudaMemcpyAsync(&last, out + n - 1, sizeof(T), cudaMemcpyDeviceToHost, st));
    RSG_CUDA(cudaStreamSynchronize(st));
    return (int32_t)last;
}
static int32_t excl_scan_i32(Arena &ar, const int32_t *in, int32_t *out, int32_t n,
                             cudaStream_t st) {
    return excl_scan(ar, in, out, n, st);
}
static int32_t select_flagged(Arena &ar, const int32_t *flag, int32_t *out, int64_t n,
                              int32_t first, cudaStream_t st) {
    int *cnt = ar.get<int>(1);
    size_t b = 0;
    cub::DeviceSelect::Flagged(nullptr, b, thrust::counting_iterator<int32_t>(first), flag, out,
                               cnt, (int)n, st);
    size_t m = ar.used;
    void *t = ar.take(b + 256);
    cub::DeviceSelect::Flagged(t, b, thrust::counting_iterator<int32_t>(first), flag, out, cnt,
                               (int)n, st);
    RSG_CHECK_LAUNCH();
    ar.used = m;
    int h = 0;
    RSG_CUDA(cudaMemcpyAsync(&h, cnt, sizeof(int), cudaMemcpyDeviceToHost, st));
    RSG_CUDA(cudaStreamSynchronize(st));
    return h;
}

// 100 hubble_scaling(1/a - 1) for a float scale factor (src/hubble.c:8-19
// with src/potential.c:197-199), in host double arithmetic.
double hubble100(const rsg_config &c, float scale) {
    double z1 = 1.0 / (double)scale, z = z1 - 1.0;
    double zz1 = 1.0 + z, a = 1.0 / zz1;
    double we = (a != 1.0) ? c.w0 + c.wa - c.wa * (a - 1.0) / log(a) : c.w0;
    return 100.0 * sqrt(c.om * (zz1 * zz1 * zz1) + c.ol * pow(a, -3.0 * (1.0 + we)));
}

DevCfg make_devcfg(const rsg_config &c) {
    DevCfg d;
    d.particle_mass = c.particle_mass;
    d.force_res = c.force_res;
    d.scale_now = c.scale_now;
    d.initial_metric_scaling = c.initial_metric_scaling;
    d.include_host_potential_ratio = c.include_host_potential_ratio;
    d.fof_fraction = c.fof_fraction;
    for (int i = 0; i < 5; i++) d.thresh_dens[i] = c.particle_thresh_dens[i];
    d.rvir_dens = c.particle_rvir_dens;
    d.rvir_dens_z0 = c.particle_rvir_dens_z0;
    d.dyn_time = c.dynamical_time;
    d.om = c.om;
    d.ol = c.ol;
    d.w0 = c.w0;
    d.wa = c.wa;
    d.hub = hubble100(c, (float)c.scale_now);
    d.min_halo_particles = c.min_halo_particles;
    d.bound_props = c.bound_props;
    d.shape_iterations = c.shape_iterations;
    d.weighted_shapes = c.weighted_shapes;
    d.exact_ll_calc = c.exact_ll_calc;
    return d;
}

// Morton-ordered candidate records and their buckets for the level's nodes
// with more than Tuning::asc_bucket_min listed halos (all: see asc_count).
static void asc_sorted(Arena &ar, HierNodes N, int32_t base, int32_t cnt, const rsg_halo *H,
                       const int32_t *glist, int all, int32_t NH, AscHalo *ah, int2 *gi,
                       AscBucket *bk, AscBucket *bk2, cudaStream_t st) {
    size_t m2 = ar.used;
    uint32_t *sk = ar.get<uint32_t>(NH), *sk2 = ar.get<uint32_t>(NH);
    int32_t *sv = ar.get<int32_t>(NH), *sv2 = ar.get<int32_t>(NH);
    int32_t *sb = ar.get<int32_t>(cnt), *se = ar.get<int32_t>(cnt);
    const int bmin = tuning().asc_bucket_min;
    launch(k_asc_sort_keys, cnt, 128, 0, st, N, base, H, glist, all, bmin, sk, sv, sb, se);
    size_t tb = 0;
    cub::DeviceSegmentedSort::SortPairs(nullptr, tb, sk, sk2, sv, sv2, NH, cnt, sb, se, st);
    void *tmp = ar.take(tb + 256);
    cub::DeviceSegmentedSort::SortPairs(tmp, tb, sk, sk2, sv, sv2, NH, cnt, sb, se, st);
    RSG_CHECK_LAUNCH();
    launch(k_asc_sorted_recs, cnt, 128, 0, st, N, base, H, glist, all, bmin, (const int32_t *)sv2,
           ah, gi);
    launch(k_asc_buckets_s, cnt, 64, 0, st, N, base, all, bmin, (const AscHalo *)ah, bk, bk2);
    ar.used = m2;
}

SubsOut find_subs_device(Arena &ar, rsg_particle *d_p, int64_t num_p, const int64_t *goff_h,
                         const int64_t *gsz_h, int64_t ngroups, const rsg_config &cfg,
                         rsg_halo *d_halos, rsg_extra_halo_info *d_extra, int64_t max_halos,
                         cudaStream_t st, int exact) {
    SubsOut out{0};
    last_stats()[RSG_STAT_6D_ITEMS] = 0;
    last_stats()[RSG_STAT_6D_SAMPLES] = 0;
    last_stats()[RSG_STAT_NEAR_6D] = 0;
    // Subgroups come out in the reference's order in both forms: the order
    // decides the linking-length sample of a child above 10000 particles
    // (src/groupies.c:295-308), and for every child the array the
    // reference's quickselect runs on, whose early exit on equal end values
    // (mutual nearest neighbours) returns a value that depends on that
    // array's order (src/groupies.c:768-786).
    // norm_sd sums in array order (bit-exact) for nodes in (seq_lo,
    // RSG_SEQ_MAX] in the plain form; the batched form sums in parallel
    // (rounding can move a normalised coordinate by one float ulp, rarely:
    // the near-threshold count bounds what that can change)
    const int seq_lo = exact ? RSG_SMALL : RSG_SEQ_MAX;
    const int seq_max = RSG_SEQ_MAX;
    const int T = 256;
    // groups with particles, their working offsets
    std::vector<int64_t> goff, gsz, woff;
    int64_t M = 0;
    for (int64_t g = 0; g < ngroups; g++) {
        if (gsz_h[g] <= 0) continue;
        if (goff_h[g] < 0 || goff_h[g] + gsz_h[g] > num_p) {
            set_error(RSG_ERR_ARGS, "group %lld out of range", (long long)g);
            throw Failure();
        }
        goff.push_back(goff_h[g]);
        gsz.push_back(gsz_h[g]);
        woff.push_back(M);
        M += gsz_h[g];
    }
    int64_t G = (int64_t)goff.size();
    if (G == 0) return out;
    if (M >= (1ll << 31) - 1) {
        set_error(RSG_ERR_ARGS, "find_subs supports up to 2^31-2 particles per call");
        throw Failure();
    }
    DevCfg dc = make_devcfg(cfg);
    DevCfg *d_dc = ar.get<DevCfg>(1);
    RSG_CUDA(cudaMemcpyAsync(d_dc, &dc, sizeof(dc), cudaMemcpyHostToDevice, st));
    int64_t *d_goff = ar.get<int64_t>(G), *d_gsz = ar.get<int64_t>(G), *d_woff = ar.get<int64_t>(G);
    RSG_CUDA(cudaMemcpyAsync(d_goff, goff.data(), 8 * G, cudaMemcpyHostToDevice, st));
    RSG_CUDA(cudaMemcpyAsync(d_gsz, gsz.data(), 8 * G, cudaMemcpyHostToDevice, st));
    RSG_CUDA(cudaMemcpyAsync(d_woff, woff.data(), 8 * G, cudaMemcpyHostToDevice, st));

    // hierarchy node table
    int64_t cap = G + (M / 10) * 2 + 4096;
    HierNodes N;
    N.cap = (int32_t)cap;
    N.start = ar.get<int32_t>(cap); N.n = ar.get<int32_t>(cap); N.parent = ar.get<int32_t>(cap);
    N.group = ar.get<int32_t>(cap); N.level = ar.get<int32_t>(cap); N.nchild = ar.get<int32_t>(cap);
    N.h0 = ar.get<int32_t>(cap); N.h1 = ar.get<int32_t>(cap); N.maxi = ar.get<int32_t>(cap);
    N.ng = ar.get<int32_t>(cap); N.target_r = ar.get<float>(cap);

    Rec *W = ar.get<Rec>(M), *W2 = ar.get<Rec>(M);
    int32_t *wgroup = ar.get<int32_t>(M);
    int32_t *eln = ar.get<int32_t>(M), *eln2 = ar.get<int32_t>(M);
    int32_t *phalo = ar.get<int32_t>(M), *phalo2 = ar.get<int32_t>(M);
    uint64_t *key = ar.get<uint64_t>(M), *key2 = ar.get<uint64_t>(M);
    uint32_t *val = ar.get<uint32_t>(M), *val2 = ar.get<uint32_t>(M);
    int *par = ar.get<int>(M + 1), *root = ar.get<int>(M + 1);
    int32_t *hflag = ar.get<int32_t>(M + 1);
    int *err = ar.get<int>(4);
    RSG_CUDA(cudaMemsetAsync(err, 0, 16, st));
    loop_limit_reset(st);
    unsigned long long *near = ar.get<unsigned long long>(1);
    RSG_CUDA(cudaMemsetAsync(near, 0, sizeof(unsigned long long), st));
    phase_mark(st, "");
    launch(k_make_w, nblk(M, T), T, 0, st, (const rsg_particle *)d_p, G, (const int64_t *)d_goff,
           (const int64_t *)d_woff, M, W, wgroup);
    launch(k_make_nodes, nblk(G, T), T, 0, st, G, (const int64_t *)d_woff, (const int64_t *)d_gsz, N);
    RSG_CHECK_LAUNCH();

    // ---------------- descending ----------------
    std::vector<int32_t> lvl_base{0}, lvl_cnt{(int32_t)G};
    int32_t nn = (int32_t)G;
    int keybits = 32 + 1;
    while ((1ll << (keybits - 32)) <= M) keybits++;
    for (int L = 0;; L++) {
        int32_t base = lvl_base[L], cnt = lvl_cnt[L];
        if (cnt == 0) break;
        if (L > 100000) {
            set_error(RSG_ERR_LIMIT, "subgroup hierarchy too deep");
            throw Failure();
        }
        size_t mark = ar.used;
        // element -> node of this level
        RSG_CUDA(cudaMemsetAsync(eln, 0xff, 4 * M, st));
        launch(k_fill_eln, cnt, T, 0, st, N, base, eln);
        {
            double *sig = ar.get<double>(2 * (int64_t)cnt);
            if (exact)
                launch(k_norm_seq, nblk(cnt, 32), 32, 0, st, W, N, base, cnt, L == 0,
                       cfg.initial_metric_scaling, sig);
            else
                launch(k_norm_warp, nblk(cnt, RSG_NORM_WARPS * 32), RSG_NORM_WARPS * 32, 0, st, W,
                       N, base, cnt, L == 0, cfg.initial_metric_scaling, sig);
            launch(k_norm_blk, cnt, 256, 0, st, W, N, base, L == 0, cfg.initial_metric_scaling, sig,
                   seq_lo, RSG_SEQ_MAX);
            if (exact) {
                launch(k_norm_par, cnt, T, 0, st, W, N, base, L == 0, cfg.initial_metric_scaling,
                       sig, seq_max);
            } else {
                int32_t *nch = ar.get<int32_t>(cnt + 1), *c0 = ar.get<int32_t>(cnt + 1);
                launch(k_nch_count, nblk(cnt + 1, T), T, 0, st, N, base, cnt, tuning().norm_chunk,
                       seq_lo, RSG_SEQ_MAX, nch);
                int32_t nc = excl_scan(ar, (const int32_t *)nch, c0, cnt + 1, st);
                if (nc > 0) {
                    NChunk *C = ar.get<NChunk>(nc);
                    NPart *P = ar.get<NPart>(nc);
                    double *mean = ar.get<double>(6 * (int64_t)cnt);
                    launch(k_nch_fill, nblk(cnt, T), T, 0, st, N, base, cnt, tuning().norm_chunk,
                           (const int32_t *)nch, (const int32_t *)c0, C);
                    launch(k_nch_sum6, nc, 256, 0, st, (const Rec *)W, (const NChunk *)C, P);
                    launch(k_nch_mean, nblk(cnt, T), T, 0, st, N, base, cnt, (const int32_t *)nch,
                           (const int32_t *)c0, (const NPart *)P, mean);
                    launch(k_nch_mom, nc, 256, 0, st, W, (const NChunk *)C, (const double *)mean, P);
                    launch(k_nch_fin, nblk(cnt, T), T, 0, st, N, base, cnt, (const int32_t *)nch,
                           (const int32_t *)c0, (const NPart *)P, L == 0,
                           cfg.initial_metric_scaling, sig);
                }
            }
            launch(k_norm_div_el, nblk(M, T), T, 0, st, W, M, (const int32_t *)eln,
                   (const double *)sig);
            RSG_CHECK_LAUNCH();
        }
        phase_mark(st, "d.norm_sd");
        int32_t *rst = N.start + base, *rn = N.n + base;
        std::vector<int32_t> hs(cnt), hn(cnt);
        RSG_CUDA(cudaMemcpyAsync(hn.data(), rn, 4 * cnt, cudaMemcpyDeviceToHost, st));
        RSG_CUDA(cudaMemcpyAsync(hs.data(), rst, 4 * cnt, cudaMemcpyDeviceToHost, st));
        RSG_CUDA(cudaStreamSynchronize(st));
        int64_t nin = 0;
        std::vector<int32_t> so(cnt);
        int64_t tot = 0;
        for (int k = 0; k < cnt; k++) {
            so[k] = (int32_t)tot;
            int nt = cfg.exact_ll_calc ? hn[k] : (hn[k] < 10000 ? hn[k] : 10000);
            tot += nt;
            nin += hn[k];
        }
        last_stats()[RSG_STAT_6D_ITEMS] += nin;
        last_stats()[RSG_STAT_6D_SAMPLES] += tot;
        // 6D kd-forest over this level's nodes (src/groupies.c:294)
        Forest<6> F = build_forest<6, Rec>(ar, W, M, rst, rn, cnt, nin, 40, st);
        phase_mark(st, "d.tree6d");
        int32_t *soff = ar.get<int32_t>(cnt);
        RSG_CUDA(cudaMemcpyAsync(soff, so.data(), 4 * cnt, cudaMemcpyHostToDevice, st));
        int32_t *sidx = ar.get<int32_t>(tot + 1);
        float *prad = ar.get<float>(tot + 1);
        unsigned *seeds = ar.get<unsigned>(cnt);
        launch(k_sample_seed, nblk(cnt, 64), 64, 0, st, N, base, cnt, seeds,
               (int)cfg.exact_ll_calc);
        launch(k_sample_idx, nblk(tot, 256), 256, 0, st, N, base, cnt, (const int32_t *)soff, sidx,
               (int64_t)tot, (int)cfg.exact_ll_calc);
        {
            // sampled nodes draw positions at random: search them in tree order
            bool sampled = false;
            for (int k = 0; k < cnt && !sampled; k++)
                sampled = !cfg.exact_ll_calc && hn[k] > 10000;
            uint32_t *order = nullptr;
            size_t m0 = ar.used;
            if (sampled) {
                uint64_t *k1 = ar.get<uint64_t>(tot), *k2 = ar.get<uint64_t>(tot);
                uint32_t *v1 = ar.get<uint32_t>(tot);
                order = ar.get<uint32_t>(tot);
                launch(k_nn_keys, nblk(tot, 256), 256, 0, st, N, base, cnt, (const int32_t *)soff,
                       (const int32_t *)sidx, (int64_t)tot, (int)cfg.exact_ll_calc, k1, v1);
                int bits = 33;
                while (bits < 64 && ((int64_t)1 << (bits - 32)) < cnt) bits++;
                sort_pairs(ar, k1, k2, v1, order, tot, bits, st);
            }
            launch(k_nn, nblk(tot, 128), 128, 0, st, F.nodes, W, N, base, cnt, soff, sidx, prad,
                   (int64_t)tot, (int)cfg.exact_ll_calc, err, (const uint32_t *)order);
            ar.used = m0;
        }
        {
            int ntmax = 0;
            for (int32_t k = 0; k < cnt; k++) {
                int nt = cfg.exact_ll_calc ? hn[k] : (hn[k] < 10000 ? hn[k] : 10000);
                if (nt <= RSG_TARGET_SMEM && nt > ntmax) ntmax = nt;
            }
            // both forms: the reference's quickselect with its early exit, whose
            // value can differ from the exact order statistic when the sample
            // holds equal distances (mutual nearest neighbours)
            static bool tgt_attr = false;
            if (!tgt_attr) {
                RSG_CUDA(cudaFuncSetAttribute(k_target_par,
                                              cudaFuncAttributeMaxDynamicSharedMemorySize,
                                              16 * RSG_TARGET_SMEM));
                tgt_attr = true;
            }
            launch(k_target_par, cnt, RSG_TGT_T, (size_t)16 * (ntmax > 0 ? ntmax : 1), st, N,
                   base, (const int32_t *)soff, (const float *)prad, (const unsigned *)seeds,
                   (float)cfg.fof_fraction, (int)cfg.exact_ll_calc);
            launch(k_target, nblk(cnt, 32), 32, 0, st, N, base, cnt, soff, prad, seeds,
                   (float)cfg.fof_fraction, (int)cfg.exact_ll_calc);
        }
        phase_mark(st, "d.nn_target");
        // subgroup labels: the reference's union-find labels (uflabels.cuh),
        // then its partition sort by label (lsort.cuh)
        {
            // later neighbours within target_r, as CSR lists
            int32_t *ncnt = par, *noff = root;
            RSG_CUDA(cudaMemsetAsync(ncnt, 0, 4 * (M + 1), st));
            int32_t *slots = ar.get<int32_t>((size_t)M * RSG_SLOT6);
            // overflow chunks: room for half a slot's worth per particle
            Chains CH;
            CH.cap = (int32_t)std::min<int64_t>(M / 2 + 1024, INT32_MAX / RSG_SLOT6);
            CH.pool = ar.get<int32_t>((size_t)CH.cap * RSG_SLOT6);
            CH.next = ar.get<int32_t>(CH.cap);
            CH.head = ar.get<int32_t>(M);
            CH.redo = ar.get<int32_t>(M);
            CH.cursor = ar.get<unsigned>(1);
            RSG_CUDA(cudaMemsetAsync(CH.cursor, 0, sizeof(unsigned), st));
            launch(k_fof6_w<2>, nblk(M, 128), 128, 0, st, F.nodes, W, M, N, base, eln,
                   (const int32_t *)nullptr, ncnt, slots, CH, err, near);
            check_i32_total(ar, ncnt, M + 1, "6D neighbour lists", st);
            int32_t ne = excl_scan(ar, ncnt, noff, (int32_t)(M + 1), st);
            int32_t *nbr = ar.get<int32_t>(ne + 1);
            launch(k_slots_csr, nblk(M, 256), 256, 0, st, eln, M, (const int32_t *)ncnt,
                   (const int32_t *)noff, (const int32_t *)slots, CH, nbr);
            // lists the pool could not hold (none unless it ran out): searched again
            launch(k_fof6_w<1>, nblk(M, 128), 128, 0, st, F.nodes, W, M, N, base, eln,
                   (const int32_t *)noff, ncnt, nbr, CH, err, near);
            phase_mark(st, "d.fof6d");
            exact_labels_csr(ar, M, eln, N.start + base, noff, nbr, phalo, st);
        }
        RSG_CHECK_LAUNCH();
        phase_mark(st, "d.labels");
        partition_sort_labels<Rec>(ar, W, phalo, M, hs, hn, st);
        phase_mark(st, "d.psort");
        launch(k_run_heads, nblk(M, T), T, 0, st, eln, M, N, base, phalo, hflag);
        int32_t *heads = ar.get<int32_t>(M);
        int32_t nh = select_flagged(ar, hflag, heads, M, 0, st);
        int32_t *cflag = ar.get<int32_t>(nh + 1), *clen = ar.get<int32_t>(nh + 1);
        int32_t *cidx = ar.get<int32_t>(nh + 1);
        int32_t nc = 0;
        if (nh) {
            launch(k_run_children, nblk(nh, T), T, 0, st, heads, nh, eln, N, base, phalo,
                                                      cfg.min_halo_particles, cflag, clen);
            nc = select_flagged(ar, cflag, cidx, nh, 0, st);
        }
        if (nn + (int64_t)nc > cap) {
            set_error(RSG_ERR_LIMIT, "subgroup node capacity exceeded");
            throw Failure();
        }
        if (nc) launch(k_make_children2, nblk(nc, T), T, 0, st, cidx, nc, heads, clen, eln, N, base, nn);
        RSG_CHECK_LAUNCH();
        ar.used = mark;
        lvl_base.push_back(nn);
        lvl_cnt.push_back(nc);
        nn += nc;
        phase_mark(st, "d.children");
    }
    int nlev = (int)lvl_base.size() - 1;  // the last entry has count 0
    {
        g_dbg_level.resize(nn);
        g_dbg_start.resize(nn);
        g_dbg_n.resize(nn);
        g_dbg_target.resize(nn);
        RSG_CUDA(cudaMemcpyAsync(g_dbg_level.data(), N.level, 4 * nn, cudaMemcpyDeviceToHost, st));
        RSG_CUDA(cudaMemcpyAsync(g_dbg_start.data(), N.start, 4 * nn, cudaMemcpyDeviceToHost, st));
        RSG_CUDA(cudaMemcpyAsync(g_dbg_n.data(), N.n, 4 * nn, cudaMemcpyDeviceToHost, st));
        RSG_CUDA(cudaMemcpyAsync(g_dbg_target.data(), N.target_r, 4 * nn, cudaMemcpyDeviceToHost, st));
        RSG_CUDA(cudaStreamSynchronize(st));
    }

    // ---------------- halos ----------------
    int32_t *nflag = ar.get<int32_t>(nn), *leaves = ar.get<int32_t>(nn);
    launch(k_leaf_flags, nblk(nn, T), T, 0, st, N, nn, nflag);
    int32_t NH = select_flagged(ar, nflag, leaves, nn, 0, st);
    if (NH > max_halos) {
        set_error(RSG_ERR_ARGS, "%d halos exceed max_halos %lld", NH, (long long)max_halos);
        throw Failure();
    }
    {
        int32_t *lk = ar.get<int32_t>(NH), *lk2 = ar.get<int32_t>(NH), *lv2 = ar.get<int32_t>(NH);
        launch(k_leaf_keys, nblk(NH, T), T, 0, st, N, leaves, NH, lk);
        sort_pairs(ar, lk, lk2, leaves, lv2, NH, 32, st);
        RSG_CUDA(cudaMemcpyAsync(leaves, lv2, 4 * NH, cudaMemcpyDeviceToDevice, st));
        launch(k_halo_ranges, nblk(nn, T), T, 0, st, N, nn, lk2, NH);
    }
    rsg_halo *H = d_halos;
    rsg_extra_halo_info *E = d_extra;
    launch(k_halo_init, nblk(NH, T), T, 0, st, H, E, NH);
    int32_t *glist = ar.get<int32_t>(NH), *redirect = ar.get<int32_t>(NH);
    // bucket b (32 halos) and super-bucket sb (1024 halos) of a node at h0 + b, h0 + sb
    AscBucket *ascb = ar.get<AscBucket>(NH), *ascb2 = ar.get<AscBucket>(NH);
    AscHalo *asch = ar.get<AscHalo>(NH);
    int2 *ascgi = ar.get<int2>(NH);
    int32_t *stk = ar.get<int32_t>(NH + 1);
    RSG_CHECK_LAUNCH();

    phase_mark(st, "halos");
    // ---------------- ascending ----------------
    for (int L = nlev - 1; L >= 0; L--) {
        int32_t base = lvl_base[L], cnt = lvl_cnt[L];
        if (cnt == 0) continue;
        size_t mark = ar.used;
        RSG_CUDA(cudaMemsetAsync(eln, 0xff, 4 * M, st));
        launch(k_fill_eln, cnt, T, 0, st, N, base, eln);
        launch(k_asc_restore, nblk(M, T), T, 0, st, W, d_p, (const int32_t *)eln, M, phalo);
        launch(k_asc_halo_mark, dim3(cnt, 8), T, 0, st, N, base, (const rsg_halo *)H, phalo);
        phase_mark(st, "a.mark");
        launch(k_asc_seed_blk, cnt, 256, 0, st, N, base, H, E, glist, redirect, cfg.force_res);
        asc_sorted(ar, N, base, cnt, H, glist, 0, NH, asch, ascgi, ascb, ascb2, st);
        launch(k_asc_assign_p, nblk(M, 128), 128, 0, st, (const Rec *)W, M, (const int32_t *)eln,
               N, base, (const rsg_halo *)H, (const rsg_extra_halo_info *)E,
               (const int32_t *)glist, (const int32_t *)redirect, (const AscBucket *)ascb,
               (const AscBucket *)ascb2, (const AscHalo *)asch, (const int2 *)ascgi,
               tuning().asc_bucket_min, phalo);
        phase_mark(st, "a.seed_assign");
        RSG_CHECK_LAUNCH();
        if (exact) {
            // reassign_halo_particles: the reference's partition by halo index
            std::vector<int32_t> hs(cnt), hn(cnt);
            RSG_CUDA(cudaMemcpyAsync(hn.data(), N.n + base, 4 * cnt, cudaMemcpyDeviceToHost, st));
            RSG_CUDA(cudaMemcpyAsync(hs.data(), N.start + base, 4 * cnt, cudaMemcpyDeviceToHost, st));
            RSG_CUDA(cudaStreamSynchronize(st));
            partition_sort_labels<Rec>(ar, W, phalo, M, hs, hn, st);
        } else {
            label_sort_stable(ar, W, phalo, eln, N, base, cnt, M, st);
        }
        phase_mark(st, "a.reassign");
        launch(k_halo_heads, nblk(M, T), T, 0, st, eln, M, N, base, phalo, H);
        launch(k_halo_tails, nblk(M, T), T, 0, st, eln, M, N, base, phalo, H);
        // growing list of the level
        int32_t *goffs = ar.get<int32_t>(cnt + 1);
        launch(k_ng, nblk(cnt + 1, T), T, 0, st, N, base, cnt, goffs, 0);
        int32_t ngr = excl_scan(ar, goffs, goffs, cnt + 1, st);
        int32_t *glv = ar.get<int32_t>(ngr + 1), *gnode = ar.get<int32_t>(ngr + 1);
        launch(k_list_growing, cnt, T, 0, st, N, base, goffs, glist, glv, gnode);
        basic_props(ar, W, H, glv, ngr, d_dc, seq_max, exact, st);
        launch(k_maxi, cnt, 256, 0, st, N, base, (const rsg_halo *)H, glist, 0);
        asc_sorted(ar, N, base, cnt, H, glist, 0, NH, asch, ascgi, ascb, ascb2, st);
        launch(k_best_parent, nblk(ngr, T), T, 0, st, N, base, cnt, goffs, glv, gnode, H, E,
               (const AscBucket *)ascb, (const AscBucket *)ascb2, (const AscHalo *)asch,
               (const int2 *)ascgi, tuning().asc_bucket_min);
        fix_parents_level(ar, N, base, cnt, H, E, err, true, st);
        basic_props(ar, W, H, glv, ngr, d_dc, seq_max, exact, st);
        RSG_CHECK_LAUNCH();
        phase_mark(st, "a.props_parents");
        if (L == 0) {
            int32_t *aoff = ar.get<int32_t>(cnt + 1);
            launch(k_ng, nblk(cnt + 1, T), T, 0, st, N, base, cnt, aoff, 1);
            int32_t na = excl_scan(ar, aoff, aoff, cnt + 1, st);
            int32_t *alist = ar.get<int32_t>(na + 1), *anode = ar.get<int32_t>(na + 1);
            launch(k_list_all, nblk(cnt, T), T, 0, st, N, base, cnt, aoff, alist);
            launch(k_list_node, nblk(cnt, T), T, 0, st, cnt, aoff, anode);
            basic_props(ar, W, H, alist, na, d_dc, seq_max, exact, st);
            launch(k_corekeys, nblk(M, T), T, 0, st, W, eln, M, phalo, H, key, val);
            sort_pairs(ar, key, key2, val, val2, M, keybits, st);
            launch(k_gather<Rec>, nblk(M, T), T, 0, st, W, val2, M, W2);
            launch(k_gather<int32_t>, nblk(M, T), T, 0, st, phalo, val2, M, phalo2);
            std::swap(W, W2);
            std::swap(phalo, phalo2);
            launch(k_maxi, cnt, 256, 0, st, N, base, (const rsg_halo *)H, glist, 1);
            asc_sorted(ar, N, base, cnt, H, glist, 1, NH, asch, ascgi, ascb, ascb2, st);
            launch(k_best_parent, nblk(na, T), T, 0, st, N, base, cnt, aoff, alist, anode, H, E,
                   (const AscBucket *)ascb, (const AscBucket *)ascb2, (const AscHalo *)asch,
                   (const int2 *)ascgi, tuning().asc_bucket_min);
            fix_parents_level(ar, N, base, cnt, H, E, err, true, st);
            RSG_CHECK_LAUNCH();
            // find_subs tail (src/groupies.c:697-703): child counts and basic
            // properties for every halo, then the additional properties.
            fix_parents_level(ar, N, base, cnt, H, E, err, false, st);
            basic_props(ar, W, H, alist, na, d_dc, seq_max, exact, st);
            RSG_CHECK_LAUNCH();
        }
        ar.used = mark;
    }
    phase_mark(st, "a.level0");
    additional_props(ar, dc, d_dc, W, M, H, E, NH, st, exact);

    // outputs
    int32_t *hgrp = ar.get<int32_t>(NH + 1);
    launch(k_halo_group, nblk(NH, T), T, 0, st, N, leaves, NH, hgrp);
    launch(k_halo_out, nblk(NH, T), T, 0, st, H, E, NH, hgrp, d_goff, d_woff);
    rsg_particle *Pcopy = ar.get<rsg_particle>(num_p);
    RSG_CUDA(cudaMemcpyAsync(Pcopy, d_p, sizeof(rsg_particle) * num_p, cudaMemcpyDeviceToDevice, st));
    launch(k_write_back, nblk(M, T), T, 0, st, W, M, wgroup, d_goff, d_woff, Pcopy, d_p);
    RSG_CHECK_LAUNCH();
    int herr[4];
    unsigned long long hnear = 0;
    RSG_CUDA(cudaMemcpyAsync(herr, err, 16, cudaMemcpyDeviceToHost, st));
    RSG_CUDA(cudaMemcpyAsync(&hnear, near, sizeof(hnear), cudaMemcpyDeviceToHost, st));
    RSG_CUDA(cudaStreamSynchronize(st));
    if (herr[0]) {
        set_error(RSG_ERR_LIMIT, "6D kd-tree traversal stack overflow");
        throw Failure();
    }
    loop_limit_check(st, "find_subs");
    last_stats()[RSG_STAT_NEAR_6D] = (int64_t)hnear;
    out.nhalos = NH;
    return out;
}

}  // namespace rsg
