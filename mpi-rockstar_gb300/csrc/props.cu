// Halo properties after the hierarchy is settled: calc_additional_halo_props
// (src/properties.c:513-556) for every halo of the call at once.
//
//  1. particle sets: the halo, its children (recursively) and, when the host
//     is not much larger, the host's particles as potential-only sources
//     (calc_particle_radii, src/groupies.c:212-270);
//  2. potentials: the reference's Barnes-Hut code reproduced on the GPU -- a
//     forest of kd-trees (10 points per leaf, exact fast3tree permutation),
//     mass centres and opening radii bottom-up, and one half-warp per leaf
//     walking the tree in the reference's order so every FP64 sum matches
//     (src/potential.c:22-192);
//  3. potential-only particles dropped, the rest sorted by r^2;
//  4. core velocity, kinetic energy, then the density/shape/NFW scans for
//     all particles and for bound particles (src/properties.c:165-510).
#include <atomic>
#include <vector>

#include <cub/cub.cuh>

#include "halo_math.cuh"
#include "kdtree_impl.cuh"

namespace rsg {

struct Seg {
    int32_t src, n, dst, halo;
    int32_t pot_only, flag;
};

struct Frame {
    int32_t x, child, stage, pot;
};

// calc_particle_radii as an explicit depth-first walk; emit(x, pot_only)
// for every visited halo in the reference's order.  The loop guard of
// src/groupies.c:241-247 checks the halos on the current path.
template <class F>
__device__ bool walk_sets(const rsg_halo *H, const rsg_extra_halo_info *E, int base,
                          double ratio, F emit) {
    Frame st[64];
    int sp = 0;
    st[sp++] = Frame{base, -1, 0, 0};
    int guard = 0;
    while (sp) {
        if (++guard > 10000000) return false;
        Frame &f = st[sp - 1];
        if (f.stage == 0) {
            bool loop = false;
            for (int j = 0; j < sp - 1; j++)
                if (st[j].x == f.x) loop = true;
            if (loop) {
                sp--;
                continue;
            }
            emit(f.x, f.pot);
            f.child = (int32_t)E[f.x].child;
            f.stage = 1;
        }
        if (f.stage == 1) {
            if (f.child > -1) {
                int c = f.child;
                f.child = (int32_t)E[c].next_cochild;
                if (sp >= 64) return false;
                st[sp++] = Frame{c, -1, 0, f.pot};
                continue;
            }
            f.stage = 2;
            if (sp == 1) {
                int64_t par = E[f.x].sub_of;
                if (par > -1 &&
                    ((double)H[par].num_child_particles * ratio < (double)H[f.x].num_child_particles)) {
                    st[sp++] = Frame{(int32_t)par, -1, 0, 1};
                    continue;
                }
            }
        }
        sp--;
    }
    return true;
}

// Per halo: records of its potential set (tot), the records of its own
// halos that stay after the potential-only ones are dropped (kept), and the
// copy segments (nseg: one per set member and segmax records).
__global__ void k_set_count(const rsg_halo *H, const rsg_extra_halo_info *E, int32_t NH,
                            double ratio, int segmax, int32_t *tot, int32_t *nseg, int32_t *kept,
                            int *err) {
    int h = blockIdx.x * blockDim.x + threadIdx.x;
    if (h > NH) return;
    if (h == NH) {
        tot[h] = 0;
        nseg[h] = 0;
        kept[h] = 0;
        return;
    }
    int t = 0, s = 0, kp = 0;
    if (H[h].num_p >= 1) {
        bool ok = walk_sets(H, E, h, ratio, [&](int x, int pot) {
            int n = (int)H[x].num_p;
            t += n;
            if (!pot) kp += n;
            s += n > 0 ? (n + segmax - 1) / segmax : 1;
        });
        if (!ok) atomicExch(err, 1);
    }
    tot[h] = t;
    nseg[h] = s;
    kept[h] = kp;
}

__global__ void k_set_segs(const rsg_halo *H, const rsg_extra_halo_info *E, int32_t NH,
                           double ratio, int segmax, const int32_t *toff, const int32_t *soff,
                           Seg *segs) {
    int h = blockIdx.x * blockDim.x + threadIdx.x;
    if (h >= NH || H[h].num_p < 1) return;
    int dst = toff[h], k = soff[h];
    int64_t bnp = H[h].num_p;
    walk_sets(H, E, h, ratio, [&](int x, int pot) {
        int flag = 0;
        if (x == h) flag = 1;
        if (!pot && ((double)H[x].num_p < (double)bnp * 0.03)) flag = 2;
        int n = (int)H[x].num_p, src = (int32_t)H[x].p_start;
        if (n <= 0) segs[k++] = Seg{src, n, dst, h, pot, flag};
        for (int o = 0; o < n; o += segmax)
            segs[k++] = Seg{src + o, min(segmax, n - o), dst + o, h, pot, flag};
        dst += n;
    });
}

// _reset_potentials (src/groupies.c:212-233)
__global__ void k_set_fill(const Seg *segs, const Rec *W, const rsg_halo *H, PotRec *PO) {
    Seg sg = segs[blockIdx.x];
    float c0 = H[sg.halo].pos[0], c1 = H[sg.halo].pos[1], c2 = H[sg.halo].pos[2];
    for (int i = threadIdx.x; i < sg.n; i += blockDim.x) {
        const Rec &q = W[sg.src + i];
        PotRec r;
#pragma unroll
        for (int d = 0; d < 6; d++) r.pos[d] = q.pos[d];
        float dx, r2 = 0.f;
        dx = fsub(q.pos[0], c0); r2 = fadd(r2, fmul(dx, dx));
        dx = fsub(q.pos[1], c1); r2 = fadd(r2, fmul(dx, dx));
        dx = fsub(q.pos[2], c2); r2 = fadd(r2, fmul(dx, dx));
        r.r2 = r2;
        r.pad = __int_as_float(sg.halo);
        r.pe = 0;
        r.ke = sg.pot_only ? -1.f : 0.f;
        r.flags = sg.flag;
        PO[sg.dst + i] = r;
    }
}

// ---- Barnes-Hut ---------------------------------------------------------
__device__ __forceinline__ double d2d(const float *a, const float *b) {
    double r2 = 0;
#pragma unroll
    for (int k = 0; k < 3; k++) {
        double dx = (double)fsub(a[k], b[k]);
        r2 = dadd(r2, dmul(dx, dx));
    }
    return r2;
}

// Internal potential-tree nodes above this size are reduced by a block.
#define RSG_BH_BIG 4096

struct BHNode {
    float mc[3], m, dmin;
};

// src/potential.c:71-82 over the node's points
__device__ float node_dmin(const PotRec *PO, int s, int n, const float *mc) {
    double sx = 0, bm = 0;
    for (int i = 0; i < n; i++) {
        double dx = d2d(mc, PO[s + i].pos);
        if (bm < dx) bm = dx;
        sx += dx;
    }
    bm = sqrt(bm) / 2.0;
    return (float)(bm + sqrt(bm * bm + sx / (n * 1.0)));
}

// leaves: mass and mass centre from their points (src/potential.c:101-113)
__global__ void k_bh_leaf(const KNode<3> *nodes, int32_t nn, const PotRec *PO, double mp,
                          BHNode *B) {
    int a = blockIdx.x * blockDim.x + threadIdx.x;
    if (a >= nn) return;
    const KNode<3> &x = nodes[a];
    if (x.div >= 0) return;
    double pos[3] = {0, 0, 0};
    for (int i = 0; i < x.n; i++)
        for (int j = 0; j < 3; j++) pos[j] += (double)PO[x.start + i].pos[j];
    BHNode b;
    b.m = (float)(mp * x.n);
    for (int j = 0; j < 3; j++) b.mc[j] = pos[j] ? (float)(pos[j] / (double)x.n) : 0.f;
    b.dmin = node_dmin(PO, x.start, x.n, b.mc);
    B[a] = b;
}
// internal nodes of one build level (src/potential.c:115-123)
__global__ void k_bh_internal(const KNode<3> *nodes, int32_t first, int32_t count,
                              const PotRec *PO, BHNode *B) {
    int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= count) return;
    int a = first + k;
    const KNode<3> &x = nodes[a];
    if (x.div < 0 || x.n > RSG_BH_BIG) return;
    const BHNode &L = B[x.left], &R = B[x.left + 1];
    BHNode b;
    b.m = fadd(L.m, R.m);
    for (int j = 0; j < 3; j++)
        b.mc[j] = b.m ? __fdiv_rn(fadd(fmul(R.mc[j], R.m), fmul(L.mc[j], L.m)), b.m) : 0.f;
    b.dmin = node_dmin(PO, x.start, x.n, b.mc);
    B[a] = b;
}

// Batched form: one warp per internal node of at most RSG_BH_BIG points,
// the sum of squared distances reduced by shuffles.
__global__ void k_bh_internal_warp(const KNode<3> *nodes, int32_t first, int32_t count,
                                   const PotRec *PO, BHNode *B) {
    int k = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
    if (k >= count) return;
    int a = first + k;
    const KNode<3> &x = nodes[a];
    if (x.div < 0 || x.n > RSG_BH_BIG) return;
    const BHNode &L = B[x.left], &R = B[x.left + 1];
    BHNode b;
    b.m = fadd(L.m, R.m);
    for (int j = 0; j < 3; j++)
        b.mc[j] = b.m ? __fdiv_rn(fadd(fmul(R.mc[j], R.m), fmul(L.mc[j], L.m)), b.m) : 0.f;
    double sx = 0, bm = 0;
    for (int i = lane; i < x.n; i += 32) {
        double dx = d2d(b.mc, PO[x.start + i].pos);
        if (bm < dx) bm = dx;
        sx += dx;
    }
    for (int o = 16; o; o >>= 1) {
        sx += __shfl_xor_sync(0xffffffffu, sx, o);
        bm = fmax(bm, __shfl_xor_sync(0xffffffffu, bm, o));
    }
    if (lane == 0) {
        bm = sqrt(bm) / 2.0;
        b.dmin = (float)(bm + sqrt(bm * bm + sx / (x.n * 1.0)));
        B[a] = b;
    }
}

// Batched form, internal nodes of more than Tuning::bh_huge points: one
// block per chunk of `chunk` points forms the chunk's sum and maximum of
// squared distances to the node's mass centre (part[item]); one thread per
// node adds the chunks in order.  item = (node, chunk); the chunks of node j
// of a level are items first[j] .. first[j + 1].
__device__ __forceinline__ BHNode bh_merge(const BHNode &L, const BHNode &R) {
    BHNode b;
    b.m = fadd(L.m, R.m);
    for (int j = 0; j < 3; j++)
        b.mc[j] = b.m ? __fdiv_rn(fadd(fmul(R.mc[j], R.m), fmul(L.mc[j], L.m)), b.m) : 0.f;
    return b;
}
__global__ void __launch_bounds__(256) k_bh_huge_part(const KNode<3> *nodes, const int2 *item,
                                                      int chunk, const PotRec *PO,
                                                      const BHNode *B, double2 *part) {
    __shared__ double s_s[8], m_s[8];
    const int2 it = item[blockIdx.x];
    const KNode<3> &x = nodes[it.x];
    const BHNode b = bh_merge(B[x.left], B[x.left + 1]);
    const int i0 = it.y * chunk, i1 = min(x.n, i0 + chunk);
    double sx = 0, bm = 0;
    for (int i = i0 + threadIdx.x; i < i1; i += 256) {
        double dx = d2d(b.mc, PO[x.start + i].pos);
        if (bm < dx) bm = dx;
        sx += dx;
    }
    for (int o = 16; o; o >>= 1) {
        sx += __shfl_down_sync(0xffffffffu, sx, o);
        bm = fmax(bm, __shfl_down_sync(0xffffffffu, bm, o));
    }
    if ((threadIdx.x & 31) == 0) {
        s_s[threadIdx.x >> 5] = sx;
        m_s[threadIdx.x >> 5] = bm;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        for (int w = 1; w < 8; w++) {
            sx += s_s[w];
            bm = fmax(bm, m_s[w]);
        }
        part[blockIdx.x] = make_double2(sx, bm);
    }
}
__global__ void k_bh_huge_fin(const KNode<3> *nodes, const int32_t *node, const int32_t *first,
                              int32_t nn, const double2 *part, BHNode *B) {
    int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= nn) return;
    int a = node[j];
    const KNode<3> &x = nodes[a];
    BHNode b = bh_merge(B[x.left], B[x.left + 1]);
    double sx = 0, bm = 0;
    for (int c = first[j]; c < first[j + 1]; c++) {
        sx += part[c].x;
        bm = fmax(bm, part[c].y);
    }
    bm = sqrt(bm) / 2.0;
    b.dmin = (float)(bm + sqrt(bm * bm + sx / (x.n * 1.0)));
    B[a] = b;
}
__global__ void k_bh_huge_flags(const KNode<3> *nodes, int32_t nn, int huge, int32_t *f) {
    int a = blockIdx.x * blockDim.x + threadIdx.x;
    if (a < nn) f[a] = nodes[a].div >= 0 && nodes[a].n > huge;
}
__global__ void k_bh_huge_sizes(const KNode<3> *nodes, const int32_t *node, int32_t nn,
                                int32_t *n) {
    int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j < nn) n[j] = nodes[node[j]].n;
}

// Large internal nodes: the block computes every point's squared distance
// to the mass centre; the maximum is a reduction and the sum is added by one
// thread in point order, as _compute_dmin does.
__global__ void __launch_bounds__(256) k_bh_internal_big(const KNode<3> *nodes, int32_t first,
                                                         int32_t count, const PotRec *PO, BHNode *B,
                                                         int exact, int huge) {
    __shared__ double dx_s[256];
    __shared__ BHNode bs;
    __shared__ double mx_s[8];
    int a = first + blockIdx.x;
    const KNode<3> &x = nodes[a];
    if (x.div < 0 || x.n <= RSG_BH_BIG) return;
    if (!exact && x.n > huge) return;  // k_bh_huge_*
    if (threadIdx.x == 0) {
        const BHNode &L = B[x.left], &R = B[x.left + 1];
        bs.m = fadd(L.m, R.m);
        for (int j = 0; j < 3; j++)
            bs.mc[j] = bs.m ? __fdiv_rn(fadd(fmul(R.mc[j], R.m), fmul(L.mc[j], L.m)), bs.m) : 0.f;
    }
    __syncthreads();
    double sx = 0, bm = 0;
    for (int b0 = 0; b0 < x.n; b0 += 256) {
        int i = b0 + threadIdx.x;
        double dx = 0;
        if (i < x.n) {
            dx = d2d(bs.mc, PO[x.start + i].pos);
            if (bm < dx) bm = dx;
        }
        if (!exact) {
            sx += dx;
            continue;
        }
        dx_s[threadIdx.x] = dx;
        __syncthreads();
        if (threadIdx.x == 0) {
            int m = min(256, x.n - b0);
            for (int t = 0; t < m; t++) sx += dx_s[t];
        }
        __syncthreads();
    }
    if (!exact) {
        for (int o = 16; o; o >>= 1) sx += __shfl_down_sync(0xffffffffu, sx, o);
        __syncthreads();
        if ((threadIdx.x & 31) == 0) dx_s[threadIdx.x >> 5] = sx;
        __syncthreads();
        if (threadIdx.x == 0) {
            sx = 0;
            for (int w = 0; w < 8; w++) sx += dx_s[w];
        }
        __syncthreads();
    }
    for (int o = 16; o; o >>= 1) bm = fmax(bm, __shfl_down_sync(0xffffffffu, bm, o));
    if ((threadIdx.x & 31) == 0) mx_s[threadIdx.x >> 5] = bm;
    __syncthreads();
    if (threadIdx.x == 0) {
        for (int w = 1; w < 8; w++) bm = fmax(bm, mx_s[w]);
        bm = sqrt(bm) / 2.0;
        BHNode b = bs;
        b.dmin = (float)(bm + sqrt(bm * bm + sx / (x.n * 1.0)));
        B[a] = b;
    }
}

// _compute_monopole_potentials(leaf, root) (src/potential.c:133-168): one
// half-warp per leaf walks the tree from the root, each lane holding one of
// the leaf's particles (leaves hold at most 10 but for duplicates; larger
// ones repeat the walk per 16).  The opening decisions belong to the leaf,
// so the walk is the same for every lane of the half-warp, which shares one
// stack in shared memory; the two halves of a warp walk two leaves.  A particle's
// potential receives the same terms in the same order as in the reference
// (the self leaf's pairs in ascending partner order, opened leaves in point
// order, monopoles as visited), so the FP64 form is bit-identical to it.
//   MODE 0: r = max(sqrt(r2), FORCE_RES) and m / r in FP64, as the
//           reference computes them;
//   MODE 1: the batched precision form: squared distance and 1/r in FP32
//           (rsqrtf), each particle's sum Kahan-compensated in FP32;
//   MODE 2: the MODE 1 terms summed in plain FP32 (no compensation), the
//           uncompensated baseline of the precision study.
// The opening decisions are the same in every mode.
#define RSG_BH_WPB 8  // warps per block (16 leaves)
template <int MODE>
__global__ void __launch_bounds__(32 * RSG_BH_WPB) k_bh_walk(const KNode<3> *nodes,
                                                             const int32_t *leaves, int32_t nl,
                                                             const BHNode *B, PotRec *PO,
                                                             double mp, double force_res,
                                                             int *err) {
    __shared__ int stk[2 * RSG_BH_WPB][RSG_STACK];
    constexpr bool F32 = MODE != 0;
    const int w = threadIdx.x >> 4, lane = threadIdx.x & 15;
    const unsigned hm = (threadIdx.x & 16) ? 0xffff0000u : 0x0000ffffu;  // this half-warp
    const int t = blockIdx.x * 2 * RSG_BH_WPB + w;
    if (t >= nl) return;  // whole half-warps
    const int a = leaves[t];
    const KNode<3> n = nodes[a];
    const BHNode bn = B[a];
    const float mpf = (float)mp, fr2f = (float)(force_res * force_res);
    int *st = stk[w];
    for (int p0 = 0; p0 < n.n; p0 += 16) {
        const int p = p0 + lane;
        const bool act = p < n.n;
        float px[3] = {0.f, 0.f, 0.f};
        double acc = 0;
        float s = 0.f, c = 0.f;
        if (act) {
            const PotRec &r = PO[n.start + p];
            px[0] = r.pos[0];
            px[1] = r.pos[1];
            px[2] = r.pos[2];
            acc = r.pe;
        }
        // adds one term to this lane's sum
        auto add = [&](double term64, float term32) {
            if (MODE == 1) {
                float y = term32 - c;
                float tt = s + y;
                c = (tt - s) - y;
                s = tt;
            } else if (MODE == 2) {
                s += term32;
            } else {
                acc += term64;
            }
        };
        // direct pair with point q (softened)
        auto pair = [&](const float *q) {
            if (F32) {
                float dx = px[0] - q[0], dy = px[1] - q[1], dz = px[2] - q[2];
                float r2 = __fmaf_rn(dz, dz, __fmaf_rn(dy, dy, dx * dx));
                add(0.0, mpf * rsqrtf(fmaxf(r2, fr2f)));
            } else {
                double r = sqrt(d2d(px, q));
                if (r < force_res) r = force_res;
                add(mp * (1.0 / r), 0.f);
            }
        };
        __syncwarp(hm);
        if (lane == 0) st[0] = n.tree;
        int sp = 1;
        __syncwarp(hm);
        while (sp) {
            const int b = st[--sp];
            __syncwarp(hm);  // every lane has read before lane 0 pushes over the slot
            const KNode<3> &n2 = nodes[b];
            if (b == a) {
                if (n.n > 20) continue;  // degenerate leaf
                for (int qi = 0; qi < n.n; qi++) {
                    const float *qp = PO[n.start + qi].pos;
                    float q[3] = {qp[0], qp[1], qp[2]};
                    if (act && p != qi) pair(q);
                }
                continue;
            }
            int i;
            for (i = 0; i < 3; i++)
                if (n.mn[i] < n2.mn[i] || n.mx[i] > n2.mx[i]) break;
            bool open = (i == 3);
            if (!open) {
                const float dm2 = fmul(B[b].dmin, B[b].dmin);
                int dec = -1;  // 0: keep the monopole, 1: open
                if (MODE != 0) {
                    // The reference's r^2 is (float) of FP64 sums of the float
                    // differences' squares.  An FP32 sum of the same squares is
                    // within 2.4e-7 of it (relative); outside a 2e-6 band around
                    // dmin^2 the FP32 value decides the same way, inside it the
                    // FP64 sum decides (GB300's FP64 pipe is narrow).
                    float dx = fsub(bn.mc[0], B[b].mc[0]), dy = fsub(bn.mc[1], B[b].mc[1]),
                          dz = fsub(bn.mc[2], B[b].mc[2]);
                    float sf = __fmaf_rn(dz, dz, __fmaf_rn(dy, dy, fmul(dx, dx)));
                    if (sf > 1e-30f && sf < 1e30f && dm2 > 1e-30f && dm2 < 1e30f) {
                        if (sf > fmul(dm2, 1.000002f)) dec = 0;
                        else if (sf < fmul(dm2, 0.999998f)) dec = 1;
                    }
                }
                if (dec < 0) {
                    float r2 = (float)d2d(bn.mc, B[b].mc);
                    open = !(r2 > dm2);
                } else {
                    open = dec == 1;
                }
            }
            if (open) {
                if (n2.div < 0) {
                    for (int qi = 0; qi < n2.n; qi++) {
                        const float *qp = PO[n2.start + qi].pos;
                        float q[3] = {qp[0], qp[1], qp[2]};
                        if (act) pair(q);
                    }
                } else {
                    if (sp + 2 > RSG_STACK) {
                        if (lane == 0) atomicExch(err, 1);
                        return;
                    }
                    if (lane == 0) {
                        st[sp] = n2.left + 1;
                        st[sp + 1] = n2.left;
                    }
                    sp += 2;
                    __syncwarp(hm);
                }
            } else if (act) {
                const BHNode &m = B[b];
                if (F32) {
                    float dx = px[0] - m.mc[0], dy = px[1] - m.mc[1], dz = px[2] - m.mc[2];
                    float r2 = __fmaf_rn(dz, dz, __fmaf_rn(dy, dy, dx * dx));
                    add(0.0, m.m * rsqrtf(r2));
                } else {
                    float r = (float)sqrt(d2d(px, m.mc));
                    add((double)__fdiv_rn(m.m, r), 0.f);
                }
            }
        }
        if (act) PO[n.start + p].pe = F32 ? acc + ((double)s - (double)c) : acc;
    }
}

// ---- sort keys: drop potential-only records, order by r^2 ----------------
__global__ void k_po_keys(const PotRec *PO, int64_t n, uint64_t *key, uint32_t *val) {
    int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= n) return;
    const PotRec &r = PO[i];
    uint64_t h = (uint64_t)__float_as_int(r.pad);
    uint64_t drop = r.ke < 0 ? 1 : 0;
    key[i] = (h << 33) | (drop << 32) | (uint64_t)f2ord(r.r2);
    val[i] = (uint32_t)i;
}
__global__ void k_po_gather(const PotRec *src, const uint32_t *perm, int64_t n, PotRec *dst) {
    int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i < n) dst[i] = src[perm[i]];
}

// ---- per-halo scans (src/properties.c:165-510) ---------------------------
// calculate_corevel
__device__ void corevel(rsg_halo &h, const PotRec *q, int64_t tot, const DevCfg &C) {
    double vel[3] = {0, 0, 0}, var[3] = {0, 0, 0}, tv, bv = 0;
    double rt = C.rvir_dens * (4.0 * M_PI / 3.0);
    int64_t j, cmax, rmax;
    for (j = tot - 1; j >= 0; j--) {
        float r2 = q[j].r2;
        if ((double)(j * j) > (double)fmul(fmul(r2, r2), r2) * (rt * rt)) break;
    }
    rmax = j;
    if (rmax < 1) return;
    for (j = tot - 1; j >= 0; j--)
        if ((double)q[j].r2 * 100.0 < (double)q[rmax].r2) break;
    cmax = j;
    if (cmax < 100) cmax = 100;
    for (int64_t i = 0; i < rmax; i++) {
        for (int k = 0; k < 3; k++) {
            double dl = (double)q[i].pos[k + 3] - vel[k];
            vel[k] += dl / ((double)(i + 1));
            var[k] += dl * ((double)q[i].pos[k + 3] - vel[k]);
        }
        tv = (var[0] + var[1] + var[2]);
        if ((i < 10) || (tv < bv * (i - 3) * i)) {
            if (i > 3) bv = tv / (double)((i - 3) * i);
            else bv = 0;
            if (i < cmax) {
                h.n_core = i;
                h.min_vel_err = (float)bv;
                for (int k = 0; k < 3; k++) h.corevel[k] = (float)vel[k];
            }
            for (int k = 0; k < 3; k++) h.bulkvel[k] = (float)vel[k];
            h.min_bulkvel_err = (float)bv;
        }
    }
    for (int k = 0; k < 3; k++) h.pos[k + 3] = h.corevel[k];
}

// compute_kinetic_energy (src/potential.c:194-211)
__device__ void kinetic(PotRec *q, int64_t n, const float *vc, const float *pc, float scale,
                        const DevCfg &C) {
    double conv = 0.5 * (double)scale / RSG_GC;
    double hub = C.hub;
    for (int64_t i = 0; i < n; i++) {
        if (q[i].ke < 0) continue;
        q[i].ke = 0;
        for (int j = 0; j < 3; j++) {
            double dv = (double)fsub(q[i].pos[j + 3], vc[j]) +
                        hub * (double)scale * (double)fsub(q[i].pos[j], pc[j]);
            q[i].ke = (float)((double)q[i].ke + dv * dv);
        }
        q[i].ke = (float)((double)q[i].ke * conv);
    }
}

// compute_kinetic_energy on its own (rsg_compute_kinetic_energy): records
// are independent, one thread each, same arithmetic as kinetic().
__global__ void k_kinetic_el(PotRec *q, int64_t n, float vc0, float vc1, float vc2, float pc0,
                             float pc1, float pc2, float scale, double hub) {
    int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= n || q[i].ke < 0) return;
    const float vc[3] = {vc0, vc1, vc2}, pc[3] = {pc0, pc1, pc2};
    double conv = 0.5 * (double)scale / RSG_GC;
    float ke = 0;
    for (int j = 0; j < 3; j++) {
        double dv = (double)fsub(q[i].pos[j + 3], vc[j]) +
                    hub * (double)scale * (double)fsub(q[i].pos[j], pc[j]);
        ke = (float)((double)ke + dv * dv);
    }
    q[i].ke = (float)((double)ke * conv);
}
void kinetic_energy_device(PotRec *d, int64_t n, const float *vc, const float *pc, float scale,
                           double hub, cudaStream_t st) {
    launch(k_kinetic_el, nblk(n, 256), 256, 0, st, d, n, vc[0], vc[1], vc[2], pc[0], pc[1], pc[2],
           scale, hub);
    RSG_CHECK_LAUNCH();
}

__device__ inline bool unbound(const PotRec &r) { return r.pe < (double)r.ke; }

// calc_shape (src/properties.c:216-326)
__device__ void shape(rsg_halo &h, const PotRec *po, int64_t tot, int bound, const DevCfg &C) {
    int64_t it = C.shape_iterations, an = 0;
    float minr = fmul((float)C.force_res, (float)C.force_res);
    double mt[3][3], orth[3][3], eig[3] = {0, 0, 0}, r = 0, dr, dr2, w = 0;
    h.b_to_a = h.c_to_a = 0;
    h.A[0] = h.A[1] = h.A[2] = 0;
    if (!(h.r > 0)) return;
    minr = (float)((double)minr * (1e6 / (double)fmul(h.r, h.r)));
    for (int64_t j = 0; j < tot; j++) {
        if (bound && unbound(po[j])) continue;
        an++;
    }
    if (an < 3 || !(h.r > 0)) return;
    if (an < it) it = an;
    for (int i = 0; i < 3; i++) {
        for (int k = 0; k < 3; k++) orth[i][k] = 0;
        orth[i][i] = 1;
        eig[i] = (double)fmul(h.r, h.r) * 1e-6;
    }
    for (int64_t i = 0; i < it; i++) {
        for (int k = 0; k < 3; k++)
            for (int l = 0; l < 3; l++) mt[k][l] = 0;
        w = 0;
        for (int64_t j = 0; j < tot; j++) {
            if (bound && unbound(po[j])) continue;
            r = 0;
            for (int k = 0; k < 3; k++) {
                dr = 0;
                for (int l = 0; l < 3; l++) dr += orth[k][l] * (double)fsub(po[j].pos[l], h.pos[l]);
                r += dr * dr / eig[k];
            }
            if (r < (double)minr) r = minr;
            if (!(r > 0 && r <= 1)) continue;
            double tw = (C.weighted_shapes) ? 1.0 / r : 1.0;
            w += tw;
            for (int k = 0; k < 3; k++) {
                dr = (double)fsub(po[j].pos[k], h.pos[k]);
                mt[k][k] += dr * dr * tw;
                for (int l = 0; l < k; l++) {
                    dr2 = (double)fsub(po[j].pos[l], h.pos[l]);
                    mt[k][l] += dr2 * dr * tw;
                    mt[l][k] = mt[k][l];
                }
            }
        }
        if (!w) return;
        for (int k = 0; k < 3; k++)
            for (int l = 0; l < 3; l++) mt[k][l] /= (double)w;
        double mt2[3][3];
        for (int k = 0; k < 3; k++)
            for (int l = 0; l < 3; l++) mt2[k][l] = mt[k][l];
        jacobi3(mt, eig, orth);
        int a = 0, b = 1, c = 2;
        if (eig[1] > eig[0]) {
            b = 0;
            a = 1;
        }
        if (eig[2] > eig[b]) {
            c = b;
            b = 2;
        }
        if (eig[b] > eig[a]) {
            int t = a;
            a = b;
            b = t;
        }
        if (!eig[a] || !eig[b] || !eig[c]) return;
        float ba = (float)sqrt(eig[b] / eig[a]);
        float ca = (float)sqrt(eig[c] / eig[a]);
        if ((fabs((double)fsub(ba, h.b_to_a)) < 0.01 * (double)h.b_to_a) &&
            (fabs((double)fsub(ca, h.c_to_a)) < 0.01 * (double)h.c_to_a))
            return;
        h.b_to_a = (ba > 0) ? ba : 0;
        h.c_to_a = (ca > 0) ? ca : 0;
        r = sqrt(eig[a]);
        for (int k = 0; k < 3; k++) {
            h.A[k] = (float)(1e3 * r * orth[a][k]);
            eig[k] *= ((double)fmul(h.r, h.r) * 1e-6) / (r * r);
        }
        h.inertia_tensor[0] = (float)mt2[0][0];
        h.inertia_tensor[1] = (float)mt2[1][1];
        h.inertia_tensor[2] = (float)mt2[2][2];
        h.inertia_tensor[3] = (float)mt2[0][1];
        h.inertia_tensor[4] = (float)mt2[1][2];
        h.inertia_tensor[5] = (float)mt2[2][0];
    }
}

// estimate_total_energy (src/properties.c:328-349)
__device__ float total_energy(const PotRec *po, int64_t tot, float *ratio, const DevCfg &C) {
    double phi = 0, tphi = 0, ke = 0, r;
    for (int64_t i = tot - 1; i >= 0; i--) {
        if (po[i].pe > (double)po[i].ke) {
            ke += po[i].ke;
            r = sqrt((double)po[i].r2);
            if (r < C.force_res) r = C.force_res;
            tphi += C.particle_mass * i / r + phi;
            phi += C.particle_mass / r;
        }
    }
    tphi /= 2.0;
    *ratio = 0;
    if (tphi) *ratio = (float)(ke / tphi);
    float sn = (float)C.scale_now;
    return (float)((ke - tphi) * C.particle_mass * RSG_GC / (double)sn);
}

// calc_shape (src/properties.c:216-326) for 32 halos per warp, in the
// reference's summation order.  Each iteration runs the record phase of
// every halo still iterating in turn -- the lanes compute the terms of 32
// records at a time (ellipsoid radius, weight, products) and lane c < 7 adds
// accumulator c over them in record order -- and then the 32 halos'
// decisions (Jacobi, the 1% rule) side by side, one per lane: left to one
// lane, that FP64 work occupied the narrow FP64 pipe for a single lane's
// result.  `B` is this warp's state in shared memory.
struct ShapeBatch {
    double v[32][7];
    double acc[32][7];
    double orth[32][3][3], eig[32][3];
    float minr[32], hp[32][3];
    int it[32], done[32];
    int set[32];  // records of halo base + q, -1 for a halo this warp skips
};
__device__ void shape_batch(rsg_halo *H, const int32_t *toff, const PotRec *PO, int32_t base,
                            int32_t NH, int bound, const DevCfg &C, ShapeBatch &B) {
    const unsigned FULL = 0xffffffffu;
    const int lane = threadIdx.x & 31;
    {
        // lane q sets up halo base + q (the loop's prologue, src/properties.c:222-250)
        const int32_t hq = base + lane;
        int done = 1, itq = 0;
        float minr = 0.f;
        if (hq < NH && B.set[lane] >= 0) {
            rsg_halo &h = H[hq];
            const PotRec *po = PO + toff[hq];
            const int64_t tot = B.set[lane];
            int64_t an = 0;
            for (int64_t j = 0; j < tot; j++) an += !(bound && unbound(po[j]));
            int64_t it = C.shape_iterations;
            minr = fmul((float)C.force_res, (float)C.force_res);
            h.b_to_a = h.c_to_a = 0;
            h.A[0] = h.A[1] = h.A[2] = 0;
            if (h.r > 0) {
                minr = (float)((double)minr * (1e6 / (double)fmul(h.r, h.r)));
                if (an >= 3) {
                    if (an < it) it = an;
                    itq = (int)it;
                    done = itq <= 0;
                    for (int i = 0; i < 3; i++) {
                        for (int k = 0; k < 3; k++) B.orth[lane][i][k] = 0;
                        B.orth[lane][i][i] = 1;
                        B.eig[lane][i] = (double)fmul(h.r, h.r) * 1e-6;
                    }
                }
            }
            B.hp[lane][0] = h.pos[0];
            B.hp[lane][1] = h.pos[1];
            B.hp[lane][2] = h.pos[2];
        }
        B.done[lane] = done;
        B.it[lane] = itq;
        B.minr[lane] = minr;
    }
    __syncwarp();
    int maxit = 0;
    for (int q = 0; q < 32; q++) maxit = max(maxit, B.done[q] ? 0 : B.it[q]);
    for (int i = 0; i < maxit; i++) {
        for (int q = 0; q < 32; q++) {
            if (B.done[q] || i >= B.it[q]) continue;
            const int32_t hq = base + q;
            const PotRec *po = PO + toff[hq];
            const int64_t tot = B.set[q];
            const float hp0 = B.hp[q][0], hp1 = B.hp[q][1], hp2 = B.hp[q][2];
            const double minr = (double)B.minr[q];
            double a = 0;  // lane c < 7 owns accumulator c (w, m00, m11, m22, m10, m20, m21)
            for (int64_t b0 = 0; b0 < tot; b0 += 32) {
                const int64_t j = b0 + lane;
                bool sk = true;
                double vv[7];
                if (j < tot && !(bound && unbound(po[j]))) {
                    const float *p = po[j].pos;
                    double dd[3] = {(double)fsub(p[0], hp0), (double)fsub(p[1], hp1),
                                    (double)fsub(p[2], hp2)};
                    double r = 0, dr;
                    for (int k = 0; k < 3; k++) {
                        dr = 0;
                        for (int l = 0; l < 3; l++) dr += B.orth[q][k][l] * dd[l];
                        r += dr * dr / B.eig[q][k];
                    }
                    if (r < minr) r = minr;
                    if (r > 0 && r <= 1) {
                        double tw = (C.weighted_shapes) ? 1.0 / r : 1.0;
                        vv[0] = tw;
                        vv[1] = dd[0] * dd[0] * tw;
                        vv[2] = dd[1] * dd[1] * tw;
                        vv[3] = dd[2] * dd[2] * tw;
                        vv[4] = dd[0] * dd[1] * tw;
                        vv[5] = dd[0] * dd[2] * tw;
                        vv[6] = dd[1] * dd[2] * tw;
                        sk = false;
                        for (int c = 0; c < 7; c++) B.v[lane][c] = vv[c];
                    }
                }
                const uint32_t skip = __ballot_sync(FULL, sk);
                __syncwarp();
                if (lane < 7) {
                    const int m = (tot - b0) < 32 ? (int)(tot - b0) : 32;
                    for (int t = 0; t < m; t++)
                        if (!((skip >> t) & 1u)) a += B.v[t][lane];
                }
                __syncwarp();
            }
            if (lane < 7) B.acc[q][lane] = a;
        }
        __syncwarp();
        // the decisions of every halo still iterating, one per lane
        if (!B.done[lane] && i < B.it[lane]) {
            rsg_halo &h = H[base + lane];
            const double *acc = B.acc[lane];
            double w = acc[0];
            if (!w) B.done[lane] = 1;
            else {
                double m[3][3] = {{acc[1], acc[4], acc[5]}, {acc[4], acc[2], acc[6]},
                                  {acc[5], acc[6], acc[3]}};
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
                    B.eig[lane][k] = e2[k];
                    for (int l = 0; l < 3; l++) B.orth[lane][k][l] = o2[k][l];
                }
                if (!e2[a2] || !e2[b] || !e2[c]) B.done[lane] = 1;
                else {
                    float ba = (float)sqrt(e2[b] / e2[a2]);
                    float ca = (float)sqrt(e2[c] / e2[a2]);
                    if ((fabs((double)fsub(ba, h.b_to_a)) < 0.01 * (double)h.b_to_a) &&
                        (fabs((double)fsub(ca, h.c_to_a)) < 0.01 * (double)h.c_to_a))
                        B.done[lane] = 1;
                    else {
                        h.b_to_a = (ba > 0) ? ba : 0;
                        h.c_to_a = (ca > 0) ? ca : 0;
                        double rr = sqrt(e2[a2]);
                        for (int k = 0; k < 3; k++) {
                            h.A[k] = (float)(1e3 * rr * o2[a2][k]);
                            B.eig[lane][k] *= ((double)fmul(h.r, h.r) * 1e-6) / (rr * rr);
                        }
                        h.inertia_tensor[0] = (float)mt2[0][0];
                        h.inertia_tensor[1] = (float)mt2[1][1];
                        h.inertia_tensor[2] = (float)mt2[2][2];
                        h.inertia_tensor[3] = (float)mt2[0][1];
                        h.inertia_tensor[4] = (float)mt2[1][2];
                        h.inertia_tensor[5] = (float)mt2[2][0];
                    }
                }
            }
        }
        __syncwarp();
    }
}

// _calc_pseudo_evolution_masses (src/properties.c:351-382)
__device__ void pseudo_masses(rsg_halo &h, const PotRec *po, int64_t tot, int bound,
                              const DevCfg &C) {
    int64_t np_ = 0, npd = 0;
    double r, r32, mx = 0, rpd = (double)h.rs * 4.0;
    if (rpd < (double)h.r / 5.0) rpd = (double)h.r / 5.0;
    rpd *= 1e-3;
    for (int64_t j = 0; j < tot; j++) {
        if (bound && unbound(po[j])) continue;
        np_++;
        r = sqrt((double)po[j].r2);
        r32 = sqrt(r);
        r32 = r32 * r32 * r32;
        if ((double)(np_ * np_) / r32 > mx) mx = (double)(np_ * np_) / r32;
        if (r < rpd) npd = np_;
    }
    h.m_pe_d = (float)(npd * C.particle_mass);
    h.m_pe_b = (float)(C.particle_mass * pow(mx, 2.0 / 3.0) /
                       cbrt(4.0 * M_PI * C.rvir_dens_z0 / 3.0));
}

// NFW pieces (src/nfw.c:14-173)
__device__ double c_to_f(double c) {
    double cp1 = 1.0 + c;
    return (c * cp1 / (log1p(c) * cp1 - c));
}
__device__ double f_to_c(double f) {
    double c = f, tc = c_to_f(c), nc;
    for (int guard = 0; fabs((f - tc) / f) > 1e-7; guard++) {
        if (guard >= 100000) {  // Newton steps converge in a handful of iterations
            loop_limit_hit();
            break;
        }
        double tc2 = c_to_f(c + 0.1), slope = (tc2 - tc) / 0.1;
        nc = c + (f - tc) / slope;
        if (nc < 0) c /= 2;
        else c = nc;
        tc = c_to_f(c);
    }
    return c;
}
__device__ float klypin_rs(float mvir, float rvir, float vmax, float rvmax, float scale) {
    if (!mvir || !rvir || !vmax) return (float)((double)rvmax / RSG_RMAX_TO_RS);
    float vm2 = (float)((double)vmax / RSG_VMAX_CONST);
    vm2 = fmul(fmul(vm2, vm2), scale);
    float f = (float)(((double)rvir / 1.0e3) * (double)vm2 / ((double)mvir * RSG_RS_CONSTANT));
    if (f < 4.625f) return (float)((double)rvmax / RSG_RMAX_TO_RS);
    float c = (float)f_to_c(f);
    if (c <= 0) return (float)((double)rvmax / RSG_RMAX_TO_RS);
    return __fdiv_rn(rvir, c);
}
__device__ __forceinline__ float nfw_menc(float r, float rs) {
    return (float)(log((double)__fdiv_rn(fadd(rs, r), rs)) - (double)__fdiv_rn(r, fadd(rs, r)));
}
__device__ float chi2_scale(float rs, const float *br, const float *w, int64_t nb) {
    float bm = (float)((double)nfw_menc(br[nb], rs) / ((double)nb)), last = 0, chi2 = 0, dx;
    for (int64_t i = 0; i < nb; i++) {
        float menc = nfw_menc(br[i + 1], rs);
        dx = __fdiv_rn(fmul(w[i], fsub(fsub(menc, last), bm)), bm);
        chi2 = fadd(chi2, fmul(dx, dx));
        last = menc;
    }
    return chi2;
}
__device__ float fit_bins(float rs, const float *br, const float *w, int64_t nb, float *chi2o) {
    if (!(rs > br[0]) || !(rs < br[nb])) rs = br[(nb + 1) / 2];
    float irs = rs, chi2 = chi2_scale(rs, br, w, nb), drs = (float)((double)rs / 10.0), lc = 1e30f;
    int64_t it = 0;
    if (!(rs > 0)) return irs;
    int guard = 0;
    while (fabs((double)fsub(chi2, lc)) > 0.005 * (double)chi2 && it < 15 && ++guard < 100000) {
        lc = chi2;
        if (fadd(rs, drs) > br[nb]) drs = (float)(0.1 * (double)fsub(br[nb], rs));
        if (fsub(rs, drs) < br[0]) drs = (float)(0.1 * (double)fsub(rs, br[0]));
        float cr = chi2_scale(fadd(rs, drs), br, w, nb), cl = chi2_scale(fsub(rs, drs), br, w, nb);
        float dx = (float)(0.5 * (double)fsub(cr, cl) / (double)drs);
        float dx2 = (float)(((double)fadd(cr, cl) - 2.0 * (double)chi2) / (double)fmul(drs, drs));
        float mv = 0;
        if (dx2 != 0) mv = __fdiv_rn(-dx, dx2);
        if (!mv) return rs;
        if (fadd(rs, mv) > 4 * rs) mv = (float)(3.0 * (double)rs);
        if ((double)fadd(rs, mv) < 0.25 * (double)rs) mv = (float)(-0.75 * (double)rs);
        float nrs = fadd(rs, mv);
        if (nrs > br[nb]) nrs = (float)((double)rs + 0.8 * (double)fsub(br[nb], rs));
        else if (nrs < br[0]) nrs = (float)((double)rs + 0.8 * (double)fsub(br[0], rs));
        float nc = chi2_scale(nrs, br, w, nb);
        if (cr < nc) {
            nc = cr;
            nrs = fadd(rs, drs);
        }
        if (cl < nc) {
            nc = cl;
            nrs = fsub(rs, drs);
        }
        if (lc < nc) {
            drs = (float)((double)drs * 0.5);
            continue;
        }
        drs = (float)(fabs((double)fsub(rs, nrs)) / 10.0);
        rs = nrs;
        chi2 = nc;
        it++;
    }
    *chi2o = chi2;
    return rs;
}
__device__ void scale_radius(rsg_halo &h, float mvir, float rvir, float vmax, float rvmax,
                             float scale, const PotRec *po, int64_t tot, int bound,
                             const DevCfg &C) {
    float br[51], w[50];
    for (int i = 0; i < 51; i++) br[i] = 0;
    for (int i = 0; i < 50; i++) w[i] = 0;
    int64_t nb = 0, an = 0, pp = 0, i, j;
    float rs = h.klypin_rs = klypin_rs(mvir, rvir, vmax, rvmax, scale);
    for (i = 0; i < tot - 1; i++) {
        if (bound && unbound(po[i])) continue;
        an++;
    }
    if (an < 100) {
        h.rs = rs;
        return;
    }
    pp = (int64_t)ceil(((double)an / (double)50));
    if (pp < 15) pp = (an) / ((int64_t)(an / 15));
    br[0] = 0;
    for (i = 0, j = 0; i < tot - 1; i++) {
        if (bound && unbound(po[i])) continue;
        if (++j == pp) {
            nb++;
            if (nb > 50) break;
            br[nb] = (float)(1e3 * 0.5 * (sqrt((double)po[i].r2) + sqrt((double)po[i + 1].r2)));
            w[nb - 1] = 1;
            j = 0;
        }
    }
    if (nb > 50) nb = 50;
    for (i = 0; i < nb; i++)
        if ((double)br[i] * 1e-3 < 3 * C.force_res) w[i] = 0.1f;
    float chi2 = 0.0f;
    h.rs = fit_bins(rs, br, w, nb, &chi2);
    h.chi2 = chi2;
}

// _calc_additional_halo_props (src/properties.c:384-510)
__device__ void more_props(rsg_halo &h, const PotRec *po, int64_t tot, int bound,
                           const DevCfg &C) {
    int64_t j, pmd = 0, np_ = 0, npa[4] = {0, 0, 0, 0}, npv = 0, dtot = 0, avg = 0, nhalf = 0;
    float scale = (float)C.scale_now;
    const double f43 = 4.0 * M_PI / 3.0;
    double dth = C.thresh_dens[0] * f43, d1 = C.thresh_dens[1] * f43;
    double d2 = C.thresh_dens[2] * f43, d3 = C.thresh_dens[3] * f43, d4 = C.thresh_dens[4] * f43;
    double rth = C.rvir_dens * f43, vconv = C.particle_mass / (double)scale;
    double r, cv, vmax = 0, rvmax = 0, L[3] = {0, 0, 0}, Jh, m = 0, ds;
    double vrms[3] = {0, 0, 0}, xa[3] = {0, 0, 0}, va[3] = {0, 0, 0}, md, cd, rvir, mvir;
    for (j = 0; j < tot; j++) {
        if (bound && unbound(po[j])) continue;
        np_++;
        r = sqrt((double)po[j].r2);
        if (r < C.force_res) r = C.force_res;
        cd = ((double)np_ / (r * r * r));
        if (cd > dth) {
            pmd = np_;
            dtot = j;
        }
        if (cd > d1) npa[0] = np_;
        if (cd > d2) npa[1] = np_;
        if (cd > d3) npa[2] = np_;
        if (cd > d4) npa[3] = np_;
        if (cd > rth) {
            cv = (double)np_ / r;
            npv = np_;
            if (pmd && cv > vmax) {
                vmax = cv;
                rvmax = r;
            }
        }
    }
    for (j = 0; j < dtot; j++) {
        if (bound && unbound(po[j])) continue;
        const float *c = h.pos, *p = po[j].pos;
        L[0] += (double)fmul(fsub(p[1], c[1]), fsub(p[5], c[5]));
        L[0] -= (double)fmul(fsub(p[2], c[2]), fsub(p[4], c[4]));
        L[1] += (double)fmul(fsub(p[2], c[2]), fsub(p[3], c[3]));
        L[1] -= (double)fmul(fsub(p[0], c[0]), fsub(p[5], c[5]));
        L[2] += (double)fmul(fsub(p[0], c[0]), fsub(p[4], c[4]));
        L[2] -= (double)fmul(fsub(p[1], c[1]), fsub(p[3], c[3]));
        avg++;
        if (avg * 2 >= pmd && !nhalf) nhalf = j;
        for (int k = 0; k < 3; k++) {
            xa[k] += ((double)p[k] - xa[k]) / ((double)avg);
            md = (double)p[k + 3] - va[k];
            va[k] += md / (double)avg;
            vrms[k] += md * ((double)p[k + 3] - va[k]);
        }
    }
    m = pmd * C.particle_mass;
    if (!bound) h.m = (float)m;
    else h.mgrav = (float)m;
    for (int k = 0; k < 3; k++) vrms[k] = (avg > 0) ? (vrms[k] / avg) : 0;
    if ((!bound) == (!C.bound_props)) {
        h.Xoff = h.Voff = 0;
        for (int k = 0; k < 3; k++) {
            ds = xa[k] - (double)h.pos[k];
            h.Xoff = (float)((double)h.Xoff + ds * ds);
            ds = va[k] - (double)h.pos[k + 3];
            h.Voff = (float)((double)h.Voff + ds * ds);
        }
        for (int k = 0; k < 4; k++) h.alt_m[k] = (float)(npa[k] * C.particle_mass);
        h.Xoff = (float)(sqrt((double)h.Xoff) * 1e3);
        h.Voff = sqrt_fd(h.Voff);
        h.vrms = (float)sqrt(vrms[0] + vrms[1] + vrms[2]);
        h.vmax = (float)(RSG_VMAX_CONST * sqrt(vmax * vconv));
        h.rvmax = (float)(rvmax * 1e3);
        h.halfmass_radius = (float)(sqrt((double)po[nhalf].r2) * 1e3);
        h.r = (float)(cbrt((3.0 / (4.0 * M_PI)) * npa[2] / C.thresh_dens[3]) * 1e3);
        shape(h, po, npa[2], bound, C);
        h.b_to_a2 = h.b_to_a;
        h.c_to_a2 = h.c_to_a;
        for (int k = 0; k < 3; k++) h.A2[k] = h.A[k];
        for (int k = 0; k < 6; k++) h.inertia_tensor2[k] = h.inertia_tensor[k];
        h.r = (float)(cbrt((3.0 / (4.0 * M_PI)) * pmd / C.thresh_dens[0]) * 1e3);
        shape(h, po, dtot, bound, C);
        rvir = cbrt((3.0 / (4.0 * M_PI)) * npv / C.rvir_dens) * 1e3;
        mvir = npv * C.particle_mass;
        scale_radius(h, (float)m, h.r, h.vmax, h.rvmax, scale, po, dtot, bound, C);
        for (j = 0; j < 3; j++) h.J[j] = (float)(C.particle_mass * (double)scale * L[j]);
        h.energy = total_energy(po, dtot, &h.kin_to_pot, C);
        Jh = C.particle_mass * (double)scale * sqrt(L[0] * L[0] + L[1] * L[1] + L[2] * L[2]);
        h.spin = (float)((m > 0) ? (Jh * sqrt(fabs((double)h.energy)) / (RSG_GC * pow(m, 2.5))) : 0);
        h.bullock_spin = (float)((m > 0) ? (Jh / (mvir * sqrt(2.0 * RSG_GC * mvir * rvir * (double)scale / 1e3))) : 0);
        pseudo_masses(h, po, tot, bound, C);
    }
}

__global__ void k_halo_scans(rsg_halo *H, const rsg_extra_halo_info *E, int32_t NH,
                             PotRec *PO, const int32_t *toff, const int32_t *kept,
                             const DevCfg *Cp) {
    int h = blockIdx.x * blockDim.x + threadIdx.x;
    if (h >= NH) return;
    rsg_halo &hh = H[h];
    if (hh.num_p < 1) return;
    const DevCfg &C = *Cp;
    PotRec *q = PO + toff[h];
    int64_t tot = kept[h];
    corevel(hh, q, tot, C);
    float sn = (float)C.scale_now;
    if (E[h].sub_of > -1) kinetic(q, tot, hh.corevel, hh.pos, sn, C);
    else kinetic(q, tot, hh.bulkvel, hh.pos, sn, C);
    more_props(hh, q, tot, 0, C);
    more_props(hh, q, tot, 1, C);
}

}  // namespace rsg
#include "props_seg.cuh"
namespace rsg {

// ---- block-cooperative scans for large halos ------------------------------
// Same arithmetic as corevel/kinetic/more_props/shape above.  The block
// computes every per-particle operand in parallel (ellipsoidal radius,
// weights, tensor products, densities, energies); sums that the reference
// accumulates in array order are then accumulated by warp 0 with one lane
// per accumulator, walking the staged operands in order, so each sum rounds
// exactly as the reference's loop while all of them advance together.
// Threshold decisions (density thresholds, Vmax) become block reductions.
#define RSG_SB 256

struct BlkBuf {
    double v[RSG_SB][9];
    unsigned char skip[RSG_SB];
    int32_t np[RSG_SB];
};

// inclusive count of non-skipped entries up to each thread of a chunk
__device__ int chunk_prefix(int flag, int *warp_tot) {
    int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    unsigned m = __ballot_sync(0xffffffffu, flag);
    int incl = __popc(m & (0xffffffffu >> (31 - lane)));
    if (lane == 31) warp_tot[w] = __popc(m);
    __syncthreads();
    int off = 0;
    for (int i = 0; i < w; i++) off += warp_tot[i];
    __syncthreads();
    return off + incl;
}

// deterministic block sum of one double (all threads call; result in all)
__device__ double bsum(double v, double *sm) {
    for (int o = 16; o; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    __syncthreads();
    if ((threadIdx.x & 31) == 0) sm[threadIdx.x >> 5] = v;
    __syncthreads();
    if (threadIdx.x == 0) {
        double t = 0;
        for (int i = 0; i < RSG_SB / 32; i++) t += sm[i];
        sm[RSG_SB / 32] = t;
    }
    __syncthreads();
    double r = sm[RSG_SB / 32];
    __syncthreads();
    return r;
}

__device__ void shape_blk(rsg_halo &h, const PotRec *po, int64_t tot, int bound,
                          const DevCfg &C, BlkBuf &B, int exact) {
    __shared__ double red_s[RSG_SB / 32 + 1];
    __shared__ double orth[3][3], eig[3], acc[7];
    __shared__ float minr_s;
    __shared__ int64_t it_s;
    __shared__ int done, an_s;
    __shared__ int wt[RSG_SB / 32];
    // number of analysed particles (bound filter)
    int cntl = 0;
    for (int64_t j = threadIdx.x; j < tot; j += RSG_SB) cntl += !(bound && unbound(po[j]));
    for (int o = 16; o; o >>= 1) cntl += __shfl_down_sync(0xffffffffu, cntl, o);
    if (threadIdx.x == 0) an_s = 0;
    __syncthreads();
    if ((threadIdx.x & 31) == 0) atomicAdd(&an_s, cntl);
    __syncthreads();
    if (threadIdx.x == 0) {
        done = 0;
        int64_t it = C.shape_iterations, an = an_s;
        float minr = fmul((float)C.force_res, (float)C.force_res);
        h.b_to_a = h.c_to_a = 0;
        h.A[0] = h.A[1] = h.A[2] = 0;
        if (!(h.r > 0)) done = 1;
        else {
            minr = (float)((double)minr * (1e6 / (double)fmul(h.r, h.r)));
            if (an < 3 || !(h.r > 0)) done = 1;
            if (an < it) it = an;
            for (int i = 0; i < 3; i++) {
                for (int k = 0; k < 3; k++) orth[i][k] = 0;
                orth[i][i] = 1;
                eig[i] = (double)fmul(h.r, h.r) * 1e-6;
            }
        }
        minr_s = minr;
        it_s = it;
    }
    (void)wt;
    __syncthreads();
    if (done) return;
    const float hp0 = h.pos[0], hp1 = h.pos[1], hp2 = h.pos[2];
    for (int64_t i = 0; i < it_s; i++) {
        double a = 0;  // lane k of warp 0 owns accumulator k (w, m00, m11, m22, m10, m20, m21)
        double part[7] = {0, 0, 0, 0, 0, 0, 0};  // batched mode: per-thread partial sums
        for (int64_t b0 = 0; b0 < tot; b0 += RSG_SB) {
            int64_t j = b0 + threadIdx.x;
            unsigned char sk = 1;
            double vv[7];
            if (j < tot && !(bound && unbound(po[j]))) {
                const float *p = po[j].pos;
                double dd[3] = {(double)fsub(p[0], hp0), (double)fsub(p[1], hp1),
                                (double)fsub(p[2], hp2)};
                double r = 0, dr;
                for (int k = 0; k < 3; k++) {
                    dr = 0;
                    for (int l = 0; l < 3; l++) dr += orth[k][l] * dd[l];
                    r += dr * dr / eig[k];
                }
                if (r < (double)minr_s) r = minr_s;
                if (r > 0 && r <= 1) {
                    double tw = (C.weighted_shapes) ? 1.0 / r : 1.0;
                    vv[0] = tw;
                    vv[1] = dd[0] * dd[0] * tw;
                    vv[2] = dd[1] * dd[1] * tw;
                    vv[3] = dd[2] * dd[2] * tw;
                    vv[4] = dd[0] * dd[1] * tw;
                    vv[5] = dd[0] * dd[2] * tw;
                    vv[6] = dd[1] * dd[2] * tw;
                    sk = 0;
                }
            }
            if (!exact) {
                if (!sk)
                    for (int c = 0; c < 7; c++) part[c] += vv[c];
                continue;
            }
            if (!sk)
                for (int c = 0; c < 7; c++) B.v[threadIdx.x][c] = vv[c];
            B.skip[threadIdx.x] = sk;
            __syncthreads();
            if (threadIdx.x < 7) {
                int m = (tot - b0) < RSG_SB ? (int)(tot - b0) : RSG_SB;
                int c = threadIdx.x;
                for (int t = 0; t < m; t++)
                    if (!B.skip[t]) a += B.v[t][c];
            }
            __syncthreads();
        }
        if (!exact)
            for (int c = 0; c < 7; c++) {
                double t = bsum(part[c], red_s);
                if (threadIdx.x == c) a = t;
            }
        if (threadIdx.x < 7) acc[threadIdx.x] = a;
        __syncthreads();
        if (threadIdx.x == 0) {
            double w = acc[0];
            if (!w) done = 1;
            else {
                double m[3][3] = {{acc[1], acc[4], acc[5]}, {acc[4], acc[2], acc[6]},
                                  {acc[5], acc[6], acc[3]}};
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
                    eig[k] = e2[k];
                    for (int l = 0; l < 3; l++) orth[k][l] = o2[k][l];
                }
                if (!e2[a2] || !e2[b] || !e2[c]) done = 1;
                else {
                    float ba = (float)sqrt(e2[b] / e2[a2]);
                    float ca = (float)sqrt(e2[c] / e2[a2]);
                    if ((fabs((double)fsub(ba, h.b_to_a)) < 0.01 * (double)h.b_to_a) &&
                        (fabs((double)fsub(ca, h.c_to_a)) < 0.01 * (double)h.c_to_a))
                        done = 1;
                    else {
                        h.b_to_a = (ba > 0) ? ba : 0;
                        h.c_to_a = (ca > 0) ? ca : 0;
                        double rr = sqrt(e2[a2]);
                        for (int k = 0; k < 3; k++) {
                            h.A[k] = (float)(1e3 * rr * o2[a2][k]);
                            eig[k] *= ((double)fmul(h.r, h.r) * 1e-6) / (rr * rr);
                        }
                        h.inertia_tensor[0] = (float)mt2[0][0];
                        h.inertia_tensor[1] = (float)mt2[1][1];
                        h.inertia_tensor[2] = (float)mt2[2][2];
                        h.inertia_tensor[3] = (float)mt2[0][1];
                        h.inertia_tensor[4] = (float)mt2[1][2];
                        h.inertia_tensor[5] = (float)mt2[2][0];
                    }
                }
            }
        }
        __syncthreads();
        if (done) return;
    }
}

struct MPState {
    int64_t pmd, npa[4], npv, dtot, avg, nhalf, j0;
    double vmax, rvmax, L[3], m, xa[3], va[3], vrms[3];
};

// lexicographic max of (cv, -j) across the block
__device__ void blk_argmax(double &cv, int64_t &j, double *scv, int64_t *sj) {
    for (int o = 16; o; o >>= 1) {
        double c2 = __shfl_down_sync(0xffffffffu, cv, o);
        int64_t j2 = __shfl_down_sync(0xffffffffu, j, o);
        if (c2 > cv || (c2 == cv && j2 < j)) { cv = c2; j = j2; }
    }
    int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    if (lane == 0) { scv[w] = cv; sj[w] = j; }
    __syncthreads();
    if (threadIdx.x == 0)
        for (int i = 1; i < RSG_SB / 32; i++)
            if (scv[i] > scv[0] || (scv[i] == scv[0] && sj[i] < sj[0])) { scv[0] = scv[i]; sj[0] = sj[i]; }
    __syncthreads();
    cv = scv[0];
    j = sj[0];
    __syncthreads();
}

__device__ void more_props_blk(rsg_halo &h, const PotRec *po, int64_t tot, int bound,
                               const DevCfg &C, BlkBuf &B, int exact) {
    __shared__ double red_m[RSG_SB / 32 + 1];
    __shared__ MPState S;
    __shared__ int want;
    __shared__ int wt[RSG_SB / 32];
    __shared__ double scv[RSG_SB / 32];
    __shared__ int64_t sj[RSG_SB / 32];
    __shared__ unsigned long long red[8];
    float scale = (float)C.scale_now;
    const double f43 = 4.0 * M_PI / 3.0;
    const double dth = C.thresh_dens[0] * f43, d1 = C.thresh_dens[1] * f43;
    const double d2 = C.thresh_dens[2] * f43, d3 = C.thresh_dens[3] * f43, d4 = C.thresh_dens[4] * f43;
    const double rth = C.rvir_dens * f43;
    // pass 1 (src/properties.c:402-433) as reductions: the thresholds keep
    // the last qualifying running count, the Vmax search the first maximum
    // after the first particle above the Delta threshold
    if (threadIdx.x < 8) red[threadIdx.x] = 0;
    if (threadIdx.x == 0) { S.j0 = INT64_MAX; }
    __syncthreads();
    int64_t base_np = 0;
    int64_t l_pmd = 0, l_dtot = 0, l_npa[4] = {0, 0, 0, 0}, l_npv = 0, l_j0 = INT64_MAX;
    for (int64_t b0 = 0; b0 < tot; b0 += RSG_SB) {
        int64_t j = b0 + threadIdx.x;
        int ok = (j < tot) && !(bound && unbound(po[j]));
        int incl = chunk_prefix(ok, wt);
        int64_t np_ = base_np + incl;
        if (ok) {
            double r = sqrt((double)po[j].r2);
            if (r < C.force_res) r = C.force_res;
            double cd = ((double)np_ / (r * r * r));
            if (cd > dth) { l_pmd = np_; l_dtot = j; if (j < l_j0) l_j0 = j; }
            if (cd > d1) l_npa[0] = np_;
            if (cd > d2) l_npa[1] = np_;
            if (cd > d3) l_npa[2] = np_;
            if (cd > d4) l_npa[3] = np_;
            if (cd > rth) l_npv = np_;
        }
        __syncthreads();
        if (threadIdx.x == RSG_SB - 1) B.np[0] = incl;
        __syncthreads();
        base_np += B.np[0];
        __syncthreads();
    }
    // counts grow with j, so the last qualifying value is the maximum
    atomicMax(&red[0], (unsigned long long)l_pmd);
    atomicMax(&red[1], (unsigned long long)l_dtot * (l_pmd > 0));
    for (int k = 0; k < 4; k++) atomicMax(&red[2 + k], (unsigned long long)l_npa[k]);
    atomicMax(&red[6], (unsigned long long)l_npv);
    atomicMin((unsigned long long *)&S.j0, (unsigned long long)l_j0);
    __syncthreads();
    // Vmax: first maximum of np/r over qualifying particles at or after j0
    double bcv = -1;
    int64_t bj = INT64_MAX;
    base_np = 0;
    for (int64_t b0 = 0; b0 < tot; b0 += RSG_SB) {
        int64_t j = b0 + threadIdx.x;
        int ok = (j < tot) && !(bound && unbound(po[j]));
        int incl = chunk_prefix(ok, wt);
        int64_t np_ = base_np + incl;
        if (ok && j >= S.j0) {
            double r = sqrt((double)po[j].r2);
            if (r < C.force_res) r = C.force_res;
            double cd = ((double)np_ / (r * r * r));
            if (cd > rth) {
                double cv = (double)np_ / r;
                if (cv > bcv || (cv == bcv && j < bj)) { bcv = cv; bj = j; }
            }
        }
        __syncthreads();
        if (threadIdx.x == RSG_SB - 1) B.np[0] = incl;
        __syncthreads();
        base_np += B.np[0];
        __syncthreads();
    }
    blk_argmax(bcv, bj, scv, sj);
    if (threadIdx.x == 0) {
        S.pmd = (int64_t)red[0];
        S.dtot = (int64_t)red[1];
        for (int k = 0; k < 4; k++) S.npa[k] = (int64_t)red[2 + k];
        S.npv = (int64_t)red[6];
        S.vmax = 0;
        S.rvmax = 0;
        if (bcv > 0 && bj != INT64_MAX) {
            S.vmax = bcv;
            double r = sqrt((double)po[bj].r2);
            if (r < C.force_res) r = C.force_res;
            S.rvmax = r;
        }
        S.avg = 0;
        S.nhalf = 0;
    }
    __syncthreads();
    // pass 2 (src/properties.c:435-448): warp 0, lanes 0-2 own L[k], lanes
    // 3-5 xavg[k], lanes 6-8 vavg[k] and vrms[k]
    if (!exact) {
        // batched mode: block sums; running means become plain means and the
        // running second moments a two-pass sum about the mean
        double lp[3] = {0, 0, 0}, xs[3] = {0, 0, 0}, vs[3] = {0, 0, 0};
        int64_t cnt = 0, nh = INT64_MAX;
        const float *c = h.pos;
        int64_t base = 0;
        for (int64_t b0 = 0; b0 < S.dtot; b0 += RSG_SB) {
            int64_t j = b0 + threadIdx.x;
            int ok = j < S.dtot && !(bound && unbound(po[j]));
            int incl = chunk_prefix(ok, wt);
            if (ok) {
                const float *p = po[j].pos;
                for (int k = 0; k < 3; k++) {
                    int x = (k + 1) % 3, y = (k + 2) % 3;
                    lp[k] += (double)fmul(fsub(p[x], c[x]), fsub(p[y + 3], c[y + 3]));
                    lp[k] -= (double)fmul(fsub(p[y], c[y]), fsub(p[x + 3], c[x + 3]));
                    xs[k] += (double)p[k];
                    vs[k] += (double)p[k + 3];
                }
                cnt++;
                int64_t run = base + incl;
                if (j >= 1 && run * 2 >= S.pmd && j < nh) nh = j;
            }
            __syncthreads();
            if (threadIdx.x == RSG_SB - 1) B.np[0] = incl;
            __syncthreads();
            base += B.np[0];
            __syncthreads();
        }
        double tot_c = bsum((double)cnt, red_m);
        for (int k = 0; k < 3; k++) {
            double t = bsum(lp[k], red_m);
            if (threadIdx.x == 0) S.L[k] = t;
            t = bsum(xs[k], red_m);
            if (threadIdx.x == 0) S.xa[k] = tot_c > 0 ? t / tot_c : 0;
            t = bsum(vs[k], red_m);
            if (threadIdx.x == 0) S.va[k] = tot_c > 0 ? t / tot_c : 0;
        }
        __syncthreads();
        double v2[3] = {0, 0, 0};
        for (int64_t j = threadIdx.x; j < S.dtot; j += RSG_SB) {
            if (bound && unbound(po[j])) continue;
            for (int k = 0; k < 3; k++) {
                double d = (double)po[j].pos[k + 3] - S.va[k];
                v2[k] += d * d;
            }
        }
        for (int k = 0; k < 3; k++) {
            double t = bsum(v2[k], red_m);
            if (threadIdx.x == 0) S.vrms[k] = t;
        }
        __shared__ unsigned long long nhs;
        if (threadIdx.x == 0) nhs = (unsigned long long)INT64_MAX;
        __syncthreads();
        atomicMin(&nhs, (unsigned long long)nh);
        __syncthreads();
        if (threadIdx.x == 0) {
            S.avg = (int64_t)tot_c;
            S.nhalf = (nhs == (unsigned long long)INT64_MAX) ? 0 : (int64_t)nhs;
        }
        __syncthreads();
    } else {
        double acc_a = 0, acc_b = 0;
        int64_t avg = 0, nhalf = 0;
        const float *c = h.pos;
        for (int64_t b0 = 0; b0 < S.dtot; b0 += RSG_SB) {
            int64_t j = b0 + threadIdx.x;
            unsigned char sk = 1;
            if (j < S.dtot && !(bound && unbound(po[j]))) {
                for (int d = 0; d < 6; d++) B.v[threadIdx.x][d] = (double)po[j].pos[d];
                sk = 0;
            }
            B.skip[threadIdx.x] = sk;
            __syncthreads();
            if (threadIdx.x < 9) {
                int lane = threadIdx.x;
                int m = (S.dtot - b0) < RSG_SB ? (int)(S.dtot - b0) : RSG_SB;
                for (int t = 0; t < m; t++) {
                    if (B.skip[t]) continue;
                    avg++;
                    if (avg * 2 >= S.pmd && !nhalf) nhalf = b0 + t;
                    const double *p = B.v[t];
                    if (lane < 3) {
                        int x = (lane + 1) % 3, y = (lane + 2) % 3;
                        // L[0] += (p1-c1)(p5-c5) - ..., as add_ang_mom orders them
                        float pa = fmul(fsub((float)p[x], c[x]), fsub((float)p[y + 3], c[y + 3]));
                        float pb = fmul(fsub((float)p[y], c[y]), fsub((float)p[x + 3], c[x + 3]));
                        acc_a += (double)pa;
                        acc_a -= (double)pb;
                    } else if (lane < 6) {
                        int k = lane - 3;
                        acc_a += (p[k] - acc_a) / ((double)avg);
                    } else {
                        int k = lane - 6;
                        double md = p[k + 3] - acc_a;
                        acc_a += md / (double)avg;
                        acc_b += md * (p[k + 3] - acc_a);
                    }
                }
            }
            __syncthreads();
        }
        if (threadIdx.x < 3) S.L[threadIdx.x] = acc_a;
        else if (threadIdx.x < 6) S.xa[threadIdx.x - 3] = acc_a;
        else if (threadIdx.x < 9) { S.va[threadIdx.x - 6] = acc_a; S.vrms[threadIdx.x - 6] = acc_b; }
        if (threadIdx.x == 0) { S.avg = avg; S.nhalf = nhalf; }
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        S.m = S.pmd * C.particle_mass;
        if (!bound) h.m = (float)S.m;
        else h.mgrav = (float)S.m;
        for (int k = 0; k < 3; k++) S.vrms[k] = (S.avg > 0) ? (S.vrms[k] / S.avg) : 0;
        want = ((!bound) == (!C.bound_props));
        if (want) {
            double ds;
            h.Xoff = h.Voff = 0;
            for (int k = 0; k < 3; k++) {
                ds = S.xa[k] - (double)h.pos[k];
                h.Xoff = (float)((double)h.Xoff + ds * ds);
                ds = S.va[k] - (double)h.pos[k + 3];
                h.Voff = (float)((double)h.Voff + ds * ds);
            }
            for (int k = 0; k < 4; k++) h.alt_m[k] = (float)(S.npa[k] * C.particle_mass);
            h.Xoff = (float)(sqrt((double)h.Xoff) * 1e3);
            h.Voff = sqrt_fd(h.Voff);
            h.vrms = (float)sqrt(S.vrms[0] + S.vrms[1] + S.vrms[2]);
            h.vmax = (float)(RSG_VMAX_CONST * sqrt(S.vmax * (C.particle_mass / (double)scale)));
            h.rvmax = (float)(S.rvmax * 1e3);
            h.halfmass_radius = (float)(sqrt((double)po[S.nhalf].r2) * 1e3);
            h.r = (float)(cbrt((3.0 / (4.0 * M_PI)) * S.npa[2] / C.thresh_dens[3]) * 1e3);
        }
    }
    __syncthreads();
    if (!want) return;
    shape_blk(h, po, S.npa[2], bound, C, B, exact);
    __syncthreads();
    if (threadIdx.x == 0) {
        h.b_to_a2 = h.b_to_a;
        h.c_to_a2 = h.c_to_a;
        for (int k = 0; k < 3; k++) h.A2[k] = h.A[k];
        for (int k = 0; k < 6; k++) h.inertia_tensor2[k] = h.inertia_tensor[k];
        h.r = (float)(cbrt((3.0 / (4.0 * M_PI)) * S.pmd / C.thresh_dens[0]) * 1e3);
    }
    __syncthreads();
    shape_blk(h, po, S.dtot, bound, C, B, exact);
    __syncthreads();
    // estimate_total_energy over [0, dtot) in descending order: lane 0 sums
    // ke, lane 1 the two coupled potential sums (src/properties.c:328-349)
    __shared__ double en[3];
    if (!exact) {
        // tphi = sum a_i + sum b_i * (number of qualifying particles before i)
        double kes = 0, ts = 0;
        int64_t base = 0;
        for (int64_t b0 = 0; b0 < S.dtot; b0 += RSG_SB) {
            int64_t i = b0 + threadIdx.x;
            int ok = i < S.dtot && po[i].pe > (double)po[i].ke;
            int incl = chunk_prefix(ok, wt);
            if (ok) {
                double r = sqrt((double)po[i].r2);
                if (r < C.force_res) r = C.force_res;
                kes += (double)po[i].ke;
                ts += C.particle_mass * i / r + (C.particle_mass / r) * (double)(base + incl - 1);
            }
            __syncthreads();
            if (threadIdx.x == RSG_SB - 1) B.np[0] = incl;
            __syncthreads();
            base += B.np[0];
            __syncthreads();
        }
        double t1 = bsum(kes, red_m), t2 = bsum(ts, red_m);
        if (threadIdx.x == 0) { en[0] = t1; en[1] = t2; }
        __syncthreads();
    } else {
        double acc_a = 0, acc_b = 0;
        for (int64_t top = S.dtot - 1; top >= 0; top -= RSG_SB) {
            int64_t i = top - threadIdx.x;
            unsigned char sk = 1;
            if (i >= 0 && po[i].pe > (double)po[i].ke) {
                double r = sqrt((double)po[i].r2);
                if (r < C.force_res) r = C.force_res;
                B.v[threadIdx.x][0] = (double)po[i].ke;
                B.v[threadIdx.x][1] = C.particle_mass * i / r;
                B.v[threadIdx.x][2] = C.particle_mass / r;
                sk = 0;
            }
            B.skip[threadIdx.x] = sk;
            __syncthreads();
            int m = (top + 1) < RSG_SB ? (int)(top + 1) : RSG_SB;
            if (threadIdx.x == 0) {
                for (int t = 0; t < m; t++)
                    if (!B.skip[t]) acc_a += B.v[t][0];
            } else if (threadIdx.x == 1) {
                for (int t = 0; t < m; t++)
                    if (!B.skip[t]) {
                        acc_a += B.v[t][1] + acc_b;
                        acc_b += B.v[t][2];
                    }
            }
            __syncthreads();
        }
        if (threadIdx.x == 0) en[0] = acc_a;
        if (threadIdx.x == 1) en[1] = acc_a;
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        double rvir = cbrt((3.0 / (4.0 * M_PI)) * S.npv / C.rvir_dens) * 1e3;
        double mvir = S.npv * C.particle_mass, m = S.m;
        scale_radius(h, (float)m, h.r, h.vmax, h.rvmax, scale, po, S.dtot, bound, C);
        for (int j = 0; j < 3; j++) h.J[j] = (float)(C.particle_mass * (double)scale * S.L[j]);
        {
            double ke = en[0], tphi = en[1] / 2.0;
            h.kin_to_pot = 0;
            if (tphi) h.kin_to_pot = (float)(ke / tphi);
            float sn = (float)C.scale_now;
            h.energy = (float)((ke - tphi) * C.particle_mass * RSG_GC / (double)sn);
        }
        double Jh = C.particle_mass * (double)scale *
                    sqrt(S.L[0] * S.L[0] + S.L[1] * S.L[1] + S.L[2] * S.L[2]);
        h.spin = (float)((m > 0) ? (Jh * sqrt(fabs((double)h.energy)) / (RSG_GC * pow(m, 2.5))) : 0);
        h.bullock_spin = (float)((m > 0) ? (Jh / (mvir * sqrt(2.0 * RSG_GC * mvir * rvir * (double)scale / 1e3))) : 0);
        pseudo_masses(h, po, tot, bound, C);
    }
    __syncthreads();
}

// calculate_corevel with the block: rmax / core_max by reductions, then the
// three running means and variances on lanes 0-2 of warp 0 (the combined
// variance, and so every decision, is shared through shuffles).
__device__ void corevel_blk(rsg_halo &h, const PotRec *q, int64_t tot, const DevCfg &C) {
    __shared__ unsigned long long rm[2];
    double rt = C.rvir_dens * (4.0 * M_PI / 3.0);
    if (threadIdx.x == 0) { rm[0] = 0; rm[1] = 0; }
    __syncthreads();
    // rmax = largest j with j*j > r2^3 * rt^2 (or -1)
    long long best = -1;
    for (int64_t j = threadIdx.x; j < tot; j += blockDim.x) {
        float r2 = q[j].r2;
        if ((double)(j * j) > (double)fmul(fmul(r2, r2), r2) * (rt * rt)) best = j;
    }
    atomicMax(&rm[0], (unsigned long long)(best + 1));
    __syncthreads();
    int64_t rmax = (int64_t)rm[0] - 1;
    if (rmax < 1) return;
    long long cb = -1;
    for (int64_t j = threadIdx.x; j < tot; j += blockDim.x)
        if ((double)q[j].r2 * 100.0 < (double)q[rmax].r2) cb = j;
    atomicMax(&rm[1], (unsigned long long)(cb + 1));
    __syncthreads();
    int64_t cmax = (int64_t)rm[1] - 1;
    if (cmax < 100) cmax = 100;
    if (threadIdx.x < 3) {
        const unsigned mask = 0x7u;
        int k = threadIdx.x;
        double vel = 0, var = 0, bv = 0;
        for (int64_t i = 0; i < rmax; i++) {
            double x = (double)q[i].pos[k + 3];
            double dl = x - vel;
            vel += dl / ((double)(i + 1));
            var += dl * (x - vel);
            double v0 = __shfl_sync(mask, var, 0), v1 = __shfl_sync(mask, var, 1),
                   v2 = __shfl_sync(mask, var, 2);
            double tv = (v0 + v1) + v2;
            if ((i < 10) || (tv < bv * (i - 3) * i)) {
                if (i > 3) bv = tv / (double)((i - 3) * i);
                else bv = 0;
                if (i < cmax) {
                    if (k == 0) {
                        h.n_core = i;
                        h.min_vel_err = (float)bv;
                    }
                    h.corevel[k] = (float)vel;
                }
                h.bulkvel[k] = (float)vel;
                if (k == 0) h.min_bulkvel_err = (float)bv;
            }
        }
        __syncwarp(mask);
        h.pos[k + 3] = h.corevel[k];
    }
    __syncthreads();
}

__global__ void __launch_bounds__(RSG_SB) k_halo_scans_blk(rsg_halo *H, const rsg_extra_halo_info *E,
                                                           const int32_t *list, PotRec *PO,
                                                           const int32_t *toff, const int32_t *kept,
                                                           const DevCfg *Cp, int exact) {
    __shared__ BlkBuf B;
    int h = list[blockIdx.x];
    rsg_halo &hh = H[h];
    const DevCfg &C = *Cp;
    PotRec *q = PO + toff[h];
    int64_t tot = kept[h];
    corevel_blk(hh, q, tot, C);
    __syncthreads();
    float sn = (float)C.scale_now;
    const float *vc = (E[h].sub_of > -1) ? hh.corevel : hh.bulkvel;
    {
        double conv = 0.5 * (double)sn / RSG_GC;
        double hub = C.hub;
        float vv[3] = {vc[0], vc[1], vc[2]}, pp[3] = {hh.pos[0], hh.pos[1], hh.pos[2]};
        for (int64_t i = threadIdx.x; i < tot; i += blockDim.x) {
            if (q[i].ke < 0) continue;
            float ke = 0;
            for (int j = 0; j < 3; j++) {
                double dv = (double)fsub(q[i].pos[j + 3], vv[j]) +
                            hub * (double)sn * (double)fsub(q[i].pos[j], pp[j]);
                ke = (float)((double)ke + dv * dv);
            }
            q[i].ke = (float)((double)ke * conv);
        }
    }
    __syncthreads();
    more_props_blk(hh, q, tot, 0, C, B, exact);
    more_props_blk(hh, q, tot, 1, C, B, exact);
}

// halos split by size: small ones one thread each, large ones one block each
__global__ void k_scan_split(const rsg_halo *H, int32_t NH, const int32_t *kept, int32_t big,
                             int32_t *fsmall, int32_t *fbig, unsigned long long *work) {
    int h = blockIdx.x * blockDim.x + threadIdx.x;
    if (h >= NH) return;
    bool act = H[h].num_p >= 1;
    fbig[h] = act && kept[h] > big;
    fsmall[h] = act && kept[h] <= big;
    if (act) {
        int b = kept[h] > big ? 0 : 1;
        atomicAdd(&work[b], (unsigned long long)kept[h]);
        atomicAdd(&work[2 + b], 1ull);
    }
}
__global__ void k_halo_scans_list(rsg_halo *H, const rsg_extra_halo_info *E, const int32_t *list,
                                  int32_t n, PotRec *PO, const int32_t *toff, const int32_t *kept,
                                  const DevCfg *Cp) {
    int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= n) return;
    int h = list[t];
    rsg_halo &hh = H[h];
    const DevCfg &C = *Cp;
    PotRec *q = PO + toff[h];
    int64_t tot = kept[h];
    corevel(hh, q, tot, C);
    float sn = (float)C.scale_now;
    if (E[h].sub_of > -1) kinetic(q, tot, hh.corevel, hh.pos, sn, C);
    else kinetic(q, tot, hh.bulkvel, hh.pos, sn, C);
    more_props(hh, q, tot, 0, C);
    more_props(hh, q, tot, 1, C);
}

__global__ void k_bh_roots(const int32_t *toff, const int32_t *tot, int32_t NH, int32_t *rflag) {
    int h = blockIdx.x * blockDim.x + threadIdx.x;
    if (h < NH) rflag[h] = tot[h] > 1;
}
__global__ void k_bh_root_arrays(const int32_t *hlist, int32_t nr, const int32_t *toff,
                                 const int32_t *tot, int32_t *rs, int32_t *rn) {
    int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= nr) return;
    rs[k] = toff[hlist[k]];
    rn[k] = tot[hlist[k]];
}
__global__ void k_leaf_list_flags(const KNode<3> *nodes, int32_t nn, int32_t *f) {
    int a = blockIdx.x * blockDim.x + threadIdx.x;
    if (a < nn) f[a] = nodes[a].div < 0;
}

static int32_t scan_i32(Arena &ar, int32_t *in, int32_t *out, int32_t n, cudaStream_t st) {
    size_t b = 0;
    cub::DeviceScan::ExclusiveSum(nullptr, b, in, out, n, st);
    size_t m = ar.used;
    void *t = ar.take(b + 256);
    cub::DeviceScan::ExclusiveSum(t, b, in, out, n, st);
    RSG_CHECK_LAUNCH();
    ar.used = m;
    int32_t last = 0;
    RSG_CUDA(cudaMemcpyAsync(&last, out + n - 1, 4, cudaMemcpyDeviceToHost, st));
    RSG_CUDA(cudaStreamSynchronize(st));
    return last;
}
static int32_t select_idx(Arena &ar, const int32_t *flag, int32_t *out, int32_t n, cudaStream_t st) {
    int *cnt = ar.get<int>(1);
    size_t b = 0;
    cub::DeviceSelect::Flagged(nullptr, b, thrust::counting_iterator<int32_t>(0), flag, out, cnt, n, st);
    size_t m = ar.used;
    void *t = ar.take(b + 256);
    cub::DeviceSelect::Flagged(t, b, thrust::counting_iterator<int32_t>(0), flag, out, cnt, n, st);
    RSG_CHECK_LAUNCH();
    ar.used = m;
    int h = 0;
    RSG_CUDA(cudaMemcpyAsync(&h, cnt, 4, cudaMemcpyDeviceToHost, st));
    RSG_CUDA(cudaStreamSynchronize(st));
    return h;
}

// FP64 direct sum over every pair of each set, the reference values of the
// potential precision study (no counterpart in the reference, which only has
// the Barnes-Hut walk): pe_i += mp * sum_{j != i} 1 / max(r_ij, FORCE_RES),
// with coordinate differences, r^2 and 1/r in FP64.  One block per tile of
// RSG_DT targets of one set (tile t of set k: tof[k] <= t < tof[k + 1]);
// sources pass through shared memory RSG_DT at a time.
#define RSG_DT 256
__global__ void k_direct_tiles(const int32_t *rn, int32_t ns, int32_t *cnt) {
    int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k <= ns) cnt[k] = k < ns ? (rn[k] + RSG_DT - 1) / RSG_DT : 0;
}
__global__ void __launch_bounds__(RSG_DT) k_direct64(PotRec *PO, const int32_t *rs,
                                                     const int32_t *rn, const int32_t *tof,
                                                     int32_t ns, double mp, double force_res) {
    __shared__ double sx[RSG_DT], sy[RSG_DT], sz[RSG_DT];
    const int32_t t = blockIdx.x;
    int32_t lo = 0, hi = ns;  // last k with tof[k] <= t
    while (hi - lo > 1) {
        int32_t mid = (lo + hi) >> 1;
        if (tof[mid] <= t) lo = mid;
        else hi = mid;
    }
    const int32_t s0 = rs[lo], n = rn[lo];
    const int32_t i = (t - tof[lo]) * RSG_DT + (int32_t)threadIdx.x;
    const bool act = i < n;
    double xi = 0, yi = 0, zi = 0;
    if (act) {
        xi = PO[s0 + i].pos[0];
        yi = PO[s0 + i].pos[1];
        zi = PO[s0 + i].pos[2];
    }
    const double fr2 = force_res * force_res, ifr = 1.0 / force_res;
    double acc = 0;
    for (int32_t j0 = 0; j0 < n; j0 += RSG_DT) {
        const int32_t jj = j0 + (int32_t)threadIdx.x;
        __syncthreads();
        if (jj < n) {
            sx[threadIdx.x] = PO[s0 + jj].pos[0];
            sy[threadIdx.x] = PO[s0 + jj].pos[1];
            sz[threadIdx.x] = PO[s0 + jj].pos[2];
        }
        __syncthreads();
        const int32_t m = min(RSG_DT, n - j0), self = i - j0;
        for (int32_t q = 0; q < m; q++) {
            double dx = xi - sx[q], dy = yi - sy[q], dz = zi - sz[q];
            double r2 = fma(dz, dz, fma(dy, dy, dx * dx));
            double inv = r2 < fr2 ? ifr : rsqrt(r2);
            acc += q == self ? 0.0 : inv;
        }
    }
    if (act) PO[s0 + i].pe += mp * acc;
}

// Potentials for the segments (rs[k], rn[k]) of PO.  Every form first builds
// the Barnes-Hut forest, which permutes each segment into tree order, so the
// records come out in the same order whatever the form:
//   0  Barnes-Hut, the reference's FP64 arithmetic (node sums in order);
//   1  Barnes-Hut, FP32 terms with Kahan-compensated FP32 sums;
//   2  Barnes-Hut, FP32 terms with plain FP32 sums;
//   3  FP64 direct sum over all pairs (precision reference).
void bh_potential(Arena &ar, PotRec *PO, int64_t npo, const int32_t *rs, const int32_t *rn,
                  int32_t ntrees, double mp, double force_res, int *err, cudaStream_t st,
                  int form) {
    const int T = 256;
    if (ntrees == 0) return;
    const int exact = form == 0;
    Forest<3> F = build_forest<3, PotRec>(ar, PO, npo, rs, rn, ntrees, npo, 10, st);
    phase_mark(st, "p.bh_tree");
    if (form == 3) {
        int32_t *cnt = ar.get<int32_t>(ntrees + 1), *tof = ar.get<int32_t>(ntrees + 1);
        launch(k_direct_tiles, nblk(ntrees + 1, T), T, 0, st, rn, ntrees, cnt);
        int32_t ntiles = scan_i32(ar, cnt, tof, ntrees + 1, st);
        if (ntiles) launch(k_direct64, ntiles, RSG_DT, 0, st, PO, rs, rn, tof, ntrees, mp, force_res);
        RSG_CHECK_LAUNCH();
        phase_mark(st, "p.direct");
        return;
    }
    BHNode *B = ar.get<BHNode>(F.nnodes);
    launch(k_bh_leaf, nblk(F.nnodes, T), T, 0, st, F.nodes, F.nnodes, PO, mp, B);
    // batched form: the nodes of more than bh_huge points, by level, and
    // their chunks (node ids ascend with the level index in the forest)
    const int huge = tuning().bh_huge, chunk = tuning().bh_chunk;
    std::vector<int32_t> hn_node, hn_first(1, 0);  // per huge node: id, first item
    std::vector<int2> hitem;
    int2 *d_item = nullptr;
    int32_t *d_hnode = nullptr, *d_hfirst = nullptr;
    double2 *d_part = nullptr;
    if (!exact) {
        int32_t *hf = ar.get<int32_t>(F.nnodes), *hid = ar.get<int32_t>(F.nnodes);
        launch(k_bh_huge_flags, nblk(F.nnodes, T), T, 0, st, F.nodes, F.nnodes, huge, hf);
        int32_t nh = select_idx(ar, hf, hid, F.nnodes, st);
        if (nh) {
            int32_t *hsz = ar.get<int32_t>(nh);
            launch(k_bh_huge_sizes, nblk(nh, T), T, 0, st, F.nodes, hid, nh, hsz);
            std::vector<int32_t> sz(nh);
            hn_node.resize(nh);
            RSG_CUDA(cudaMemcpyAsync(hn_node.data(), hid, 4 * nh, cudaMemcpyDeviceToHost, st));
            RSG_CUDA(cudaMemcpyAsync(sz.data(), hsz, 4 * nh, cudaMemcpyDeviceToHost, st));
            RSG_CUDA(cudaStreamSynchronize(st));
            for (int32_t j = 0; j < nh; j++) {
                int nc = (sz[j] + chunk - 1) / chunk;
                for (int c = 0; c < nc; c++) hitem.push_back(make_int2(hn_node[j], c));
                hn_first.push_back((int32_t)hitem.size());
            }
            d_item = ar.get<int2>(hitem.size());
            d_part = ar.get<double2>(hitem.size());
            d_hnode = ar.get<int32_t>(nh);
            d_hfirst = ar.get<int32_t>(nh + 1);
            RSG_CUDA(cudaMemcpyAsync(d_item, hitem.data(), sizeof(int2) * hitem.size(),
                                     cudaMemcpyHostToDevice, st));
            RSG_CUDA(cudaMemcpyAsync(d_hnode, hn_node.data(), 4 * nh, cudaMemcpyHostToDevice, st));
            RSG_CUDA(cudaMemcpyAsync(d_hfirst, hn_first.data(), 4 * (nh + 1),
                                     cudaMemcpyHostToDevice, st));
        }
    }
    size_t hj = hn_node.size();  // huge nodes not yet done (taken from the back: deepest first)
    for (int l = F.nlv - 2; l >= 0; l--) {
        int32_t a = F.lv_first[l], b = F.lv_first[l + 1];
        if (b > a) {
            if (exact)
                launch(k_bh_internal, nblk(b - a, 64), 64, 0, st, F.nodes, a, b - a, PO, B);
            else
                launch(k_bh_internal_warp, nblk((int64_t)(b - a) * 32, 256), 256, 0, st, F.nodes, a,
                       b - a, PO, B);
            launch(k_bh_internal_big, b - a, 256, 0, st, F.nodes, a, b - a, PO, B, exact, huge);
            size_t j1 = hj;
            while (hj > 0 && hn_node[hj - 1] >= a) hj--;
            if (j1 > hj) {
                int32_t i0 = hn_first[hj], i1 = hn_first[j1];
                launch(k_bh_huge_part, i1 - i0, 256, 0, st, F.nodes, (const int2 *)d_item + i0,
                       chunk, PO, (const BHNode *)B, d_part + i0);
                launch(k_bh_huge_fin, nblk((int)(j1 - hj), 64), 64, 0, st, F.nodes,
                       (const int32_t *)d_hnode + hj, (const int32_t *)d_hfirst + hj,
                       (int32_t)(j1 - hj), (const double2 *)d_part, B);
            }
        }
    }
    phase_mark(st, "p.bh_mass");
    int32_t *lf = ar.get<int32_t>(F.nnodes), *leaves = ar.get<int32_t>(F.nnodes);
    launch(k_leaf_list_flags, nblk(F.nnodes, T), T, 0, st, F.nodes, F.nnodes, lf);
    int32_t nl = select_idx(ar, lf, leaves, F.nnodes, st);
    const int wb = nblk((int64_t)nl * 16, 32 * RSG_BH_WPB);
    if (form == 0)
        launch(k_bh_walk<0>, wb, 32 * RSG_BH_WPB, 0, st, F.nodes, leaves, nl, B, PO, mp, force_res,
               err);
    else if (form == 1)
        launch(k_bh_walk<1>, wb, 32 * RSG_BH_WPB, 0, st, F.nodes, leaves, nl, B, PO, mp, force_res,
               err);
    else
        launch(k_bh_walk<2>, wb, 32 * RSG_BH_WPB, 0, st, F.nodes, leaves, nl, B, PO, mp, force_res,
               err);
    RSG_CHECK_LAUNCH();
    phase_mark(st, "p.bh_walk");
}

// Batched property scans of every halo (kernels in props_seg.cuh).
static void seg_count(const Chunk *CH, int32_t nc, int32_t NH, const int32_t *c0,
                      const int32_t *nch, const uint8_t *flag, CP *cp, int32_t *cnt,
                      cudaStream_t st) {
    launch(k_sg_cnt_chunk, nc, RSG_CT, 0, st, CH, flag, cp);
    launch(k_sg_cnt_off, nblk(NH, 128), 128, 0, st, NH, c0, nch, cp);
    launch(k_sg_cnt_scan, nc, RSG_CT, 0, st, CH, flag, (const CP *)cp, cnt);
}

static void seg_props(Arena &ar, const DevCfg &dc, const DevCfg *d_dc, PotRec *PO, int32_t npo,
                      rsg_halo *H, const rsg_extra_halo_info *E, int32_t NH,
                      const int32_t *toff, const int32_t *kept, cudaStream_t st) {
    const int HT = 128;
    const int HB = nblk(NH, HT);
    size_t mark = ar.used;
    int32_t *nch = ar.get<int32_t>(NH + 1), *c0 = ar.get<int32_t>(NH + 1);
    launch(k_sg_nch, nblk(NH + 1, HT), HT, 0, st, H, NH, kept, nch);
    int32_t nc = scan_i32(ar, nch, c0, NH + 1, st);
    HS *S = ar.get<HS>(NH);
    Chunk *CH = ar.get<Chunk>(nc + 1);
    CP *cp = ar.get<CP>(nc + 1);
    uint8_t *flag = ar.get<uint8_t>(npo + 1), *flag2 = ar.get<uint8_t>(npo + 1);
    int32_t *cnt = ar.get<int32_t>(npo + 1), *cnt2 = ar.get<int32_t>(npo + 1);
    double *g = ar.get<double>(npo + 1);
    float *vel = ar.get<float>(3 * (size_t)npo + 3);
    launch(k_sg_fill, HB, HT, 0, st, NH, toff, kept, c0, nch, CH);
    // calculate_corevel, then the kinetic energies
    launch(k_cv_rmax, nc, RSG_CT, 0, st, CH, PO, d_dc, cp);
    launch(k_cv_fin1, HB, HT, 0, st, NH, H, c0, nch, cp, S);
    launch(k_cv_cmax, nc, RSG_CT, 0, st, CH, PO, toff, S, cp);
    launch(k_cv_fin2, HB, HT, 0, st, NH, H, c0, nch, cp, PO, toff, S);
    launch(k_cv_sums, nc, RSG_CT, 0, st, CH, PO, S, cp);
    launch(k_cv_off, HB, HT, 0, st, NH, H, c0, nch, S, cp);
    launch(k_cv_scan, nc, RSG_CT, 0, st, CH, PO, S, cp, g, vel);
    launch(k_cv_fin3, HB, HT, 0, st, NH, H, c0, nch, cp, S, toff, g, vel);
    launch(k_sg_kinetic, nc, RSG_CT, 0, st, CH, PO, H, E, d_dc);
    phase_mark(st, "p.corevel");
    // _calc_additional_halo_props for bound = 0 and 1; only the pass whose
    // fields are kept ((!bound) == (!BOUND_PROPS)) runs beyond the masses
    for (int bound = 0; bound < 2; bound++) {
        bool want = ((!bound) == (!dc.bound_props));
        launch(k_sg_flag, nc, RSG_CT, 0, st, CH, PO, S, bound, 0, flag);
        seg_count(CH, nc, NH, c0, nch, flag, cp, cnt, st);
        launch(k_sg_p1, nc, RSG_CT, 0, st, CH, PO, flag, cnt, d_dc, cp);
        launch(k_sg_p1_fin, HB, HT, 0, st, NH, H, c0, nch, cp, d_dc, bound, S);
        if (!want) continue;
        launch(k_sg_vmax, nc, RSG_CT, 0, st, CH, PO, flag, cnt, S, d_dc, cp);
        launch(k_sg_vmax_fin, HB, HT, 0, st, NH, H, c0, nch, cp, PO, toff, d_dc, S);
        launch(k_sg_p2, nc, RSG_CT, 0, st, CH, PO, H, flag, cnt, S, cp);
        launch(k_sg_p2_fin, HB, HT, 0, st, NH, H, c0, nch, cp, S);
        launch(k_sg_v2, nc, RSG_CT, 0, st, CH, PO, flag, S, cp);
        launch(k_sg_v2_fin, HB, HT, 0, st, NH, H, c0, nch, cp, PO, toff, d_dc, S);
        phase_mark(st, "p.passes");
        for (int which = 0; which < 2; which++) {
            launch(k_sh_init, HB, HT, 0, st, NH, H, cnt, toff, d_dc, which, S);
            launch(k_sh_small, nblk(NH, 128), 128, 0, st, NH, H, toff,
                   (const PotRec *)PO, d_dc, (const HS *)S, bound);
            for (int64_t i = 0; i < dc.shape_iterations; i++) {
                launch(k_sh_sum, nc, RSG_CT, 0, st, CH, PO, H, flag, S, d_dc, cp);
                launch(k_sh_fin, HB, HT, 0, st, NH, H, c0, nch, cp, S);
            }
        }
        phase_mark(st, "p.shape");
        launch(k_sg_flag, nc, RSG_CT, 0, st, CH, PO, S, bound, 1, flag2);
        seg_count(CH, nc, NH, c0, nch, flag2, cp, cnt2, st);
        launch(k_sg_energy, nc, RSG_CT, 0, st, CH, PO, flag2, cnt2, d_dc, cp);
        launch(k_sg_energy_fin, HB, HT, 0, st, NH, H, c0, nch, cp, S);
        launch(k_nfw_init, HB, HT, 0, st, NH, H, cnt, toff, d_dc, S);
        launch(k_nfw_bins, nc, RSG_CT, 0, st, CH, PO, flag, cnt, S);
        launch(k_nfw_fit, HB, HT, 0, st, NH, H, d_dc, S);
        launch(k_sg_pseudo, nc, RSG_CT, 0, st, CH, PO, H, flag, cnt, cp);
        launch(k_sg_final, HB, HT, 0, st, NH, H, c0, nch, cp, d_dc, S);
        phase_mark(st, "p.final");
    }
    RSG_CHECK_LAUNCH();
    ar.used = mark;
}

// Potential form of the batched path (bh_potential's forms 0-3; the plain
// path always uses form 0), process-wide, set by rsg_set_potential_form.
static std::atomic<int> g_pot_form{1};
int batched_potential_form() { return g_pot_form.load(std::memory_order_relaxed); }
int set_batched_potential_form(int f) { return g_pot_form.exchange(f); }

// When g_keep_po is set (rsg_keep_halo_records), the potential records of
// this host thread's last additional_props call (sorted by halo, then
// potential-only last, then radius; pe and ke final) are kept in g_dbg_po.
std::atomic<bool> g_keep_po{false};
thread_local std::vector<PotRec> g_dbg_po;

void additional_props(Arena &ar, const DevCfg &dc, const DevCfg *d_dc, const Rec *W,
                      int64_t M, rsg_halo *H, rsg_extra_halo_info *E, int32_t NH,
                      cudaStream_t st, int exact) {
    const int T = 256;
    if (NH == 0) return;
    size_t mark = ar.used;
    int *err = ar.get<int>(2);
    RSG_CUDA(cudaMemsetAsync(err, 0, 8, st));
    loop_limit_reset(st);
    unsigned long long *work = ar.get<unsigned long long>(4);
    RSG_CUDA(cudaMemsetAsync(work, 0, 32, st));
    int32_t *tot = ar.get<int32_t>(NH + 1), *nseg = ar.get<int32_t>(NH + 1);
    int32_t *toff = ar.get<int32_t>(NH + 1), *soff = ar.get<int32_t>(NH + 1);
    int32_t *kept = ar.get<int32_t>(NH + 1);
    const int segmax = tuning().seg_max;
    launch(k_set_count, nblk(NH + 1, 64), 64, 0, st, H, E, NH, dc.include_host_potential_ratio,
           segmax, tot, nseg, kept, err);
    check_i32_total(ar, tot, NH + 1, "potential records", st);
    int32_t npo = scan_i32(ar, tot, toff, NH + 1, st);
    phase_mark(st, "p.sets");
    int32_t ns = scan_i32(ar, nseg, soff, NH + 1, st);
    Seg *segs = ar.get<Seg>(ns + 1);
    PotRec *PO = ar.get<PotRec>(npo + 1), *PO2 = ar.get<PotRec>(npo + 1);
    launch(k_set_segs, nblk(NH, 64), 64, 0, st, H, E, NH, dc.include_host_potential_ratio, segmax,
           toff, soff, segs);
    if (ns) launch(k_set_fill, ns, 128, 0, st, segs, W, H, PO);
    RSG_CHECK_LAUNCH();
    // potentials
    {
        size_t m2 = ar.used;
        int32_t *rflag = ar.get<int32_t>(NH), *hl = ar.get<int32_t>(NH);
        launch(k_bh_roots, nblk(NH, T), T, 0, st, toff, tot, NH, rflag);
        int32_t nr = select_idx(ar, rflag, hl, NH, st);
        int32_t *rs = ar.get<int32_t>(nr + 1), *rn = ar.get<int32_t>(nr + 1);
        if (nr) launch(k_bh_root_arrays, nblk(nr, T), T, 0, st, hl, nr, toff, tot, rs, rn);
        bh_potential(ar, PO, npo, rs, rn, nr, dc.particle_mass, dc.force_res, err, st,
                     exact ? 0 : batched_potential_form());
        ar.used = m2;
    }
    // drop potential-only records and sort every halo's records by r^2
    {
        size_t m2 = ar.used;
        uint64_t *k1 = ar.get<uint64_t>(npo + 1), *k2 = ar.get<uint64_t>(npo + 1);
        uint32_t *v1 = ar.get<uint32_t>(npo + 1), *v2 = ar.get<uint32_t>(npo + 1);
        launch(k_po_keys, nblk(npo, T), T, 0, st, PO, npo, k1, v1);
        int bits = 33;
        while ((1ll << (bits - 33)) <= NH) bits++;
        size_t b = 0;
        cub::DeviceRadixSort::SortPairs(nullptr, b, k1, k2, v1, v2, npo, 0, bits, st);
        void *t = ar.take(b + 256);
        cub::DeviceRadixSort::SortPairs(t, b, k1, k2, v1, v2, npo, 0, bits, st);
        launch(k_po_gather, nblk(npo, T), T, 0, st, PO, v2, npo, PO2);
        RSG_CHECK_LAUNCH();
        ar.used = m2;
    }
    phase_mark(st, "p.sort");
    {
        int32_t *fs = ar.get<int32_t>(NH), *fbg = ar.get<int32_t>(NH);
        int32_t *ls = ar.get<int32_t>(NH), *lb = ar.get<int32_t>(NH);
        launch(k_scan_split, nblk(NH, T), T, 0, st, H, NH, kept, 1024, fs, fbg, work);
        if (exact) {
            int32_t nsm = select_idx(ar, fs, ls, NH, st);
            int32_t nbg = select_idx(ar, fbg, lb, NH, st);
            launch(k_halo_scans_blk, nbg, RSG_SB, 0, st, H, E, lb, PO2, toff, kept, d_dc, exact);
            launch(k_halo_scans_list, nblk(nsm, 32), 32, 0, st, H, E, ls, nsm, PO2, toff, kept,
                   d_dc);
        } else {
            seg_props(ar, dc, d_dc, PO2, npo, H, E, NH, toff, kept, st);
        }
    }
    RSG_CHECK_LAUNCH();
    phase_mark(st, "p.scans");
    if (g_keep_po.load()) {
        g_dbg_po.resize(npo);
        if (npo)
            RSG_CUDA(cudaMemcpyAsync(g_dbg_po.data(), PO2, sizeof(PotRec) * npo,
                                     cudaMemcpyDeviceToHost, st));
    } else if (!g_dbg_po.empty()) {
        // the switch went off since this thread's last kept call
        std::vector<PotRec>().swap(g_dbg_po);
    }
    int herr[2];
    unsigned long long hwork[4];
    RSG_CUDA(cudaMemcpyAsync(herr, err, 8, cudaMemcpyDeviceToHost, st));
    RSG_CUDA(cudaMemcpyAsync(hwork, work, 32, cudaMemcpyDeviceToHost, st));
    RSG_CUDA(cudaStreamSynchronize(st));
    loop_limit_check(st, "halo properties");
    int64_t *S = last_stats();
    S[RSG_STAT_POT_RECORDS] = npo;
    S[RSG_STAT_KEPT_BIG] = (int64_t)hwork[0];
    S[RSG_STAT_KEPT_SMALL] = (int64_t)hwork[1];
    S[RSG_STAT_HALOS_BIG] = (int64_t)hwork[2];
    S[RSG_STAT_HALOS_SMALL] = (int64_t)hwork[3];
    if (herr[0]) {
        set_error(RSG_ERR_LIMIT, "halo walk or potential tree traversal exceeded its bound");
        throw Failure();
    }
    ar.used = mark;
}

}  // namespace rsg
