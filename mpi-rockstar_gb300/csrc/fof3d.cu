// 3D friends-of-friends with the reference's skip acceleration
// (rockstar(), src/rockstar.c:53-128; src/fof.c:112-255), reformulated so
// that every step is data parallel and the partition is identical.
//
// The reference visits particles in kd-tree order.  A particle i with more
// than FOF_SKIP_THRESH (16) neighbours inside r ("dense") marks all of them
// as skipped and merges with every particle within 2r that is already in a
// group.  Written as a function of the neighbour sets S_r(i):
//   * dense(i)      <=> |S_r(i)| > 16, a property of i alone;
//   * seeds         = the lexicographically-first maximal independent set of
//                     the dense particles in tree order (a dense particle is
//                     processed iff no earlier processed dense particle has
//                     it in its r-sphere);
//   * processed(i)  <=> no seed s < i has i in S_r(s);
//   * g(j)          = the first processed k with |S_r(k)| >= 2 and
//                     j in S_r(k): the moment j joins some group;
//   * the partition is the connected components of the links
//       {(k, j) : k processed, |S_r(k)| >= 2, j in S_r(k)}
//     plus {(s, j) : s seed, j in S_2r(s), g(j) <= s}.
// Sphere searches walk the same kd-tree with the same float tests as
// src/fast3tree.c:293-414, so S_r is the reference's set, node shortcut
// included.
#include <limits.h>

#include <cooperative_groups.h>
#include <cub/cub.cuh>
#include <thrust/binary_search.h>
#include <thrust/execution_policy.h>

#include "kdtree_impl.cuh"
#include "lsort.cuh"
#include "uflabels.cuh"

namespace rsg {

namespace cg = cooperative_groups;

// The reference's squared distance of a leaf point (dx = c[t] - q[t], dist
// += dx * dx for t = 0, 1, 2 in order, each rounded; src/fast3tree.c:
// 398-405), x and y subtracted and squared as one packed pair; cxy holds
// c[0], c[1].  dist starts at 0 and the first square is not negative, so
// 0 + dx0^2 is dx0^2.
__device__ __forceinline__ float dist3_p(unsigned long long cxy, float cz, const Rec &q) {
    const unsigned long long qxy = *reinterpret_cast<const unsigned long long *>(q.pos);
    float p0, p1;
    f2_split(f2_sqr(f2_sub(cxy, qxy)), p0, p1);
    const float dz = fsub(cz, q.pos[2]);
    return fadd(fadd(p0, p1), fmul(dz, dz));
}
// The reference's two box tests, in its operation order:
// _fast3tree_box_not_intersect_sphere and _fast3tree_box_inside_sphere
// (src/fast3tree.c:293-330).
__device__ __forceinline__ bool box_out3(const KNode<3> &nd, const float *c, float r2) {
    float d = 0.f, e;
#pragma unroll
    for (int i = 0; i < 3; i++) {
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
__device__ __forceinline__ bool box_inside3(const KNode<3> &nd, const float *c, float r,
                                            float r2) {
    if (fabsf(fsub(c[0], nd.mn[0])) > r) return false;
    float dist = 0.f;
#pragma unroll
    for (int i = 0; i < 3; i++) {
        float dx = fsub(nd.mn[i], c[i]);
        dx = fmul(dx, dx);
        float dx2 = fsub(c[i], nd.mx[i]);
        dx2 = fmul(dx2, dx2);
        if (dx2 > dx) dx = dx2;
        dist = fadd(dist, dx);
        if (dist > r2) return false;
    }
    return true;
}

// Sphere search (src/fast3tree.c:377-414) on tree `root` of a 3D forest.
// on_range(start, n) receives nodes that lie entirely inside the sphere
// (shortcut of :386-392), on_point(j) leaf points with dist < r^2.  Either
// returns false to stop the walk.  Callers that only want points after
// index `after` skip the nodes that hold none (the tests of every other node
// are unchanged, so the points found after `after` are the same).
template <class FR, class FP>
__device__ bool sphere3(const KNode<3> *nodes, int root, const Rec *recs, const float *c,
                        float r, int *errflag, FR on_range, FP on_point, int after = -1) {
    int stack[RSG_STACK];
    int sp = 0;
    stack[sp++] = root;
    const float r2 = fmul(r, r);
    while (sp) {
        const KNode<3> &nd = nodes[stack[--sp]];
        if (nd.start + nd.n <= after + 1) continue;
        if (box_out3(nd, c, r2)) continue;
        if (box_inside3(nd, c, r, r2)) {
            if (!on_range(nd.start, nd.n)) return false;
            continue;
        }
        if (nd.div < 0) {
            const unsigned long long cxy = f2_pack(c[0], c[1]);
            for (int k = 0; k < nd.n; k++) {
                int j = nd.start + k;
                if (dist3_p(cxy, c[2], recs[j]) < r2)
                    if (!on_point(j)) return false;
            }
            continue;
        }
        if (sp + 2 > RSG_STACK) {
            atomicExch(errflag, 1);
            return false;
        }
        stack[sp++] = nd.left + 1;  // right, visited after left
        stack[sp++] = nd.left;
    }
    return true;
}

// The same search for the 32 queries of a warp (one per lane, `active`
// lanes only) with one shared walk: a stack entry carries the lanes that
// still need the subtree and each lane applies its own tests, so every lane meets exactly
// the nodes and points of its own walk, in the same order.  A callback
// returning false ends that lane's walk; nodes holding no index after the
// lane's `after` are dropped for that lane (the points it finds after
// `after` are unchanged).
// on_leaf(j, hit), when given (LEAF = true), replaces on_point for leaf
// points: every lane calls it for every point of a leaf any lane tests, in
// converged code, with hit telling whether the point is in this lane's
// sphere (warp-level ballots inside it are safe).  It cannot end a walk.
struct NoLeaf {
    __device__ void operator()(int, bool) const {}
};
// on_coop(m2, start, n), when given (COOP = true), replaces on_range: every
// lane calls it, in converged code, for a node that the lanes of mask m2 take
// whole (all of them meet the same node in a shared walk), so the warp can
// work through the node's points together.  It cannot end a walk.
struct NoCoop {
    __device__ void operator()(unsigned, int, int) const {}
};
template <class FR, class FP, bool LEAF = false, class FL = NoLeaf, bool COOP = false,
          class FC = NoCoop>
__device__ void sphere3_warp(const KNode<3> *nodes, const Rec *recs, const float *c, bool active,
                             float r, int after, int *errflag, FR on_range, FP on_point,
                             FL on_leaf = FL(), FC on_coop = FC()) {
    const unsigned FULL = 0xffffffffu;
    const unsigned bit = 1u << (threadIdx.x & 31);
    const float r2 = fmul(r, r);
    int sn[RSG_STACK];
    unsigned sm[RSG_STACK];
    unsigned live = __ballot_sync(FULL, active);
    if (!live) return;
    int sp = 0;
    sn[sp] = 0;
    sm[sp++] = live;
    while (sp) {
        --sp;
        const int xi = sn[sp];
        const unsigned m = sm[sp] & live;
        if (!m) continue;
        const KNode<3> &nd = nodes[xi];
        int kind = 0;  // 1 out, 2 inside, 3 leaf points, 4 descend
        if (m & bit) {
            kind = 1;
            if (nd.start + nd.n > after + 1 && !box_out3(nd, c, r2))
                kind = box_inside3(nd, c, r, r2) ? 2 : (nd.div < 0 ? 3 : 4);
        }
        bool stop = false;
        if (COOP) {
            const unsigned m2 = __ballot_sync(FULL, kind == 2);
            if (m2) on_coop(m2, nd.start, nd.n);
        } else if (kind == 2) {
            stop = !on_range(nd.start, nd.n);
        }
        if (__any_sync(FULL, kind == 3)) {
            const unsigned long long cxy = f2_pack(c[0], c[1]);
            for (int k = 0; k < nd.n; k++) {
                int j = nd.start + k;
                bool hit = false;
                if (kind == 3 && !stop) hit = dist3_p(cxy, c[2], recs[j]) < r2;
                if (LEAF) on_leaf(j, hit);
                else if (hit) stop = !on_point(j);
            }
        }
        live &= ~__ballot_sync(FULL, stop);
        unsigned down = __ballot_sync(FULL, kind == 4) & live;
        if (down) {
            if (sp + 2 > RSG_STACK) {
                if (bit == 1u) atomicExch(errflag, 1);
                return;
            }
            sn[sp] = nd.left + 1;
            sm[sp++] = down;
            sn[sp] = nd.left;
            sm[sp++] = down;
        }
    }
}

// Warp-cooperative form of sphere3 for one query shared by the warp (the
// position c of particle q): every point after `after` of the reference
// walk's result set -- the points of the nodes it takes whole and the leaf
// points nearer than r -- is handed to exactly one lane.  All lanes call it
// together; every lane calls visit(j, valid) in converged code, once per
// round of up to 32 points (valid false on a lane without a point), so
// warp-level operations may be used inside visit.
// Down q's root-to-leaf path the reference walk only descends until a node
// it takes whole or whose other child it would enter (not out by its test,
// holding an index after `after`); the warp starts there.  From there it
// takes up to 32 nodes of a stack in shared memory per round and spreads
// the points of the whole nodes and leaves met over its lanes.  The set of
// points is the walk's; the order is not (the reference's is ascending
// index, left subtree first).  The stack takes 32 nodes at a time while 64
// slots and a tree depth of margin are free, one at a time otherwise
// (depth-first growth is bounded by the tree depth); a tree deeper than
// RSG_STACK sets errflag, as the scalar walk does.
#define RSG_WSTK 1024
template <class FV>
__device__ void warp_sphere3(const KNode<3> *nodes, const Rec *recs, int q, const float *c,
                             float r, int after, int *S, int *errflag, FV visit) {
    const unsigned FULL = 0xffffffffu;
    const int lane = threadIdx.x & 31;
    const unsigned below = (1u << lane) - 1u;
    const float r2 = fmul(r, r);
    int x = 0;
    for (int depth = 0; depth < RSG_STACK; depth++) {
        const KNode<3> &nd = nodes[x];
        if (nd.div < 0 || box_inside3(nd, c, r, r2)) break;
        const KNode<3> &L = nodes[nd.left];
        const bool inL = q < L.start + L.n;
        const KNode<3> &O = inL ? nodes[nd.left + 1] : L;
        if (O.start + O.n > after + 1 && !box_out3(O, c, r2)) break;
        x = inL ? nd.left : nd.left + 1;
    }
    __syncwarp();
    if (lane == 0) S[0] = x;
    int sp = 1;
    __syncwarp();
    while (sp > 0) {
        const int take = (sp + 64 <= RSG_WSTK - RSG_STACK) ? min(sp, 32) : 1;
        const int xi = lane < take ? S[sp - 1 - lane] : -1;
        sp -= take;
        __syncwarp();
        // 0 nothing, 1 whole node, 2 leaf points, 3 descend
        int kind = 0, s0 = 0, m0 = 0, left = 0;
        if (xi >= 0) {
            const KNode<3> &nd = nodes[xi];
            if (nd.start + nd.n > after + 1 && !box_out3(nd, c, r2)) {
                kind = box_inside3(nd, c, r, r2) ? 1 : (nd.div < 0 ? 2 : 3);
                s0 = nd.start;
                m0 = nd.n;
                left = nd.left;
            }
        }
        const unsigned dm = __ballot_sync(FULL, kind == 3);
        const int room = (RSG_WSTK - sp) >> 1;  // child pairs that fit
        if (kind == 3 && __popc(dm & below) < room) {
            const int at = sp + 2 * __popc(dm & below);
            S[at] = left + 1;
            S[at + 1] = left;
        }
        if (__popc(dm) > room) {
            if (lane == 0) atomicExch(errflag, 1);
            return;
        }
        sp += 2 * __popc(dm);
        // the points after `after` of this round's whole nodes and leaves
        const bool pts = kind == 1 || kind == 2;
        const int a0 = pts ? max(s0, after + 1) : 0;
        const int np = pts ? max(0, s0 + m0 - a0) : 0;
        int incl = np;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const int v = __shfl_up_sync(FULL, incl, o);
            if (lane >= o) incl += v;
        }
        const int total = __shfl_sync(FULL, incl, 31);
        for (int base = 0; base < total; base += 32) {
            const int flat = base + lane;
            int o = 0;
#pragma unroll
            for (int step = 16; step >= 1; step >>= 1) {
                const int v = __shfl_sync(FULL, incl, o + step - 1);
                if (v <= flat) o += step;
            }
            const int oi = __shfl_sync(FULL, incl, o), on = __shfl_sync(FULL, np, o);
            const int oa = __shfl_sync(FULL, a0, o), ok = __shfl_sync(FULL, kind, o);
            int j = -1;
            bool v = false;
            if (flat < total) {
                j = oa + (flat - (oi - on));
                v = true;
                if (ok == 2) v = dist3_p(f2_pack(c[0], c[1]), c[2], recs[j]) < r2;
            }
            visit(j, v);
        }
        __syncwarp();
    }
}

// ---- kernels --------------------------------------------------------------
__global__ void k_make_recs(const rsg_particle *p, int64_t n, Rec *recs, int *bad) {
    int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= n) return;
    Rec r;
    bool fin = true;
#pragma unroll
    for (int d = 0; d < 6; d++) {
        r.pos[d] = p[i].pos[d];
        fin &= isfinite(r.pos[d]);
    }
    r.ridx = (int32_t)i;
    r.aux = 0;
    recs[i] = r;
    if (!fin) atomicExch(bad, 1);
}

// Duplicate candidates: a particle equal (bitwise position, or id) to its
// successor in tree order (src/rockstar.c:379-389 compares with the next
// kept particle, which is the successor whenever nothing was removed).
__global__ void k_dup_probe(const Rec *recs, const rsg_particle *p, int64_t n, int *any) {
    int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i + 1 >= n) return;
    const Rec &a = recs[i], &b = recs[i + 1];
    bool same = true;
#pragma unroll
    for (int d = 0; d < 6; d++) same &= (__float_as_uint(a.pos[d]) == __float_as_uint(b.pos[d]));
    if (same || p[a.ridx].id == p[b.ridx].id) atomicExch(any, 1);
}

// Sequential duplicate removal, only run when k_dup_probe found one.
__global__ void k_dedupe_serial(Rec *recs, const rsg_particle *p, int64_t n, int64_t *n_out) {
    if (blockIdx.x || threadIdx.x) return;
    if (n < 2) { *n_out = n; return; }
    int64_t last = n - 1;
    for (int64_t i = n - 2; i >= 0; i--) {
        bool same = true;
        for (int d = 0; d < 6; d++)
            same &= (__float_as_uint(recs[i].pos[d]) == __float_as_uint(recs[last].pos[d]));
        if (same || p[recs[last].ridx].id == p[recs[i].ridx].id) {
            n--;
            recs[i] = recs[n];
            continue;
        }
        last = i;
    }
    *n_out = n;
}

// Warp forms of the searches: queries are list[0..nq) (ascending particle
// indices, so a warp's queries are neighbours in the tree), or all
// particles when list is null.
__device__ __forceinline__ bool warp_query(const int *list, int nq, int *q) {
    int t = blockIdx.x * blockDim.x + threadIdx.x;
    *q = (t < nq) ? (list ? list[t] : t) : -1;
    return *q >= 0;
}
__device__ __forceinline__ bool warp_idle(int nq) {
    return (int64_t)blockIdx.x * blockDim.x + (threadIdx.x & ~31u) >= nq;
}
// |S_r(i)| capped at 17 (the reference only asks whether it exceeds 16)
__global__ void __launch_bounds__(128) k_count_w(const KNode<3> *nodes, const Rec *recs, int n,
                                                 float r, uint8_t *cnt, int *err) {
    if (warp_idle(n)) return;
    int i;
    bool act = warp_query(nullptr, n, &i);
    float c[3] = {0, 0, 0};
    if (act) { c[0] = recs[i].pos[0]; c[1] = recs[i].pos[1]; c[2] = recs[i].pos[2]; }
    int k = 0;
    sphere3_warp(
        nodes, recs, c, act, r, -1, err,
        [&](int s, int m) { k += m; return k <= 16; },
        [&](int j) { k++; return k <= 16; });
    if (act) cnt[i] = (uint8_t)(k > 17 ? 17 : k);
}
// Later dense neighbours of every dense particle k (j > k, j in S_r(k)),
// counted then listed; skipcnt[j] counts the dense k that can skip j.
// With llist, k's entries go to llist[loff[k] - lbase ...] (lbase: the
// offset of the first particle of the chunk being listed).
// The counting pass takes whole nodes together (the lanes meeting a node
// share it): each lane counts its later dense points from the prefix count
// dpfx (dense particles before an index), and the lanes stride over the
// node's points, each dense point j getting one atomic that adds the number
// of queries below j (the queries ascend with the lane, so those lanes are a
// prefix of the warp).
template <bool FILL>
__global__ void __launch_bounds__(128) k_llist_w(const KNode<3> *nodes, const Rec *recs,
                                                 const int *dense, int nd, float r,
                                                 const uint8_t *cnt, const int *dpfx,
                                                 const int64_t *loff, int64_t lbase, int *lcnt,
                                                 int *llist, int *skipcnt, int *err) {
    if (warp_idle(nd)) return;
    int k;
    bool act = warp_query(dense, nd, &k);
    float c[3] = {0, 0, 0};
    if (act) { c[0] = recs[k].pos[0]; c[1] = recs[k].pos[1]; c[2] = recs[k].pos[2]; }
    int m = 0;
    int64_t base = (loff && act) ? loff[k] - lbase : 0;
    auto add = [&](int j) {
        if (j > k && cnt[j] > 16) {
            if (llist) llist[base + m] = j;
            else atomicAdd(&skipcnt[j], 1);
            m++;
        }
    };
    // leaf points: the warp's lanes that count the same point j add their
    // counts to skipcnt[j] with one atomic
    const unsigned lane = threadIdx.x & 31;
    auto leaf = [&](int j, bool hit) {
        bool inc = hit && j > k && cnt[j] > 16;
        if (llist) {
            if (inc) llist[base + m] = j;
        } else {
            unsigned b = __ballot_sync(0xffffffffu, inc);
            if (b && lane == (unsigned)(__ffs(b) - 1)) atomicAdd(&skipcnt[j], __popc(b));
        }
        m += inc;
    };
    auto range = [&](int s, int q) {
        for (int j = s; j < s + q; j++) add(j);
        return true;
    };
    auto point = [&](int j) {
        add(j);
        return true;
    };
    const int kq = act ? k : INT_MAX;
    auto coop = [&](unsigned m2, int s, int q) {
        if ((m2 >> lane) & 1u) {
            const int a = max(s, k + 1);
            if (a < s + q) m += dpfx[s + q] - dpfx[a];
        }
        const int k31 = __shfl_sync(0xffffffffu, kq, 31);
        for (int b = 0; b < q; b += 32) {
            const int j = s + b + lane;
            int p = 0;  // lanes whose query is below j
#pragma unroll
            for (int step = 16; step >= 1; step >>= 1)
                if (__shfl_sync(0xffffffffu, kq, p + step - 1) < j) p += step;
            if (p == 31 && k31 < j) p = 32;
            const int c2 = __popc(m2 & (p >= 32 ? 0xffffffffu : ((1u << p) - 1u)));
            if (j < s + q && c2 && cnt[j] > 16) atomicAdd(&skipcnt[j], c2);
        }
    };
    sphere3_warp<decltype(range), decltype(point), true, decltype(leaf), !FILL,
                 decltype(coop)>(nodes, recs, c, act, r, act ? k : INT_MAX - 1, err, range,
                                 point, leaf, coop);
    if (act && !llist) lcnt[k] = m;
}
// The seeds' searches run one warp per seed (warp_sphere3): a seed's
// spheres hold hundreds to thousands of points, and its neighbours in tree
// order are mostly skipped particles with no search of their own, so a
// thread per particle would leave the warp to one lane.
#define RSG_SEED_WARPS 4
#define SEED_LOOP(ns)                                                                  \
    for (int t = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; t < (ns);               \
         t += (gridDim.x * blockDim.x) >> 5)
// every point after seed s of S_r(s) is skipped (src/rockstar.c:75-77)
__global__ void __launch_bounds__(RSG_SEED_WARPS * 32)
    k_seed_mark_w(const KNode<3> *nodes, const Rec *recs, const int *seeds, int ns, float r,
                  uint8_t *skipped, int *err) {
    __shared__ int stk[RSG_SEED_WARPS][RSG_WSTK];
    int *S = stk[threadIdx.x >> 5];
    SEED_LOOP(ns) {
        const int k = seeds[t];
        const float c[3] = {recs[k].pos[0], recs[k].pos[1], recs[k].pos[2]};
        warp_sphere3(nodes, recs, k, c, r, k, S, err, [&](int j, bool v) {
            if (v) skipped[j] = 1;
        });
    }
}
// g(j) over the seeds' spheres (see k_gtime_r)
__global__ void __launch_bounds__(RSG_SEED_WARPS * 32)
    k_gtime_seed_w(const KNode<3> *nodes, const Rec *recs, const int *seeds, int ns, float r,
                   int *gtime, int *err) {
    __shared__ int stk[RSG_SEED_WARPS][RSG_WSTK];
    int *S = stk[threadIdx.x >> 5];
    SEED_LOOP(ns) {
        const int k = seeds[t];
        const float c[3] = {recs[k].pos[0], recs[k].pos[1], recs[k].pos[2]};
        warp_sphere3(nodes, recs, k, c, r, -1, S, err, [&](int j, bool v) {
            if (v) atomicMin(&gtime[j], k);
        });
    }
}
// f(k) of the seeds (see k_fptr3): the first particle of S_r(k) in walk
// order -- the smallest index -- labelled before k
__global__ void __launch_bounds__(RSG_SEED_WARPS * 32)
    k_fptr_seed_w(const KNode<3> *nodes, const Rec *recs, const int *seeds, int ns, float r,
                  const int *gtime, int *ptr, int *err) {
    __shared__ int stk[RSG_SEED_WARPS][RSG_WSTK];
    int *S = stk[threadIdx.x >> 5];
    const int lane = threadIdx.x & 31;
    SEED_LOOP(ns) {
        const int k = seeds[t];
        const int gk = gtime[k];
        if (gk < k) {
            if (lane == 0) ptr[k] = gk;
            continue;
        }
        const float c[3] = {recs[k].pos[0], recs[k].pos[1], recs[k].pos[2]};
        int best = INT_MAX;
        warp_sphere3(nodes, recs, k, c, r, -1, S, err, [&](int j, bool v) {
            if (v && j < best && gtime[j] < k) best = j;
        });
        best = __reduce_min_sync(0xffffffffu, best);
        if (lane == 0) ptr[k] = best == INT_MAX ? k : gtime[best];
    }
}
// Candidate merges of the seeds (see k_cand3): both spheres, S_r(k) with
// the particles labelled before k, then S_2r(k) with those labelled by k.
// A label is emitted once per sphere at its first occurrence in walk order
// (the smallest index, which is the key's last field): a per-warp hash
// table keeps the smallest index of every label met; a label that finds no
// slot is emitted at every occurrence (a repeat is a no-op merge).
#define RSG_CAND_HT 128
__device__ __forceinline__ void cand_emit(int k, int phase, int j, int F, int W, int64_t cap,
                                          unsigned long long *count, uint64_t *ckey, int32_t *cF,
                                          int32_t *cW) {
    cg::coalesced_group g = cg::coalesced_threads();
    unsigned long long base = 0;
    if (g.thread_rank() == 0) base = atomicAdd(count, (unsigned long long)g.size());
    const unsigned long long u = g.shfl(base, 0) + g.thread_rank();
    if ((int64_t)u < cap) {
        ckey[u] = ((uint64_t)(uint32_t)k << 32) | ((uint64_t)phase << 31) | (uint32_t)j;
        cF[u] = F;
        cW[u] = W;
    }
}
__global__ void __launch_bounds__(RSG_SEED_WARPS * 32)
    k_cand_seed_w(const KNode<3> *nodes, const Rec *recs, const int *seeds, int ns, float r,
                  float r2x, const int *gtime, const int32_t *lab0, const int32_t *sfid,
                  int64_t cap, unsigned long long *count, uint64_t *ckey, int32_t *cF,
                  int32_t *cW, int *err) {
    __shared__ int stk[RSG_SEED_WARPS][RSG_WSTK];
    __shared__ int hk[RSG_SEED_WARPS][RSG_CAND_HT], hv[RSG_SEED_WARPS][RSG_CAND_HT];
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    int *S = stk[w], *K = hk[w], *Vv = hv[w];
    SEED_LOOP(ns) {
        const int k = seeds[t];
        const int F = sfid[k];
        const float c[3] = {recs[k].pos[0], recs[k].pos[1], recs[k].pos[2]};
        for (int phase = 0; phase < 2; phase++) {
            for (int e = lane; e < RSG_CAND_HT; e += 32) {
                K[e] = -1;
                Vv[e] = INT_MAX;
            }
            __syncwarp();
            warp_sphere3(nodes, recs, k, c, phase ? r2x : r, -1, S, err, [&](int j, bool v) {
                if (!v) return;
                const int gj = gtime[j];
                if (!(phase == 0 ? gj < k : gj <= k)) return;
                const int W = lab0[j];
                if (W == F) return;
                const unsigned h = ((unsigned)W * 2654435761u) >> 25;  // 7 bits
                for (int pr = 0; pr < 8; pr++) {
                    const int e = (h + pr) & (RSG_CAND_HT - 1);
                    const int old = atomicCAS(&K[e], -1, W);
                    if (old == -1 || old == W) {
                        atomicMin(&Vv[e], j);
                        return;
                    }
                }
                cand_emit(k, phase, j, F, W, cap, count, ckey, cF, cW);
            });
            __syncwarp();
            for (int e = lane; e < RSG_CAND_HT; e += 32)
                if (K[e] != -1) cand_emit(k, phase, Vv[e], F, K[e], cap, count, ckey, cF, cW);
            __syncwarp();
        }
    }
}

// g(j): the first processed particle k with |S_r(k)| >= 2 (in tree order)
// whose r-sphere holds j -- the moment link_particle_to_fof gives j its
// label (src/fof.c:112-140).
__global__ void k_gtime_r(const KNode<3> *nodes, const Rec *recs, int n, float r,
                          const uint8_t *cnt, const uint8_t *skipped, const uint8_t *state,
                          int *gtime, int *err) {
    int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n || skipped[k] || cnt[k] < 2 || state[k] == 1) return;  // seeds: k_gtime_seed_w
    float c[3] = {recs[k].pos[0], recs[k].pos[1], recs[k].pos[2]};
    sphere3(
        nodes, 0, recs, c, r, err,
        [&](int a, int m) {
            for (int j = a; j < a + m; j++) atomicMin(&gtime[j], k);
            return true;
        },
        [&](int j) {
            atomicMin(&gtime[j], k);
            return true;
        });
}

// f(k), the set event k works on (src/fof.c:116-131): k's own label when an
// earlier event gave it one, else the label of the first particle of S_r(k)
// (walk order) labelled before k, else a new set (ptr = k).  -1: no event.
__global__ void k_fptr3(const KNode<3> *nodes, const Rec *recs, int n, float r,
                        const uint8_t *cnt, const uint8_t *skipped, const uint8_t *state,
                        const int *gtime, int *ptr, int *err) {
    int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n || state[k] == 1) return;  // seeds: k_fptr_seed_w
    if (skipped[k] || cnt[k] < 2) {
        ptr[k] = -1;
        return;
    }
    int gk = gtime[k];
    if (gk < k) {
        ptr[k] = gk;
        return;
    }
    int p = k;
    float c[3] = {recs[k].pos[0], recs[k].pos[1], recs[k].pos[2]};
    sphere3(
        nodes, 0, recs, c, r, err,
        [&](int a, int m) {
            for (int j = a; j < a + m; j++)
                if (gtime[j] < k) {
                    p = gtime[j];
                    return false;
                }
            return true;
        },
        [&](int j) {
            if (gtime[j] < k) {
                p = gtime[j];
                return false;
            }
            return true;
        });
    ptr[k] = p;
}

// Candidate merges of event k in walk order: for every particle of S_r(k)
// labelled before k, link_particle_to_fof joins f(k)'s set to that
// particle's set (src/fof.c:133-139); a seed then does the same for every
// particle of S_2r(k) labelled by then (link_fof_to_fof, src/fof.c:142-158,
// k_cand_seed_w).  A label equal to f(k), or one this event already
// emitted, changes nothing and is skipped.  Keys order the candidates in
// time: (k, sphere, position in the result list), the position being the
// particle index (the walk lists points in ascending index order).
#define RSG_CAND_SEEN 8
__global__ void k_cand3(const KNode<3> *nodes, const Rec *recs, int n, float r,
                        const uint8_t *cnt, const uint8_t *skipped, const uint8_t *state,
                        const int *gtime, const int32_t *lab0, const int32_t *sfid, int64_t cap,
                        unsigned long long *count, uint64_t *ckey, int32_t *cF, int32_t *cW,
                        int *err) {
    int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n || skipped[k] || cnt[k] < 2 || state[k] == 1) return;  // seeds: k_cand_seed_w
    const int F = sfid[k];
    int seen[RSG_CAND_SEEN];
    int ns = 0;
    auto visit = [&](int j) {
        int gj = gtime[j];
        if (gj < k) {
            int W = lab0[j];
            bool dup = (W == F);
            for (int q = 0; q < ns; q++) dup |= (seen[q] == W);
            if (!dup) {
                if (ns < RSG_CAND_SEEN) seen[ns++] = W;
                unsigned long long t = atomicAdd(count, 1ull);
                if ((int64_t)t < cap) {
                    ckey[t] = ((uint64_t)(uint32_t)k << 32) | (uint32_t)j;
                    cF[t] = F;
                    cW[t] = W;
                }
            }
        }
    };
    float c[3] = {recs[k].pos[0], recs[k].pos[1], recs[k].pos[2]};
    sphere3(
        nodes, 0, recs, c, r, err,
        [&](int a, int m) {
            for (int j = a; j < a + m; j++) visit(j);
            return true;
        },
        [&](int j) {
            visit(j);
            return true;
        });
}

// The ordered independent set of the dense particles (the seeds), decided
// frontier by frontier.  Every dense particle enters the queue once, when it
// is decided (or, for a particle decided beyond the chunk being walked, when
// its own chunk starts); a frontier is queue[head, tail).  One warp walks the
// later list of each frontier particle k: a seed marks its later neighbours
// as skipped, and every decided particle releases one pending earlier
// neighbour of each.  A particle with none pending that was not skipped is a
// seed (all its earlier potential skippers are decided and none of them is
// a seed).  When the lists are built one chunk of particles [c0, cend) at a
// time (lbase = loff[c0]), a particle decided beyond cend has no list yet:
// it keeps its state and enters the first frontier of its own chunk.
struct KahnCtl {
    int head, tail, next, iters, hit, overflow, cend, pad;
    int64_t lbase;
};
struct KahnList {
    const int64_t *loff;
    const int *llist;
    int *queue, qcap;
    KahnCtl *ctl;
    int *state, *skipcnt;
};
__device__ __forceinline__ void kahn_push(int *queue, int qcap, KahnCtl *ctl, int j) {
    cg::coalesced_group g = cg::coalesced_threads();
    int base = 0;
    if (g.thread_rank() == 0) base = atomicAdd(&ctl->next, (int)g.size());
    const int at = g.shfl(base, 0) + (int)g.thread_rank();
    if (at < qcap) queue[at] = j;
    else ctl->overflow = 1;
}
__global__ void k_kahn(KahnList L) {
    const int lane = threadIdx.x & 31;
    const int w0 = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int nw = (gridDim.x * blockDim.x) >> 5;
    const KahnCtl &C = *L.ctl;
    const int head = C.head, tail = C.tail, cend = C.cend;
    const int64_t lbase = C.lbase;
    for (int f = head + w0; f < tail; f += nw) {
        const int k = L.queue[f];
        const int sk = L.state[k];
        const int64_t e1 = L.loff[k + 1] - lbase;
        for (int64_t e = L.loff[k] - lbase + lane; e < e1; e += 32) {
            const int j = L.llist[e];
            if (sk == 1 && atomicCAS(&L.state[j], 0, 2) == 0 && j < cend)
                kahn_push(L.queue, L.qcap, L.ctl, j);
            if (atomicSub(&L.skipcnt[j], 1) == 1 && atomicCAS(&L.state[j], 0, 1) == 0 && j < cend)
                kahn_push(L.queue, L.qcap, L.ctl, j);
        }
    }
}
// Next frontier: the particles queued by the step just run.  False when
// there are none or a limit was reached.
__device__ __forceinline__ bool kahn_advance(KahnCtl *ctl, int qcap, int limit) {
    const int old = ctl->tail;
    const int nt = min(ctl->next, qcap);
    ctl->head = old;
    ctl->tail = nt;
    const int it = ++ctl->iters;
    bool more = nt > old && !ctl->overflow;
    if (more && it >= limit) {
        ctl->hit = 1;
        more = false;
    }
    return more;
}
__global__ void k_kahn_next(KahnCtl *ctl, int qcap, int limit) { kahn_advance(ctl, qcap, limit); }
__global__ void k_kahn_next_g(KahnCtl *ctl, int qcap, int limit, cudaGraphConditionalHandle h) {
    cudaGraphSetConditional(h, kahn_advance(ctl, qcap, limit) ? 1u : 0u);
}
// Dense particles with no earlier potential skipper are seeds; those before
// the first chunk's end start the first frontier.
__global__ void k_kahn_init(const int *dense, int nd, const int *skipcnt, int cend, int *state,
                            int *queue, int qcap, KahnCtl *ctl) {
    int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= nd) return;
    const int i = dense[t];
    if (skipcnt[i] == 0) {
        state[i] = 1;
        if (i < cend) kahn_push(queue, qcap, ctl, i);
    }
}
// First frontier of a later chunk: its dense particles already decided
// while earlier chunks were walked.
__global__ void k_kahn_chunk(const int *dense, int nd, const int *state, int *queue, int qcap,
                             KahnCtl *ctl) {
    int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= nd) return;
    const int i = dense[t];
    if (state[i] != 0) kahn_push(queue, qcap, ctl, i);
}
// A chunk's walk begins: its list range and the frontier queued for it.
__global__ void k_kahn_start(KahnCtl *ctl, int qcap, int cend, int64_t lbase) {
    ctl->cend = cend;
    ctl->lbase = lbase;
    ctl->head = ctl->tail;
    ctl->tail = min(ctl->next, qcap);
}
struct ChunkTarget {
    int64_t step;
    __host__ __device__ int64_t operator()(int64_t t) const { return (t + 1) * step; }
};
__global__ void k_state8(const int *s32, int n, uint8_t *s8) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) s8[i] = (uint8_t)s32[i];
}

// Label of every particle: the smallfof of the set it joined (root null),
// or the final root of that set.
__global__ void k_lab3(const int *gtime, int n, const int32_t *sfid, const int32_t *root,
                       int32_t *lab) {
    int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= n) return;
    int gj = gtime[j];
    lab[j] = (gj == 0x7f7f7f7f) ? -1 : (root ? root[sfid[gj]] : sfid[gj]);
}
__global__ void k_gather_out(const Rec *recs, const rsg_particle *in, int n, rsg_particle *out) {
    int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k < n) out[k] = in[recs[k].ridx];
}
// After the partition sort: particles without a label first, then one run
// per label in ascending order (src/fof.c:226-255 walks them in this order).
__global__ void k_run_heads3(const int32_t *lab, int n, int *head) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    head[i] = lab[i] >= 0 && (i == 0 || lab[i - 1] != lab[i]);
}
// Runs of at least MIN_HALO_PARTICLES become groups, in run order.
__global__ void k_runs3(const int *hpos, const int *nh, int n, int64_t minsz, int64_t *roff,
                        int64_t *rsz, int32_t *keep) {
    int g = blockIdx.x * blockDim.x + threadIdx.x;
    if (g >= *nh) return;
    int s = hpos[g];
    int e = (g + 1 < *nh) ? hpos[g + 1] : n;
    roff[g] = s;
    rsz[g] = e - s;
    keep[g] = (e - s) >= minsz;
}

__global__ void k_mark_undecided(const int *dense, int nd, uint8_t *state) {
    int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t < nd) state[dense[t]] = 0;
}
__global__ void k_take2(const int32_t *idx, int m, const int32_t *a, const int32_t *b,
                        int32_t *a2, int32_t *b2) {
    int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= m) return;
    a2[t] = a[idx[t]];
    b2[t] = b[idx[t]];
}
__global__ void k_iota(int *a, int n) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) a[i] = i;
}

struct SeedFlag {
    const uint8_t *state;
    __device__ uint8_t operator()(int i) const { return state[i] == 1; }
};
struct DFlag {
    const uint8_t *c;
    __device__ uint8_t operator()(int i) const { return c[i] > 16; }
};
struct DenseI {
    __host__ __device__ int operator()(uint8_t c) const { return c > 16; }
};
static int sm_count() {
    int dev = 0, v = 0;
    RSG_CUDA(cudaGetDevice(&dev));
    RSG_CUDA(cudaDeviceGetAttribute(&v, cudaDevAttrMultiProcessorCount, dev));
    return v > 0 ? v : 1;
}
// The seed frontiers of one chunk as one graph: a while node whose body runs
// a step (k_kahn) and advances the frontier (k_kahn_next_g sets the loop
// condition), so no step waits for the host.
struct KahnGraph {
    cudaGraph_t g = nullptr;
    cudaGraphExec_t e = nullptr;
    void build(int GK, int TK, KahnList L, int limit) {
        RSG_CUDA(cudaGraphCreate(&g, 0));
        cudaGraphConditionalHandle h;
        RSG_CUDA(cudaGraphConditionalHandleCreate(&h, g, 1, cudaGraphCondAssignDefault));
        cudaGraphNodeParams cp = {};
        cp.type = cudaGraphNodeTypeConditional;
        cp.conditional.handle = h;
        cp.conditional.type = cudaGraphCondTypeWhile;
        cp.conditional.size = 1;
        cudaGraphNode_t cn, wn, nn;
        RSG_CUDA(cudaGraphAddNode(&cn, g, nullptr, nullptr, 0, &cp));
        cudaGraph_t body = cp.conditional.phGraph_out[0];
        void *wargs[] = {(void *)&L};
        cudaKernelNodeParams kp = {};
        kp.func = (void *)k_kahn;
        kp.gridDim = dim3(GK);
        kp.blockDim = dim3(TK);
        kp.kernelParams = wargs;
        RSG_CUDA(cudaGraphAddKernelNode(&wn, body, nullptr, 0, &kp));
        KahnCtl *ctl = L.ctl;
        int qcap = L.qcap;
        void *nargs[] = {(void *)&ctl, (void *)&qcap, (void *)&limit, (void *)&h};
        kp.func = (void *)k_kahn_next_g;
        kp.gridDim = dim3(1);
        kp.blockDim = dim3(1);
        kp.kernelParams = nargs;
        RSG_CUDA(cudaGraphAddKernelNode(&nn, body, &wn, 1, &kp));
        RSG_CUDA(cudaGraphInstantiate(&e, g, 0));
    }
    cudaStream_t ran = nullptr;
    void run(cudaStream_t st) {
        ran = st;
        RSG_CUDA(cudaGraphLaunch(e, st));
    }
    ~KahnGraph() {
        if (ran) cudaStreamSynchronize(ran);  // not destroyed while it runs
        if (e) cudaGraphExecDestroy(e);
        if (g) cudaGraphDestroy(g);
    }
};
// Indices i < n with pred(i), ascending, into out; returns their number.
template <class Pred>
static int select_where(Arena &ar, int n, Pred pred, int *out, cudaStream_t st) {
    thrust::transform_iterator<Pred, thrust::counting_iterator<int>, uint8_t> it(
        thrust::counting_iterator<int>(0), pred);
    size_t mark = ar.used;
    int *cnt = ar.get<int>(1);
    size_t b = 0;
    cub::DeviceSelect::Flagged(nullptr, b, thrust::counting_iterator<int>(0), it, out, cnt, n, st);
    void *t = ar.take(b + 256);
    cub::DeviceSelect::Flagged(t, b, thrust::counting_iterator<int>(0), it, out, cnt, n, st);
    RSG_CHECK_LAUNCH();
    int h = 0;
    RSG_CUDA(cudaMemcpyAsync(&h, cnt, sizeof(int), cudaMemcpyDeviceToHost, st));
    RSG_CUDA(cudaStreamSynchronize(st));
    ar.used = mark;
    return h;
}

// The later-dense list buffer of the calls whose list does not fit in the
// arena, kept per host thread (see fof3d_device).
struct ListCache {
    void *p = nullptr;
    size_t bytes = 0;
};
static thread_local ListCache g_list_cache;

struct FofOut {
    int64_t num_p;
    int64_t nfofs;
};

// Device-resident 3D FOF.  d_in: caller particles (n); d_out: permuted
// particles; d_off/d_sz: groups (capacity n/2+1).
FofOut fof3d_device(Arena &ar, const rsg_particle *d_in, int64_t n64, const rsg_config &cfg,
                    rsg_particle *d_out, int64_t *d_off, int64_t *d_sz, cudaStream_t st) {
    FofOut res{0, 0};
    if (n64 <= 0) return res;
    if (n64 >= (1ll << 31) - 2) {
        set_error(RSG_ERR_ARGS, "3D FOF supports up to 2^31-2 particles");
        throw Failure();
    }
    int n = (int)n64;
    const int T = 256;
    Rec *recs = ar.get<Rec>(n);
    int *flags = ar.get<int>(8);
    RSG_CUDA(cudaMemsetAsync(flags, 0, sizeof(int) * 8, st));
    phase_mark(st, "");
    launch(k_make_recs, nblk(n, T), T, 0, st, d_in, n, recs, flags);
    int32_t *seg = ar.get<int32_t>(2);
    int32_t hseg[2] = {0, n};
    RSG_CUDA(cudaMemcpyAsync(seg, hseg, sizeof(hseg), cudaMemcpyHostToDevice, st));
    size_t mark = ar.used;
    Forest<3> F = build_forest<3, Rec>(ar, recs, n, seg, seg + 1, 1, n, 20, st);
    launch(k_dup_probe, nblk(n, T), T, 0, st, recs, d_in, n, flags + 1);
    int hflags[8];
    RSG_CUDA(cudaMemcpyAsync(hflags, flags, sizeof(hflags), cudaMemcpyDeviceToHost, st));
    RSG_CUDA(cudaStreamSynchronize(st));
    if (hflags[0]) {
        set_error(RSG_ERR_INPUT, "non-finite particle coordinates");
        throw Failure();
    }
    if (hflags[1]) {
        int64_t *dn = ar.get<int64_t>(1);
        launch(k_dedupe_serial, 1, 1, 0, st, recs, d_in, n, dn);
        int64_t nn = 0;
        RSG_CUDA(cudaMemcpyAsync(&nn, dn, sizeof(nn), cudaMemcpyDeviceToHost, st));
        RSG_CUDA(cudaStreamSynchronize(st));
        n = (int)nn;
        hseg[1] = n;
        RSG_CUDA(cudaMemcpyAsync(seg, hseg, sizeof(hseg), cudaMemcpyHostToDevice, st));
        ar.used = mark;
        F = build_forest<3, Rec>(ar, recs, n, seg, seg + 1, 1, n, 20, st);
    }
    res.num_p = n;
    float r = (float)(cfg.avg_particle_spacing * cfg.fof_linking_length);
    float r2x = (float)(2.0 * (double)r);
    int *err = flags + 2;

    uint8_t *cnt = ar.get<uint8_t>(n);
    phase_mark(st, "fof.tree3d");
    const int TW = 128;
    launch(k_count_w, nblk(n, TW), TW, 0, st, F.nodes, recs, n, r, cnt, err);
    phase_mark(st, "fof.count");
    // dense particles (more than 16 neighbours), in tree order
    int *dense = ar.get<int>(n);
    int nd = select_where(ar, n, DFlag{cnt}, dense, st);
    // later-dense-neighbour lists and pending-skipper counts
    // (64-bit offsets: the lists can hold more than 2^31 entries)
    int *lcnt = ar.get<int>(n + 1), *skipcnt = ar.get<int>(n);
    int64_t *loff = ar.get<int64_t>(n + 1);
    RSG_CUDA(cudaMemsetAsync(lcnt, 0, sizeof(int) * (n + 1), st));
    RSG_CUDA(cudaMemsetAsync(skipcnt, 0, sizeof(int) * n, st));
    // dense particles before every index (the counting pass's whole nodes)
    int *dpfx = ar.get<int>(n + 1);
    {
        thrust::transform_iterator<DenseI, const uint8_t *, int> dit((const uint8_t *)cnt, DenseI{});
        size_t pb = 0;
        cub::DeviceScan::ExclusiveSum(nullptr, pb, dit, dpfx, n + 1, st);
        size_t m0 = ar.used;
        void *pt = ar.take(pb + 256);
        cub::DeviceScan::ExclusiveSum(pt, pb, dit, dpfx, n + 1, st);
        ar.used = m0;
    }
    launch(k_llist_w<false>, nblk(nd, TW), TW, 0, st, F.nodes, recs, (const int *)dense, nd, r,
           (const uint8_t *)cnt, (const int *)dpfx, (const int64_t *)nullptr, (int64_t)0, lcnt,
           (int *)nullptr, skipcnt, err);
    size_t cb = 0;
    thrust::transform_iterator<ToI64, const int32_t *, int64_t> lc64((const int32_t *)lcnt, ToI64{});
    cub::DeviceScan::ExclusiveSum(nullptr, cb, lc64, loff, n + 1, st);
    void *ct = ar.take(cb + 256);
    cub::DeviceScan::ExclusiveSum(ct, cb, lc64, loff, n + 1, st);
    int64_t ne = 0;
    RSG_CUDA(cudaMemcpyAsync(&ne, loff + n, sizeof(int64_t), cudaMemcpyDeviceToHost, st));
    RSG_CUDA(cudaStreamSynchronize(st));
    // The list lives in the arena when it fits beside what the rest of the FOF
    // takes from it (< 256 B per particle: the label derivation and the
    // partition sort).  A larger one (hundreds of entries
    // per particle in very dense snapshots) gets an allocation of its own for
    // this call, as large as free device memory allows (less 1 GiB, or
    // RSG_FOF_LIST_ENTRIES entries when that is set); when the whole list
    // does not fit, it is built and walked one chunk of particles at a time,
    // chunks in particle order.  A fixed arena holds the list whole or fails.
    // That allocation stays with the host thread for its later calls, as the
    // arena does: allocating and freeing a hundred gigabytes costs tens of
    // milliseconds each, and the free waits for the device.
    int *llist;
    int64_t lcap = ne > 0 ? ne : 1;  // entries the list buffer holds
    size_t lat = (ar.used + 255) & ~(size_t)255;
    const char *lenv = getenv("RSG_FOF_LIST_ENTRIES");
    int64_t lforce = lenv ? atoll(lenv) : 0;
    if (ar.fixed || (!lforce && lat + sizeof(int) * (size_t)lcap + (size_t)256 * n + (64u << 20) <= ar.cap)) {
        llist = ar.get<int>(lcap);
    } else {
        ListCache &lc = g_list_cache;
        size_t fb = 0, tb = 0;
        RSG_CUDA(cudaMemGetInfo(&fb, &tb));
        fb += lc.bytes;  // the kept buffer is this call's to use
        int64_t avail = fb > ((size_t)1 << 30) ? (int64_t)((fb - ((size_t)1 << 30)) / sizeof(int)) : 0;
        if (lforce > 0) avail = lforce;
        if (avail < lcap) lcap = avail;
        const size_t need = sizeof(int) * (size_t)(lcap > 0 ? lcap : 1);
        if (lc.bytes < need) {
            if (lc.p) RSG_CUDA(cudaFree(lc.p));
            lc.p = nullptr;
            lc.bytes = 0;
            RSG_CUDA(cudaMalloc(&lc.p, need));
            lc.bytes = need;
        }
        llist = (int *)lc.p;
    }
    // chunk boundaries: particles c[t] .. c[t+1], dense entries d[t] .. d[t+1]
    std::vector<int> cb_h(2, 0), db_h(2, 0);
    std::vector<int64_t> lb_h(1, 0);
    cb_h[1] = n;
    db_h[1] = nd;
    if (lcap < ne) {
        int maxl = 0;
        {
            int *dmax = ar.get<int>(1);
            size_t mb = 0;
            cub::DeviceReduce::Max(nullptr, mb, lcnt, dmax, n, st);
            size_t m0 = ar.used;
            void *mt = ar.take(mb + 256);
            cub::DeviceReduce::Max(mt, mb, lcnt, dmax, n, st);
            ar.used = m0;
            RSG_CUDA(cudaMemcpyAsync(&maxl, dmax, sizeof(int), cudaMemcpyDeviceToHost, st));
            RSG_CUDA(cudaStreamSynchronize(st));
        }
        int64_t step = lcap - maxl;
        if (step < (int64_t)maxl || step < (1 << 16)) {
            set_error(RSG_ERR_LIMIT, "later-dense lists need more device memory than is free");
            throw Failure();
        }
        int64_t m = (ne + step - 1) / step;  // chunks
        int *cbd = ar.get<int>(m + 1), *dbd = ar.get<int>(m + 1);
        thrust::transform_iterator<ChunkTarget, thrust::counting_iterator<int64_t>, int64_t> tgt(
            thrust::counting_iterator<int64_t>(0), ChunkTarget{step});
        thrust::lower_bound(thrust::cuda::par_nosync.on(st), loff, loff + n + 1, tgt, tgt + (m - 1), cbd);
        thrust::lower_bound(thrust::cuda::par_nosync.on(st), dense, dense + nd, cbd, cbd + (m - 1), dbd);
        cb_h.assign(m + 1, 0);
        db_h.assign(m + 1, 0);
        RSG_CUDA(cudaMemcpyAsync(cb_h.data() + 1, cbd, sizeof(int) * (m - 1), cudaMemcpyDeviceToHost, st));
        RSG_CUDA(cudaMemcpyAsync(db_h.data() + 1, dbd, sizeof(int) * (m - 1), cudaMemcpyDeviceToHost, st));
        RSG_CUDA(cudaStreamSynchronize(st));
        cb_h[m] = n;
        db_h[m] = nd;
        lb_h.assign(m + 1, 0);
        for (int64_t t = 0; t <= m; t++)
            RSG_CUDA(cudaMemcpyAsync(&lb_h[t], loff + cb_h[t], sizeof(int64_t), cudaMemcpyDeviceToHost, st));
        RSG_CUDA(cudaStreamSynchronize(st));
        for (int64_t t = 0; t < m; t++)
            if (lb_h[t + 1] - lb_h[t] > lcap) {
                set_error(RSG_ERR_LIMIT, "later-dense list chunk exceeds its buffer");
                throw Failure();
            }
    }
    const int nchunks = (int)cb_h.size() - 1;
    int *state32 = ar.get<int>(n);
    RSG_CUDA(cudaMemsetAsync(state32, 0, sizeof(int) * n, st));
    int *queue = ar.get<int>(nd + 1);
    const int qcap = nd + 1;
    KahnCtl *ctl = (KahnCtl *)ar.get<int64_t>(8);
    RSG_CUDA(cudaMemsetAsync(ctl, 0, sizeof(KahnCtl), st));
    launch(k_kahn_init, nblk(nd, T), T, 0, st, (const int *)dense, nd, (const int *)skipcnt,
           cb_h[1], state32, queue, qcap, ctl);
    const KahnList KL{(const int64_t *)loff, (const int *)llist, queue, qcap, ctl, state32, skipcnt};
    // every step but a chunk's last decides a particle
    const int limit = nd + nchunks + 2;
    int kres = 0;
    RSG_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&kres, k_kahn, 256, 0));
    const int TK = 256, GK = (kres > 0 ? kres : 1) * sm_count();
    // the frontier steps run as a device-side graph loop; with per-launch
    // event timing, and in fixed storage (instantiating a graph may take
    // device memory), the host drives the same steps
    const bool host_loop = launch_stats().selecting || ar.fixed;
    KahnGraph G;
    if (!host_loop && nd > 0) G.build(GK, TK, KL, limit);
    for (int t = 0; t < nchunks; t++) {
        int d0 = db_h[t], d1 = db_h[t + 1];
        if (d1 <= d0) continue;
        int64_t lbase = lb_h.size() > 1 ? lb_h[t] : 0;
        launch(k_llist_w<true>, nblk(d1 - d0, TW), TW, 0, st, F.nodes, recs,
               (const int *)dense + d0, d1 - d0, r, (const uint8_t *)cnt, (const int *)dpfx,
               (const int64_t *)loff, lbase, lcnt, llist, skipcnt, err);
        if (t > 0)
            launch(k_kahn_chunk, nblk(d1 - d0, T), T, 0, st, (const int *)dense + d0, d1 - d0,
                   (const int *)state32, queue, qcap, ctl);
        launch(k_kahn_start, 1, 1, 0, st, ctl, qcap, cb_h[t + 1], lbase);
        if (!host_loop) {
            G.run(st);
            continue;
        }
        for (;;) {
            launch(k_kahn, GK, TK, 0, st, KL);
            launch(k_kahn_next, 1, 1, 0, st, ctl, qcap, limit);
            KahnCtl hc;
            RSG_CUDA(cudaMemcpyAsync(&hc, ctl, sizeof(hc), cudaMemcpyDeviceToHost, st));
            RSG_CUDA(cudaStreamSynchronize(st));
            if (hc.tail <= hc.head || hc.hit || hc.overflow) break;
        }
    }
    KahnCtl kc;
    RSG_CUDA(cudaMemcpyAsync(&kc, ctl, sizeof(kc), cudaMemcpyDeviceToHost, st));
    RSG_CUDA(cudaStreamSynchronize(st));
    if (kc.hit || kc.overflow || kc.next != nd) {
        set_error(RSG_ERR_LIMIT, "3D FOF seed selection left %lld of %d dense particles undecided",
                  (long long)nd - kc.next, nd);
        throw Failure();
    }
    if (G.e) launch_stats().launches += 2 * (int64_t)kc.iters;
    phase_mark(st, "fof.elist");
    // non-dense particles: state 0 (never seeds)
    uint8_t *state = ar.get<uint8_t>(n);
    launch(k_state8, nblk(n, T), T, 0, st, state32, n, state);
    phase_mark(st, "fof.seeds");
    if (getenv("RSG_TIMING"))
        fprintf(stderr, "  [fof] dense %d, dense pairs %lld in %d chunk(s), frontier steps %d\n",
                nd, (long long)ne, nchunks, kc.iters);
    last_stats()[RSG_STAT_DENSE] = nd;
    last_stats()[RSG_STAT_DENSE_PAIRS] = ne;
    last_stats()[RSG_STAT_SEED_STEPS] = kc.iters;
    int *seeds = ar.get<int>(nd + 1);
    const int nseed = select_where(ar, n, SeedFlag{state}, seeds, st);
    const int TS = RSG_SEED_WARPS * 32;
    const int GS = (int)nblk((int64_t)nseed * 32, TS);
    uint8_t *skipped = ar.get<uint8_t>(n);
    RSG_CUDA(cudaMemsetAsync(skipped, 0, n, st));
    launch(k_seed_mark_w, GS, TS, 0, st, F.nodes, recs, (const int *)seeds, nseed, r, skipped,
           err);
    // labels exactly as the reference's union-find leaves them (uflabels.cuh)
    int *gtime = ar.get<int>(n);
    RSG_CUDA(cudaMemsetAsync(gtime, 0x7f, sizeof(int) * n, st));  // 0x7f7f7f7f: never
    launch(k_gtime_r, nblk(n, T), T, 0, st, F.nodes, recs, n, r, (const uint8_t *)cnt,
           (const uint8_t *)skipped, (const uint8_t *)state, gtime, err);
    launch(k_gtime_seed_w, GS, TS, 0, st, F.nodes, recs, (const int *)seeds, nseed, r, gtime, err);
    int32_t *ptr = ar.get<int32_t>(n), *sfid = ar.get<int32_t>(n), *nsc = ar.get<int32_t>(n + 1);
    launch(k_fptr3, nblk(n, T), T, 0, st, F.nodes, recs, n, r, (const uint8_t *)cnt,
           (const uint8_t *)skipped, (const uint8_t *)state, (const int *)gtime, ptr, err);
    launch(k_fptr_seed_w, GS, TS, 0, st, F.nodes, recs, (const int *)seeds, nseed, r,
           (const int *)gtime, ptr, err);
    RSG_CHECK_LAUNCH();
    int64_t S = uf_resolve(ar, ptr, n, sfid, nsc, st);
    phase_mark(st, "fof.first_links");
    // candidate merges, in time order
    unsigned long long *ccount = ar.get<unsigned long long>(1);
    int64_t ccap = (int64_t)n / 2 + 1024;
    size_t cmark = ar.used;
    uint64_t *ckey = nullptr;
    int32_t *cF = nullptr, *cW = nullptr;
    unsigned long long hc = 0;
    int32_t *lab0 = ar.get<int32_t>(n);
    {
        // lab0[j] = f(g(j)): the set j joined when it was labelled
        launch(k_lab3, nblk(n, T), T, 0, st, (const int *)gtime, n, (const int32_t *)sfid,
               (const int32_t *)nullptr, lab0);
    }
    cmark = ar.used;
    for (int pass = 0; pass < 2; pass++) {
        ar.used = cmark;
        ckey = ar.get<uint64_t>(ccap);
        cF = ar.get<int32_t>(ccap);
        cW = ar.get<int32_t>(ccap);
        RSG_CUDA(cudaMemsetAsync(ccount, 0, sizeof(unsigned long long), st));
        launch(k_cand3, nblk(n, T), T, 0, st, F.nodes, recs, n, r, (const uint8_t *)cnt,
               (const uint8_t *)skipped, (const uint8_t *)state, (const int *)gtime,
               (const int32_t *)lab0, (const int32_t *)sfid, ccap, ccount, ckey, cF, cW, err);
        launch(k_cand_seed_w, GS, TS, 0, st, F.nodes, recs, (const int *)seeds, nseed, r, r2x,
               (const int *)gtime, (const int32_t *)lab0, (const int32_t *)sfid, ccap, ccount,
               ckey, cF, cW, err);
        RSG_CHECK_LAUNCH();
        RSG_CUDA(cudaMemcpyAsync(&hc, ccount, sizeof(hc), cudaMemcpyDeviceToHost, st));
        RSG_CUDA(cudaStreamSynchronize(st));
        if ((int64_t)hc <= ccap) break;
        ccap = (int64_t)hc;  // exact size, second pass
    }
    int64_t nc = (int64_t)hc;
    if (nc >= 0x7f7f7f7f) {
        set_error(RSG_ERR_LIMIT, "3D FOF: too many label merges (%lld)", (long long)nc);
        throw Failure();
    }
    int32_t *cF2 = ar.get<int32_t>(nc + 1), *cW2 = ar.get<int32_t>(nc + 1);
    if (nc > 0) {
        uint64_t *ckey2 = ar.get<uint64_t>(nc);
        int32_t *cidx = ar.get<int32_t>(nc), *cidx2 = ar.get<int32_t>(nc);
        launch(k_iota, nblk(nc, T), T, 0, st, cidx, (int)nc);
        size_t sb = 0;
        cub::DeviceRadixSort::SortPairs(nullptr, sb, ckey, ckey2, cidx, cidx2, (int)nc, 0, 64, st);
        void *stmp = ar.take(sb + 256);
        cub::DeviceRadixSort::SortPairs(stmp, sb, ckey, ckey2, cidx, cidx2, (int)nc, 0, 64, st);
        launch(k_take2, nblk(nc, T), T, 0, st, (const int32_t *)cidx2, (int)nc,
               (const int32_t *)cF, (const int32_t *)cW, cF2, cW2);
    }
    int32_t *sroot = ar.get<int32_t>(S + 1);
    uf_roots(ar, cF2, cW2, nc, S, sroot, st);
    int32_t *lab = ar.get<int32_t>(n);
    launch(k_lab3, nblk(n, T), T, 0, st, (const int *)gtime, n, (const int32_t *)sfid,
           (const int32_t *)sroot, lab);
    RSG_CHECK_LAUNCH();
    phase_mark(st, "fof.labels");
    // the reference's partition sort by label (src/fof.c:184-224), then the
    // groups of build_fullfofs (src/fof.c:226-255)
    {
        std::vector<int32_t> s0(1, 0), n0(1, n);
        partition_sort_labels<Rec>(ar, recs, lab, n, s0, n0, st);
    }
    launch(k_gather_out, nblk(n, T), T, 0, st, (const Rec *)recs, d_in, n, d_out);
    int *head = ar.get<int>(n), *hpos = ar.get<int>(n), *nh = ar.get<int>(1);
    launch(k_run_heads3, nblk(n, T), T, 0, st, (const int32_t *)lab, n, head);
    size_t hb = 0;
    cub::DeviceSelect::Flagged(nullptr, hb, thrust::counting_iterator<int>(0), head, hpos, nh, n,
                               st);
    void *htmp = ar.take(hb + 256);
    cub::DeviceSelect::Flagged(htmp, hb, thrust::counting_iterator<int>(0), head, hpos, nh, n, st);
    int64_t *roff = ar.get<int64_t>(n / 2 + 1), *rsz = ar.get<int64_t>(n / 2 + 1);
    int32_t *keep = ar.get<int32_t>(n / 2 + 1);
    launch(k_runs3, nblk(n / 2 + 1, T), T, 0, st, (const int *)hpos, (const int *)nh, n,
           (int64_t)cfg.min_halo_particles, roff, rsz, keep);
    int hnh = 0;
    RSG_CUDA(cudaMemcpyAsync(&hnh, nh, sizeof(int), cudaMemcpyDeviceToHost, st));
    RSG_CUDA(cudaStreamSynchronize(st));
    int *nk = ar.get<int>(1);
    size_t kb = 0;
    cub::DeviceSelect::Flagged(nullptr, kb, roff, keep, d_off, nk, hnh, st);
    void *ktmp = ar.take(kb + 256);
    cub::DeviceSelect::Flagged(ktmp, kb, roff, keep, d_off, nk, hnh, st);
    cub::DeviceSelect::Flagged(ktmp, kb, rsz, keep, d_sz, nk, hnh, st);
    RSG_CHECK_LAUNCH();
    RSG_CUDA(cudaMemcpyAsync(&hnh, nk, sizeof(int), cudaMemcpyDeviceToHost, st));
    RSG_CUDA(cudaMemcpyAsync(hflags, flags, sizeof(hflags), cudaMemcpyDeviceToHost, st));
    RSG_CUDA(cudaStreamSynchronize(st));
    if (hflags[2]) {
        set_error(RSG_ERR_LIMIT, "kd-tree traversal stack overflow");
        throw Failure();
    }
    res.nfofs = hnh;
    last_stats()[RSG_STAT_PARTICLES] = n;
    last_stats()[RSG_STAT_GROUPS] = hnh;
    phase_mark(st, "fof.output");
    return res;
}

}  // namespace rsg
